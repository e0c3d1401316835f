#!/usr/bin/env python
"""Benchmark: rays/s of the GPU SPH iso-surface march (reference: the CPU
RayMarcher, src/app/AdvancedRenderer/RayMarcher.cpp:256-344).

Workload (one "step" = one rendered frame): the 1,000,000-particle sloshing
scene (950k fluid below y = 0.4 + 0.08 sin(2 pi x) cos(3 pi z) + N(0, 0.005),
50k spray above), support radius 0.04 (h = 0.02), iso = 0.5 x lattice rest
density, 1920x1080, step 0.25 h, max 1024 steps, 8 bisection iterations.
Synthetic, seeded particles; the scene stays resident in HBM for `value`.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value  rays/s over all N GPUs (each rank renders its own frame: replicas,
       weak scaling), device time of splat + march + shade per frame, CUDA
       events on the launching stream, L2 flushed (512 MiB write) between
       frames outside the events.
e2e    the same frame through the C ABI with pinned HOST buffers: particle
       upload + grid build + bound table (next to the splat) + splat + march +
       shade, the march writing position, normal, depth and colour into the
       library's pinned host memory; wall clock per frame.
--impl reference times the CPU marcher (the oracle port of the reference's
       loop, bisection 0, skipping off, all host threads but one as
       RayMarcher.cpp:67 does) on a bounded random pixel sample per step.
learned  the same frame with the learned hit-interval proposal
       (FM_MARCH_PROPOSAL, weights fluidmarch/proposal_sloshing.npz), timed the
       same way; every timed frame includes the per-frame judge (fm_set_judge:
       the plain march of a 1-in-64 sample of 8x4 pixel blocks compared on the
       device), and
       the last frame is also judged whole against the plain march of the same
       frame (hit masks, |depth difference| <= 1e-4 x scene extent).
batch  64 scenes of the sloshing family (50k..2M particles, 1-4 views each
       at 640x480 / 1280x720 / 1920x1080) in one graph launch per frame.
anisotropic  the same frame with the reference's default marcher
       (PerPixel_Anisotropic: per-sample WPCA kernels, k_n 0.5, k_r 2, k_s 2000,
       N_eps 1, extended radius 2 H, iso = half the median anisotropic density
       inside the fluid), next to the CPU port of it on a pixel sample.
particle_files  the bench frame as gzip BGEO files: host decode, scene from
       a file, autoplay of a file series.
grid_build  the uniform-grid build of the 1M frame and of a 4M frame from
       device positions, against 64 B per particle + 16 B per cell.
"""

from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "bachelor-thesis_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "rays/s and 1080p frames/s: learned vs plain GPU march at fixed depth error"
UNIT = "rays/s"
L2_FLUSH_BYTES = 512 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip", default="exact", choices=["exact", "off"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of the cpu_baseline sample")
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--profile", action="store_true", help="short plain run of --steps frames for ncu")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-proposal comparison")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched 64-scene measurement")
    ap.add_argument("--no-aniso", action="store_true", help="skip the anisotropic-march measurement")
    ap.add_argument("--no-autotune", action="store_true",
                    help="time the batch with the context's work split instead of the autotuned one")
    ap.add_argument("--no-files", action="store_true", help="skip the particle-file loading measurement")
    ap.add_argument("--no-grid", action="store_true", help="skip the grid-build measurement")
    return ap.parse_args()


def workload_config(sc, cam, skip):
    return {"workload": "sloshing surface, plain GPU march", "particles": sc.n, "support_radius": sc.support,
            "h": sc.support / 2, "iso": sc.iso, "width": cam.width, "height": cam.height, "step": sc.step,
            "max_steps": sc.max_steps, "bisect_iters": sc.bisect, "skip": skip,
            "l2": "flushed between frames (512 MiB write)", "parallelism": "replicas"}


def cpu_info():
    model = platform.processor() or ""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    return os.cpu_count() or 1, model or platform.machine()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ["index", "clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + ",".join(self.FIELDS),
                                          "--format=csv,noheader,nounits", "-lms", "200", "-i", str(self.device)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_march():
    """The march kernels' ncu figures from the committed summary (profiles/march_sloshing_1080p.json):
    DRAM bytes, issue-active and lane fractions, L1/L2 throughput of k_march and k_march_long, with the
    commit and date of the capture.  These are not measured by this run."""
    p = os.path.join(ROOT, "profiles", "march_sloshing_1080p.json")
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def march_roofline(st, g, npx, march_ms, peak, peak_kind):
    """Roofline of the march stage (k_march + k_march_long, CUDA events around fm_march).

    HBM: the bytes the march has to move between HBM and the SMs once per frame -- the cell-sorted
    particles (16 B each), the sub-cell start table (4 B x (8 n_cells + 1)), the exact-skip bound table
    (4 B x 512 n_cells), the start depths (4 B per pixel) and the four output planes (position, normal,
    colour 16 B, hit distance 4 B per pixel) -- over the stage's time.  The candidate stream the
    reference's loop implies (16 B for every particle in the 27 cells of every density evaluation,
    RayMarcher.cpp:308-325) is served from L1/L2 and reported beside it, not as an HBM figure."""
    hbm_bytes = 16 * g["n_particles"] + 4 * (8 * g["n_cells"] + 1) + 4 * 512 * g["n_cells"] + (4 + 52) * npx
    t = march_ms / 1000.0
    achieved = hbm_bytes / t / 1e9
    prof = profiled_march()
    cand = 16 * st["candidates"]
    traffic = None
    if prof.get("kernels"):
        traffic = sum(k.get("dram_bytes", 0) for k in prof["kernels"].values())
    return {
        "bound": "hbm", "kernel": "march stage (k_march + k_march_long)", "achieved": achieved, "peak": peak,
        "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
        "algorithmic_bytes_per_launch": hbm_bytes,
        "note": "HBM bytes the march must move once per frame over the stage time; the stage is far below "
                "the HBM roof and is bound by instruction issue (profiled.issue_active); traffic is the "
                "profiled DRAM bytes of both kernels",
        "candidate_stream": {"bytes_per_frame": cand, "evals": st["evals"], "candidates": st["candidates"],
                             "achieved_gbs": cand / t / 1e9,
                             "note": "16 B x particles in the 27 cells of every density evaluation, served "
                                     "from L1/L2 (each streamed particle serves the lanes that need it)"},
        "profiled": prof or None,
    }


def cpu_baseline_sample(sc, cam, depth, fr, target_s, threads):
    """Time the oracle port (bisection 0, skip off) on a seeded random pixel sample."""
    import oracle as O

    rng = np.random.default_rng(1234)
    npx = cam.width * cam.height
    n = 2000
    spent = 0.0
    total_px = 0
    while True:
        pix = np.sort(rng.choice(npx, n, replace=False)).astype(np.int64)
        t0 = time.perf_counter()
        O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 0, depth, skip_mode=0, pixels=pix, threads=threads,
                want_colour=False)
        dt = time.perf_counter() - t0
        spent += dt
        total_px += n
        if spent >= target_s or n >= npx:
            break
        n = int(min(npx, max(n * 2, n * (target_s - spent) / max(dt, 1e-3))))
    return total_px / spent, total_px, spent


def frame_parity(O, fr, sc, cam, gpu, threads):
    """The bench frame's GPU outputs against the oracle, every pixel: the FP32 restatement of the
    reference loop plus bisection (RayMarcher.cpp:256-344; bit-exact expected) and its FP64 twin (the
    the benchmark spec's tolerances: hit masks identical except where |rho - iso| <= 1e-3 iso, depth within
    1e-4 of the scene extent, normals within 0.5 degrees)."""
    t0 = time.perf_counter()
    z = gpu["start_depth"]
    args = (fr, cam, sc.iso, sc.step, sc.max_steps)
    o32 = O.march(*args, sc.bisect, z, threads=threads)
    differ = np.zeros(z.size, bool)
    for k in ("position", "normal", "depth", "colour"):
        a = np.ascontiguousarray(gpu[k]).view(np.uint32).reshape(z.size, -1)
        b = np.ascontiguousarray(o32[k]).view(np.uint32).reshape(z.size, -1)
        differ |= np.any(a != b, axis=1)
    hg = gpu["position"][:, 3] == 1
    # masks: decided at the first sample with rho >= iso, so compared on the marches without bisection
    o32_0 = O.march(*args, 0, z, threads=threads, want_colour=False)
    o64_0 = O.march(*args, 0, z, threads=threads, precision=64, want_colour=False)
    h64 = o64_0["position"][:, 3] == 1
    mism = hg != h64
    rho = np.where(hg & ~h64, o32_0["rho"], o64_0["rho"])
    outside = int(np.sum(mism & (np.abs(rho - sc.iso) > 1e-3 * sc.iso)))
    o64 = O.march(*args, sc.bisect, z, threads=threads, precision=64, want_colour=False)
    both = hg & (o64["position"][:, 3] == 1)
    ext = float(np.max(sc.xyz.max(0) - sc.xyz.min(0)))
    derr = np.abs(gpu["depth"][both].astype(np.float64) - o64["depth"][both]) / ext
    n1 = gpu["normal"][both, :3].astype(np.float64)
    n2 = o64["normal"][both, :3].astype(np.float64)
    c = np.sum(n1 * n2, 1) / np.linalg.norm(n1, axis=1) / np.linalg.norm(n2, axis=1)
    ang = np.degrees(np.arccos(np.clip(c, -1.0, 1.0)))
    return {
        "pixels": int(z.size), "started": int(np.sum(z < 1)), "hits": int(hg.sum()),
        "oracle_fp32": {"pixels_differing": int(differ.sum()),
                        "hit_mask_mismatch": int(np.sum(hg != (o32["position"][:, 3] == 1))),
                        "compared": "position, normal, hit distance, colour bits"},
        "oracle_fp64": {"hit_mask_mismatch": int(mism.sum()), "mismatch_outside_1e-3_iso": outside,
                        "hits_compared": int(both.sum()),
                        "depth_within_1e-4_extent": float(np.mean(derr <= 1e-4)) if derr.size else None,
                        "max_depth_err_extent": float(derr.max()) if derr.size else None,
                        "normal_within_0.5_deg": float(np.mean(ang <= 0.5)) if ang.size else None,
                        "max_normal_deg": float(ang.max()) if ang.size else None},
        "seconds": time.perf_counter() - t0, "threads": threads,
    }


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle as O
    from fluidmarch import scenes

    O.build_oracle(ref=False)
    sc = scenes.sloshing()
    cam = sc.cameras[0]
    fr = O.build_frame(sc.xyz, sc.support)
    depth = O.splat(sc.xyz, sc.support, cam)
    cores, model = cpu_info()
    threads = max(1, cores - 1)
    rng = np.random.default_rng(77)
    npx = cam.width * cam.height
    per_step = 100_000  # ~0.1 s of the reference loop per step on a 16-core host
    times = []
    for i in range(args.warmup + args.steps):
        pix = np.sort(rng.choice(npx, per_step, replace=False)).astype(np.int64)
        t0 = time.perf_counter()
        O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 0, depth, skip_mode=0, pixels=pix, threads=threads,
                want_colour=False)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    total = sum(times)
    v = per_step * len(times) / total
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            # the GPU arm's workload; the reference's loop has no bisection and here
            # evaluates every sample (its skip flags are a CompactNSearch call that is
            # not part of the reference tree), on a pixel sample of that frame
            "config": workload_config(sc, cam, args.skip),
            "reference_loop": {"bisect_iters": 0, "skip": "off",
                               "sample": f"{per_step} random pixels of the 1920x1080 frame per step"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{per_step} seeded random pixels per step, {len(times)} steps; "
                                       f"CPU {model}, {cores} host cores"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_learned(args, fm, torch, ctx, ext, scene, sc, cam, out, flush, skip, plain_ms, plain_st):
    """The learned-proposal march of the same frame, timed like the plain one, judged against it."""
    from fluidmarch import proposal as PR

    params, meta = PR.load()
    margin_lo, margin_hi, min_near = 0.5, 0.5, 8.0
    prop = fm.Proposal(ctx, params, margin_lo, margin_hi, min_near)
    fm.set_proposal(ctx, prop)
    npx = cam.width * cam.height
    dev = out["depth"].device
    lo = {k: torch.empty_like(v) for k, v in out.items()}
    P_l = fm.MarchParams(sc.iso, sc.step, sc.max_steps, sc.bisect, skip, external_depth=True, proposal=True)

    def frame():
        fm.splat_depth(scene, cam, lo["start_depth"])
        fm.march(scene, cam, P_l, lo["position"], lo["normal"], lo["depth"], lo["colour"], lo["start_depth"])

    extent = float((sc.xyz.max(0) - sc.xyz.min(0)).max())
    tol = 1e-4 * extent
    ctx.set_stats(True)
    frame()
    ctx.sync()
    st = ctx.stats()
    ctx.set_stats(False)
    # every timed learned frame is judged: the plain march of a 1-in-64 sample of 8x4 pixel blocks
    # (a different one each frame), compared on the device
    judge_stride = 64
    ctx.set_judge(judge_stride, tol)
    for _ in range(args.warmup):
        frame()
    ctx.sync()
    ctx.judge_frames(reset=True)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(ext):
        for e0, e1 in ev:
            flush.zero_()
            e0.record(ext)
            frame()
            e1.record(ext)
        ext.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    jf = ctx.judge_frames(reset=True)
    ctx.set_judge(0, 0.0)
    j = fm.judge(ctx, out["depth"], lo["depth"], tol)
    # the plain march without empty-space skipping (the reference's loop) and with
    # the reference's own skip flags, for comparison (a few frames each)
    def timed_plain(mode):
        P_m = fm.MarchParams(sc.iso, sc.step, sc.max_steps, sc.bisect, mode, external_depth=True)
        ts = []
        for k in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(ext):
                flush.zero_()
                e0.record(ext)
                fm.splat_depth(scene, cam, lo["start_depth"])
                fm.march(scene, cam, P_m, lo["position"], lo["normal"], lo["depth"], lo["colour"], lo["start_depth"])
                e1.record(ext)
                ext.synchronize()
            if k > 0:
                ts.append(e0.elapsed_time(e1))
        return float(np.mean(ts))

    # where proposed rays go: intervals of this frame against the plain march's hit mask
    iv = torch.zeros((npx, 2), dtype=torch.int32, device=dev)
    fm.proposal_intervals(scene, cam, P_l, lo["start_depth"], iv)
    ctx.sync()
    started = lo["start_depth"] < 1
    proposed = (iv[:, 1] > 0) & started
    plain_hit = out["depth"] > 0
    # no proposal can remove a hit ray's crossing sample, its bisections or its normal
    floor = plain_st["hits"] * (sc.bisect + 2)
    causes = {"proposed": int(proposed.sum().item()),
              "proposed_plain_misses": int((proposed & ~plain_hit).sum().item()),
              "proposed_plain_hits": int((proposed & plain_hit).sum().item()),
              "plain_evals": plain_st["evals"], "learned_evals": st["evals"],
              "evals_floor_hits_x_bisect_plus_2": floor,
              "max_vs_plain_by_evaluations": plain_st["evals"] / max(1, floor),
              "note": "a ray the plain march misses has no crossing in any interval and always falls back; "
                      "a perfect, free proposal still evaluates each hit's crossing, bisections and normal"}
    off = [timed_plain(fm.FM_SKIP_OFF)]
    ref_skip = timed_plain(fm.FM_SKIP_REFERENCE)
    fm.set_proposal(ctx, None)
    prop.close()
    return {"rays_per_s": npx / (ms / 1e3), "frames_per_s": 1e3 / ms, "ms_per_frame": ms,
            "vs_plain": plain_ms / ms, "plain_ms_per_frame": plain_ms,
            "plain_skip_off_ms_per_frame": float(np.mean(off)), "vs_plain_skip_off": float(np.mean(off)) / ms,
            "plain_reference_skip_ms_per_frame": ref_skip, "vs_plain_reference_skip": ref_skip / ms,
            "depth_tol": tol, "judge": j, "hits_within_tol": j["within_tol"] / max(1, j["hits_ref"]),
            "per_frame_judge": dict(jf, stride=judge_stride,
                                    hits_within_tol=jf["within_tol"] / max(1, jf["hits_ref"]),
                                    note="inside every timed learned frame: plain march of a 1-in-stride sample of "
                                         "8x4 pixel blocks, compared with the learned march on the device"),
            "mask_identical": j["mask_mismatch"] == 0,
            "margins_support_radii": [margin_lo, margin_hi], "min_near_support_radii": min_near,
            "counters": {k: st[k] for k in ("evals", "proposed", "fallbacks", "deferred")},
            "fallback_causes": causes,
            "proposal": {"weights": "fluidmarch/proposal_sloshing.npz", "train_scenes": meta.get("train_scenes"),
                         "heldout_scenes": meta.get("heldout_scenes"), "heldout": meta.get("heldout")}}


def run_aniso(args, fm, torch, ctx, ext, scene, sc, cam, out):
    """The reference's default (anisotropic) march of the same frame, GPU and the CPU port."""
    import oracle as O

    O.build_oracle(ref=False)
    aniso = (2.0, 0.5, 2.0, 2000.0, 1)
    fr = O.build_frame(sc.xyz, sc.support)
    x = sc.xyz
    inner = x[(x[:, 1] < 0.2) & (x[:, 0] > 0.3) & (x[:, 0] < 0.7) & (x[:, 2] > 0.3) & (x[:, 2] < 0.7)][:200]
    iso = float(np.float32(0.5 * np.median(O.density_aniso(fr, inner, aniso))))
    ctx.set_anisotropy(*aniso)
    P = fm.MarchParams(iso, sc.step, sc.max_steps, sc.bisect, fm.FM_SKIP_OFF, external_depth=True, anisotropic=True)
    npx = cam.width * cam.height

    def frame():
        fm.splat_depth(scene, cam, out["start_depth"])
        fm.march(scene, cam, P, out["position"], out["normal"], out["depth"], out["colour"], out["start_depth"])

    frame()
    ctx.sync()
    steps = 3
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(ext):
        for e0, e1 in ev:
            e0.record(ext)
            frame()
            e1.record(ext)
        ext.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    hits = int((out["depth"] > 0).sum().item())
    # with the reference's own skip flags (the renderer's mode; results differ from skip off
    # where a flagged cell is jumped over)
    P_ref = fm.MarchParams(iso, sc.step, sc.max_steps, sc.bisect, fm.FM_SKIP_REFERENCE, external_depth=True,
                           anisotropic=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(ext):
        e0.record(ext)
        fm.splat_depth(scene, cam, out["start_depth"])
        fm.march(scene, cam, P_ref, out["position"], out["normal"], out["depth"], out["colour"], out["start_depth"])
        e1.record(ext)
        ext.synchronize()
    ms_ref = e0.elapsed_time(e1)
    # exact skip (samples whose bound box has no particle within the support radius have
    # density 0): the same outputs as skip off
    P_ex = fm.MarchParams(iso, sc.step, sc.max_steps, sc.bisect, fm.FM_SKIP_EXACT, external_depth=True,
                          anisotropic=True)
    for _ in range(2):  # the first builds the bound table of the scene at this iso
        fm.splat_depth(scene, cam, out["start_depth"])
        fm.march(scene, cam, P_ex, out["position"], out["normal"], out["depth"], out["colour"], out["start_depth"])
    ctx.sync()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(ext):
        for e0, e1 in ev:
            e0.record(ext)
            fm.splat_depth(scene, cam, out["start_depth"])
            fm.march(scene, cam, P_ex, out["position"], out["normal"], out["depth"], out["colour"],
                     out["start_depth"])
            e1.record(ext)
        ext.synchronize()
    ms_ex = sum(a.elapsed_time(b) for a, b in ev) / steps
    hits_ex = int((out["depth"] > 0).sum().item())
    frame()  # the skip-off outputs again, for the CPU sample below
    ctx.sync()
    # the CPU port on a sample of started pixels (bisection 0, as the reference)
    depth = out["start_depth"].cpu().numpy()
    started = np.nonzero(depth < 1)[0]
    rng = np.random.default_rng(9)
    pix = np.sort(rng.choice(started, min(600, started.size), replace=False)).astype(np.int64)
    cores, _ = cpu_info()
    t0 = time.perf_counter()
    O.march_aniso(fr, cam, iso, sc.step, sc.max_steps, 0, depth, aniso, pixels=pix, threads=max(1, cores - 1))
    cpu_s = time.perf_counter() - t0
    frac = started.size / npx
    return {"iso": iso, "params": {"radius_mult": 2.0, "k_n": 0.5, "k_r": 2.0, "k_s": 2000.0, "n_eps": 1},
            "ms_per_frame": ms, "rays_per_s": npx / (ms / 1e3), "hits": hits, "bisect_iters": sc.bisect,
            "ms_per_frame_reference_skip": ms_ref, "rays_per_s_reference_skip": npx / (ms_ref / 1e3),
            "ms_per_frame_exact_skip": ms_ex, "rays_per_s_exact_skip": npx / (ms_ex / 1e3),
            "exact_skip_hits_equal": hits_ex == hits,
            "cpu_port_rays_per_s": (pix.size / cpu_s) / frac if frac > 0 else None,
            "cpu_sample": f"{pix.size} started pixels, bisection 0, {max(1, cores - 1)} threads, scaled by the "
                          f"started fraction {frac:.3f} to all pixels"}


def run_files(args, fm, torch, ctx, sc):
    """Particle files: the bench scene as gzip BGEO frames, loaded into scenes (host decode + GPU gather +
    grid build), against building the scene from positions already in host memory."""
    import shutil
    import tempfile

    from fluidmarch import bgeo

    tmp = tempfile.mkdtemp(prefix="fm_bgeo_")
    try:
        rng = np.random.default_rng(7)
        n = sc.n
        attrs = {"v": ("vector", rng.normal(size=(n, 3)).astype(np.float32)), "id": ("int", np.arange(n))}
        frames = 6
        prefix = os.path.join(tmp, "ParticleData_Fluid_")
        for i in range(1, frames + 1):
            jitter = rng.normal(0, 1e-4, sc.xyz.shape).astype(np.float32)
            bgeo.write(f"{prefix}{i}.bgeo", sc.xyz + jitter, attrs, compressed=True, level=1)
        path = f"{prefix}1.bgeo"
        size = os.path.getsize(path)
        t = []
        for _ in range(3):
            t0 = time.perf_counter()
            bgeo.read(path)
            t.append(time.perf_counter() - t0)
        host_ms = 1e3 * min(t)
        t = []
        for _ in range(3):
            t0 = time.perf_counter()
            s = bgeo.load_scene(ctx, path, sc.support)
            t.append(time.perf_counter() - t0)
            s.close()
        scene_ms = 1e3 * min(t)
        t = []
        for _ in range(3):
            t0 = time.perf_counter()
            s = fm.Scene(ctx, sc.xyz, sc.support)
            ctx.sync()
            t.append(time.perf_counter() - t0)
            s.close()
        mem_ms = 1e3 * min(t)
        series = {}
        for threads in (0, 4):
            ds = bgeo.Dataset(prefix, ".bgeo", -1, threads)
            ds.load(ctx, 0, sc.support)
            t0 = time.perf_counter()
            for i in range(1, frames):
                ds.load(ctx, i, sc.support)
            series[f"threads_{threads}"] = 1e3 * (time.perf_counter() - t0) / (frames - 1)
            ds.close()
        info = bgeo.info(path)
        return {"particles": n, "record_words": info["record_words"], "file_mb": size / 1e6,
                "data_mb": 4 * info["record_words"] * n / 1e6,
                "host_decode_ms": host_ms, "scene_from_file_ms": scene_ms, "scene_from_host_memory_ms": mem_ms,
                "autoplay_ms_per_frame": series,
                "note": "gzip level 1 BGEO with velocity and id attributes; scene_from_file = decode on one host "
                        "core + record upload + byte-swap gather kernel + grid build; autoplay = the next frame "
                        "of a 6-frame series with host threads decoding ahead"}
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def run_grid(args, fm, torch, ctx, ext, sc, flush, peak):
    """The uniform-grid build (AABB and grid, cell keys, counting sort, start tables, sorted gather) of the bench frame
    and of a 4M-particle frame of the same layout, from positions in device memory, L2 flushed before each
    build; algorithmic bytes 64 B per particle + 16 B per cell."""
    from fluidmarch import scenes

    res = {}
    cases = [("1m", sc.xyz, sc.support),
             ("4m", scenes._sloshing_xyz(np.random.default_rng(4000), 4_000_000), float(np.float32(2 * 0.0126)))]
    for name, xyz, support in cases:
        xyz_d = torch.from_numpy(xyz).cuda()
        torch.cuda.synchronize()
        s = fm.Scene(ctx, xyz_d, support)
        for _ in range(3):
            s.update(xyz_d)
        ctx.sync()
        ts = []
        with torch.cuda.stream(ext):
            for _ in range(max(5, args.steps // 2)):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(ext)
                s.update(xyz_d)
                e1.record(ext)
                ext.synchronize()
                ts.append(e0.elapsed_time(e1))
        g = s.grid()
        s.close()
        ms = float(np.median(ts))
        alg = 64 * g["n_particles"] + 16 * g["n_cells"]
        res[name] = {"particles": g["n_particles"], "cells": g["n_cells"], "ms": ms, "algorithmic_bytes": alg,
                     "achieved_gbs": alg / ms / 1e6, "frac_of_hbm_peak": alg / ms / 1e6 / peak}
        del xyz_d
    res["note"] = ("fm_scene_update from device positions: bounds pass, a one-thread pass that computes the grid "
                   "on the device, cell keys and key histogram with ranks, its scan, scatter, per-sub-cell sort "
                   "by input index with the gather, one host sync at the end; median of the builds, each after "
                   "an L2 flush")
    return res


def run_batch(args, fm, torch, ctx, ext, dev):
    """The batched configuration: 64 sloshing-family scenes, 1-4 views each, one graph launch per frame."""
    from fluidmarch import scenes

    t0 = time.perf_counter()
    bs = scenes.batch_scenes()
    gen_s = time.perf_counter() - t0
    views, keep = [], []
    for sc in bs:
        s = fm.Scene(ctx, sc.xyz, sc.support)
        keep.append(s)
        p = fm.MarchParams(sc.iso, sc.step, sc.max_steps, sc.bisect, fm.FM_SKIP_EXACT)
        for cam in sc.cameras:
            npx = cam.width * cam.height
            o = {"position": torch.empty((npx, 4), device=dev), "normal": torch.empty((npx, 4), device=dev),
                 "depth": torch.empty(npx, device=dev), "colour": torch.empty((npx, 4), device=dev)}
            keep.append(o)
            views.append(fm.View(s, cam, p, **o))
    torch.cuda.synchronize()
    b = fm.Batch(ctx, views)  # the context's work split (8x4 tiles, deferral after 24 sums in a batch)
    tuned = None
    if not args.no_autotune:
        # the batch's own autotuner picks tile shape, tiles per claim and deferral
        # (untimed; the timed launches below run the chosen split)
        t1 = time.perf_counter()
        best, ms = b.autotune(reps=1)
        tuned = {"best": best, "ms": ms, "seconds": time.perf_counter() - t1}
    b.run()
    ctx.sync()
    steps = max(3, min(args.steps, 5))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(ext):
        for e0, e1 in ev:
            e0.record(ext)
            b.run(ext.cuda_stream)
            e1.record(ext)
        ext.synchronize()
    ms = sum(a.elapsed_time(c) for a, c in ev) / steps
    info = b.info()
    b.close()
    for s in keep:
        if hasattr(s, "close"):
            s.close()
    return {"workload": "64 sloshing-family scenes, 50k..2M particles, 1-4 views at 640x480/1280x720/1920x1080",
            "views": info["n_views"], "pixels": info["pixels"], "particles": info["particles"],
            "graph_nodes": info["graph_nodes"], "config": info["config"], "autotune": tuned,
            "ms_per_frame": ms, "rays_per_s": info["pixels"] / (ms / 1e3), "frames_per_s": info["n_views"] / (ms / 1e3),
            "steps": steps, "scene_generation_s": gen_s}


def run_ours(args):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import __graft_entry__ as ge

    ge.build()
    import fluidmarch as fm
    from fluidmarch import scenes
    from fluidmarch.replicas import throughput

    sc = scenes.sloshing(seed=1000 + rank, width=args.width, height=args.height)
    cam = sc.cameras[0]
    npx = cam.width * cam.height
    skip = fm.FM_SKIP_EXACT if args.skip == "exact" else fm.FM_SKIP_OFF
    ctx = fm.Context(local)
    # every launch, the L2 flush and the timing events go to the context's own stream
    ext = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    xyz_d = torch.from_numpy(sc.xyz).cuda()
    torch.cuda.synchronize()
    scene = fm.Scene(ctx, xyz_d, sc.support)
    dev = torch.device("cuda", local)
    out = {"position": torch.empty((npx, 4), device=dev), "normal": torch.empty((npx, 4), device=dev),
           "depth": torch.empty(npx, device=dev), "colour": torch.empty((npx, 4), device=dev),
           "start_depth": torch.empty(npx, device=dev)}
    torch.cuda.synchronize()
    P_ext = fm.MarchParams(sc.iso, sc.step, sc.max_steps, sc.bisect, skip, external_depth=True)

    def frame():
        fm.splat_depth(scene, cam, out["start_depth"])
        fm.march(scene, cam, P_ext, out["position"], out["normal"], out["depth"], out["colour"], out["start_depth"])

    # counters for the algorithmic bytes (untimed run; after a first frame, so
    # the scene's skip table is the one the timed frames use)
    frame()
    ctx.sync()
    ctx.set_stats(True)
    frame()
    ctx.sync()
    st = ctx.stats()
    ctx.set_stats(False)

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        frame()
    ctx.sync()
    if args.profile:
        # a short, plain run for ncu (no e2e, no CPU baseline)
        for _ in range(args.steps):
            frame()
        ctx.sync()
        print(json.dumps({"profile_run": True, "frames": args.steps, "march_counters": st}))
        return
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ctx.sync()
    with ClockSampler(local) as clk, torch.cuda.stream(ext):
        for e0, e1, e2 in ev:
            flush.zero_()
            e0.record(ext)
            fm.splat_depth(scene, cam, out["start_depth"])
            e1.record(ext)
            fm.march(scene, cam, P_ext, out["position"], out["normal"], out["depth"], out["colour"],
                     out["start_depth"])
            e2.record(ext)
        ext.synchronize()
    if dist:
        dist.barrier()
    total_ms = sum(e0.elapsed_time(e2) for e0, _, e2 in ev)
    march_ms = sum(e1.elapsed_time(e2) for _, e1, e2 in ev)
    splat_ms = sum(e0.elapsed_time(e1) for e0, e1, _ in ev)
    # replicas: every rank rendered its own frames; all rays over the slowest rank's time
    value, _, t_max_s = throughput(npx * args.steps, total_ms / 1000.0, dist, dev)
    t_max = 1000.0 * t_max_s

    # e2e through the C ABI with host buffers in the library's pinned memory
    # (fm_host_alloc: the march writes the outputs there directly)
    xyz_np = ctx.host_array(sc.xyz.shape)
    xyz_np[...] = sc.xyz
    hp = {"position": ctx.host_array((npx, 4)), "normal": ctx.host_array((npx, 4)), "depth": ctx.host_array((npx,)),
          "colour": ctx.host_array((npx, 4))}
    P_full = fm.MarchParams(sc.iso, sc.step, sc.max_steps, sc.bisect, skip)

    def e2e_frame():
        scene.update(xyz_np)
        fm.march(scene, cam, P_full, hp["position"], hp["normal"], hp["depth"], hp["colour"])

    for _ in range(max(1, args.warmup // 2)):
        e2e_frame()
    ctx.sync()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_frame()
    ctx.sync()  # the march into pinned buffers returns at once; the last frame must be written
    e2e_s = time.perf_counter() - t0
    e2e_value, _, _ = throughput(npx * args.steps, e2e_s, dist, dev)

    learned = None
    if rank == 0 and not args.no_learned:
        learned = run_learned(args, fm, torch, ctx, ext, scene, sc, cam, out, flush, skip, total_ms / args.steps, st)
    batch = None
    if rank == 0 and not args.no_batch:
        batch = run_batch(args, fm, torch, ctx, ext, dev)
    aniso = None
    if rank == 0 and not args.no_aniso:
        aniso = run_aniso(args, fm, torch, ctx, ext, scene, sc, cam, out)
    files = None
    if rank == 0 and not args.no_files:
        files = run_files(args, fm, torch, ctx, sc)
    grid = None
    if rank == 0 and not args.no_grid:
        grid = run_grid(args, fm, torch, ctx, ext, sc, flush, measured_peaks()[0])

    if rank == 0:
        peak, peak_kind = measured_peaks()
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded particles)",
            "config": workload_config(sc, cam, args.skip),
            "frames_per_s": 1000.0 * args.steps * world / t_max,
            "stage_ms": {"splat": splat_ms / args.steps, "march": march_ms / args.steps},
            "march_counters": st,
            "roofline": march_roofline(st, scene.grid(), npx, march_ms / args.steps, peak, peak_kind),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 12 * sc.n,
                    "d2h_bytes_per_step": npx * (16 + 16 + 4 + 16)},
            # per frame: fill, sampled splat, tile maxima, cull, survivor splat, march, long rays
            "gpu_launches": 7 * args.steps,
            "clocks": clk.summary(),
        }
        if learned:
            line["learned"] = learned
        if batch:
            line["batch"] = batch
        if aniso:
            line["anisotropic"] = aniso
        if files:
            line["particle_files"] = files
        if grid:
            line["grid_build"] = grid
        if world == 1 and not args.no_cpu_baseline:
            # CPU legs, after all GPU timing: the oracle port of the reference loop timed on a
            # pixel sample (cpu_baseline), then the oracle as the checker of the bench frame (parity)
            import oracle as O

            O.build_oracle(ref=False)
            fr = O.build_frame(sc.xyz, sc.support)
            frame()  # the plain frame again (the anisotropic leg wrote these planes)
            ctx.sync()
            gpu = {k: v.cpu().numpy() for k, v in out.items()}
            depth = gpu["start_depth"]
            cores, model = cpu_info()
            threads = max(1, cores - 1)
            v, npix, secs = cpu_baseline_sample(sc, cam, depth, fr, args.cpu_seconds, threads)
            line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                                    "sample": f"{npix} seeded random pixels of the same 1920x1080 frame "
                                              f"({secs:.1f} s), bisection 0, skipping off; CPU {model}, "
                                              f"{cores} host cores"}
            line["parity"] = frame_parity(O, fr, sc, cam, gpu, threads)
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
