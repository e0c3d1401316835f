"""Learned proposal and batching at scale.

The workload: scenes of the sloshing family with 4,000,000 particles
(h = 0.0126, support 0.0252, step h/4, 1024 steps, 8 bisections), 16 views
per scene at 3840x2160 on a seeded camera orbit, 8 scenes per launch: 128
views, 1.06 G rays per launch.

* ``fine_tune``  fine-tunes the committed proposal MLP (trained at 1M
  particles, 1920x1080) on plain-march first hits of separate seeded
  4M-particle scenes rendered at 3840x2160, with the same trainer kernels
  (forward, backward, Adam) and a lower learning rate;
* ``ScaleRun``   puts the 8 x 16 views into two batches, one marching with the
  learned proposal and one plain (exact skip), each one CUDA-graph launch per
  frame.  The two share the position / normal / colour planes and keep their
  own depth planes, so every learned view is judged against its plain view
  (hit masks, depth error within 1e-4 of the scene extent) on the device.

    python -m fluidmarch.scale [--scenes 8] [--views 16] [--width 3840] [--height 2160]
                               [--particles 4000000] [--steps 2] [--warmup 1]

prints one JSON object: fine-tuning coverage before / after, both batches'
rays/s, and the per-view judge results.
"""

from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

import fluidmarch as fm
from fluidmarch import proposal as PR
from fluidmarch import scenes

FT_SEED0, FT_HELDOUT_SEED0, EVAL_SEED0 = 300_000, 350_000, 400_000
MARGINS = (0.5, 0.5, 8.0)  # margin_lo, margin_hi, min_near in support radii


def _torch():
    import torch

    return torch


def orbit(seed: int, views: int, width: int, height: int) -> list:
    """`views` cameras on one circle around the column: seeded radius, height and phase."""
    rng = np.random.default_rng(seed)
    rad = rng.uniform(1.5, 2.1)
    y = rng.uniform(0.8, 1.6)
    phase = rng.uniform(0, 2 * math.pi)
    cams = []
    for k in range(views):
        a = phase + 2 * math.pi * k / views
        cams.append(scenes.make_camera((0.5 + rad * math.cos(a), y, 0.5 + rad * math.sin(a)), (0.5, 0.3, 0.5),
                                       width, height))
    return cams


def fine_tune(ctx: fm.Context, P0: np.ndarray, n: int, width: int, height: int, train_scenes: int = 24,
              heldout_scenes: int = 4, per_scene: int = 8192, epochs: int = 8, lr: float = 5e-4, log=None) -> tuple:
    """(fine-tuned parameters, coverage report before and after on held-out scenes)."""
    X, T = PR.collect(ctx, range(FT_SEED0, FT_SEED0 + train_scenes), per_scene, n, width, height)
    Xh, Th = PR.collect(ctx, range(FT_HELDOUT_SEED0, FT_HELDOUT_SEED0 + heldout_scenes), per_scene, n, width,
                        height)
    before = PR.evaluate(ctx, P0, Xh, Th)
    P = PR.train(ctx, X, T, epochs=epochs, lr=lr, init=P0, log=log)
    after = PR.evaluate(ctx, P, Xh, Th)
    return P, {"train_scenes": train_scenes, "heldout_scenes": heldout_scenes, "rays": int(X.shape[0]),
               "heldout_rays": int(Xh.shape[0]), "epochs": epochs, "lr": lr, "before": before, "after": after}


class ScaleRun:
    """The scenes, the views and the two batches (learned and plain) of one scale workload."""

    def __init__(self, ctx: fm.Context, proposal: fm.Proposal, n_scenes: int = 8, views: int = 16,
                 width: int = 3840, height: int = 2160, n: int = 4_000_000, seed0: int = EVAL_SEED0):
        torch = _torch()
        self.ctx = ctx
        H, iso, step, max_steps = PR.family_settings(n)
        self.H = H
        self.settings = {"support": H, "iso": iso, "step": step, "max_steps": max_steps, "bisect": 8}
        self.scenes, self.xyz, self.extent, self.cams = [], [], [], []
        for i in range(n_scenes):
            xyz = PR.sloshing_xyz_gpu(seed0 + i, n)
            self.xyz.append(xyz)
            self.extent.append(float((xyz.max(0).values - xyz.min(0).values).max()))
            self.scenes.append(fm.Scene(ctx, xyz, H))
            self.cams.append(orbit(seed0 + i, views, width, height))
        torch.cuda.synchronize()
        npx = width * height
        nv = n_scenes * views
        dev = dict(device="cuda", dtype=torch.float32)
        # shared planes (written by whichever batch ran last), own depth planes
        self.position = torch.zeros((nv, npx, 4), **dev)
        self.normal = torch.zeros((nv, npx, 4), **dev)
        self.colour = torch.zeros((nv, npx, 4), **dev)
        self.depth_plain = torch.zeros((nv, npx), **dev)
        self.depth_learned = torch.zeros((nv, npx), **dev)
        self.start_depth = torch.zeros((nv, npx), **dev)
        plain = fm.MarchParams(iso, step, max_steps, 8, fm.FM_SKIP_EXACT)
        learned = fm.MarchParams(iso, step, max_steps, 8, fm.FM_SKIP_EXACT, proposal=True)
        vp, vl = [], []
        for i in range(n_scenes):
            for k in range(views):
                j = i * views + k
                common = dict(position=self.position[j], normal=self.normal[j], colour=self.colour[j],
                              start_depth=self.start_depth[j])
                vp.append(fm.View(self.scenes[i], self.cams[i][k], plain, depth=self.depth_plain[j], **common))
                vl.append(fm.View(self.scenes[i], self.cams[i][k], learned, depth=self.depth_learned[j], **common))
        fm.set_proposal(ctx, proposal)
        try:
            self.plain = fm.Batch(ctx, vp)
            self.learned = fm.Batch(ctx, vl)  # keeps its own copy of the proposal
        finally:
            fm.set_proposal(ctx, None)
        self.views, self.npx = nv, npx
        self.pixels = nv * npx

    def time(self, batch: fm.Batch, steps: int, warmup: int) -> float:
        """Mean ms per launch over `steps` CUDA-event-timed launches after `warmup` (outputs exceed L2)."""
        torch = _torch()
        st = torch.cuda.Stream()
        with torch.cuda.stream(st):
            for _ in range(warmup):
                batch.run(st.cuda_stream)
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
            for e0, e1 in ev:
                e0.record(st)
                batch.run(st.cuda_stream)
                e1.record(st)
        st.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) / steps

    def judge(self) -> list:
        """Per view: the learned depth plane judged against the plain one (tolerance 1e-4 of the extent)."""
        out = []
        for j in range(self.views):
            tol = 1e-4 * self.extent[j // len(self.cams[0])]
            r = fm.judge(self.ctx, self.depth_plain[j], self.depth_learned[j], tol)
            r["hits_within_tol"] = r["within_tol"] / max(1, r["hits_ref"])
            out.append(r)
        return out

    def close(self):
        self.learned.close()
        self.plain.close()
        for s in self.scenes:
            s.close()


def run(ctx: fm.Context, n_scenes: int = 8, views: int = 16, width: int = 3840, height: int = 2160,
        n: int = 4_000_000, steps: int = 2, warmup: int = 1, tune: bool = True, log=None) -> tuple:
    """(report, ScaleRun): fine-tune, build both batches, time them, judge every view."""
    P0, meta = PR.load()
    t0 = time.time()
    ft = None
    P = P0
    if tune:
        P, ft = fine_tune(ctx, P0, n, width, height, log=log)
        ft["seconds"] = time.time() - t0
    prop = fm.Proposal(ctx, P, *MARGINS)
    sr = ScaleRun(ctx, prop, n_scenes, views, width, height, n)
    prop.close()
    ms_plain = sr.time(sr.plain, steps, warmup)
    ms_learned = sr.time(sr.learned, steps, warmup)
    jv = sr.judge()
    rep = {
        "workload": f"{n_scenes} sloshing scenes x {n} particles, {views} views each at {width}x{height}",
        "settings": sr.settings,
        "views": sr.views,
        "rays_per_launch": sr.pixels,
        "fine_tune": ft,
        "margins_support_radii": list(MARGINS[:2]),
        "min_near_support_radii": MARGINS[2],
        "plain": {"ms_per_launch": ms_plain, "rays_per_s": sr.pixels / (ms_plain / 1e3),
                  "frames_per_s": sr.views / (ms_plain / 1e3)},
        "learned": {"ms_per_launch": ms_learned, "rays_per_s": sr.pixels / (ms_learned / 1e3),
                    "frames_per_s": sr.views / (ms_learned / 1e3)},
        "learned_vs_plain": ms_plain / ms_learned,
        "judge": {
            "views_mask_identical": sum(int(r["mask_mismatch"] == 0) for r in jv),
            "min_hits_within_tol": min(r["hits_within_tol"] for r in jv),
            "max_err": max(r["max_err"] for r in jv),
            "per_view": [{k: r[k] for k in ("hits_ref", "mask_mismatch", "within_tol", "max_err", "tol")}
                         for r in jv],
        },
    }
    return rep, sr


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--scenes", type=int, default=8)
    ap.add_argument("--views", type=int, default=16)
    ap.add_argument("--width", type=int, default=3840)
    ap.add_argument("--height", type=int, default=2160)
    ap.add_argument("--particles", type=int, default=4_000_000)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--no-tune", action="store_true", help="use the committed weights as they are")
    a = ap.parse_args(argv)
    ctx = fm.Context(0)
    rep, sr = run(ctx, a.scenes, a.views, a.width, a.height, a.particles, a.steps, a.warmup, not a.no_tune)
    sr.close()
    print(json.dumps(rep))


if __name__ == "__main__":
    main()
