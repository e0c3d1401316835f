"""GPU splat + march + shading against the CPU oracle and the reference's golden vectors.

Bit-exact where the oracle follows the same summation order (it does: the
canonical cell order), and within the stated tolerances against the FP64
re-evaluation of the same march:
  * hit/miss mask identical except where |rho_hit - iso| <= 1e-3 iso,
  * hit depth within 1e-4 of the scene extent,
  * normals within 0.5 degrees.
"""

import glob
import math
import os

import numpy as np
import pytest

import oracle as O
from fluidmarch import scenes

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def gpu_render(fm, ctx, sc, cam, bisect, skip=0, external=None):
    s = fm.Scene(ctx, sc.xyz, sc.support)
    p = fm.MarchParams(sc.iso, sc.step, sc.max_steps, bisect, skip, external is not None)
    npx = cam.width * cam.height
    out = {"position": np.zeros((npx, 4), np.float32), "normal": np.zeros((npx, 4), np.float32),
           "depth": np.zeros(npx, np.float32), "colour": np.zeros((npx, 4), np.float32),
           "start_depth": (np.array(external, np.float32) if external is not None else np.zeros(npx, np.float32))}
    fm.march(s, cam, p, out["position"], out["normal"], out["depth"], out["colour"], out["start_depth"])
    s.close()
    return out


def assert_same(g, o, pixels=None):
    for k in ("position", "normal", "depth", "colour"):
        a = g[k] if pixels is None else g[k][pixels]
        b = o[k] if pixels is None else o[k][pixels]
        bad = np.nonzero(np.any((bits(a) != bits(b)).reshape(a.shape[0], -1), axis=1))[0]
        assert bad.size == 0, f"{k}: {bad.size} pixels differ, first {bad[:5]}"


# ---- splat -------------------------------------------------------------------

@pytest.mark.parametrize("which", ["small", "dam"])
def test_splat_bitwise(fmlib, ctx, which):
    sc = scenes.small_scene(seed=3, n=5000, width=160, height=120) if which == "small" else scenes.dam_break()
    cam = sc.cameras[0]
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    d = fmlib.splat_depth(s, cam)
    o = O.splat(sc.xyz, sc.support, cam)
    assert np.array_equal(bits(d), bits(o))
    assert (d < 1).sum() > 1000


def test_splat_sloshing_1080p(fmlib, ctx):
    sc = scenes.sloshing()
    cam = sc.cameras[0]
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    d = fmlib.splat_depth(s, cam)
    o = O.splat(sc.xyz, sc.support, cam)
    assert np.array_equal(bits(d), bits(o))


# ---- march, bit-exact against the oracle --------------------------------------

@pytest.mark.parametrize("bisect", [0, 8])
@pytest.mark.parametrize("skip", [0, 1, 2])
def test_march_small_bitwise(fmlib, ctx, bisect, skip):
    sc = scenes.small_scene(seed=21, n=8000, width=120, height=90)
    cam = sc.cameras[0]
    g = gpu_render(fmlib, ctx, sc, cam, bisect, skip)
    fr = O.build_frame(sc.xyz, sc.support)
    depth = O.splat(sc.xyz, sc.support, cam)
    assert np.array_equal(bits(g["start_depth"]), bits(depth))
    o = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, bisect, depth, skip_mode=2 if skip == 2 else 0, threads=0)
    assert_same(g, o)
    assert (g["position"][:, 3] == 1).sum() > 500


@pytest.mark.parametrize("bisect", [0, 8])
def test_march_dam_break_full(fmlib, ctx, bisect):
    """640x480 dam break (64,000 particles, support 0.1): every pixel bit-exact against the oracle."""
    sc = scenes.dam_break()
    cam = sc.cameras[0]
    g = gpu_render(fmlib, ctx, sc, cam, bisect)
    fr = O.build_frame(sc.xyz, sc.support)
    o = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, bisect, g["start_depth"], threads=0)
    assert_same(g, o)
    assert (g["position"][:, 3] == 1).sum() > 50000


@pytest.fixture(scope="module")
def slosh(fmlib, ctx):
    """The 1920x1080 frame of the 1,000,000-particle sloshing scene (support 0.04, iso 0.5 rest density,
    step 0.005, 1024 steps, 8 bisections, exact skip) on the GPU, and the oracle's march of every pixel
    from the GPU's start depths (whose splat is checked against the oracle's separately)."""
    sc = scenes.sloshing()
    cam = sc.cameras[0]
    g = gpu_render(fmlib, ctx, sc, cam, 8, skip=1)
    fr = O.build_frame(sc.xyz, sc.support)
    o = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 8, g["start_depth"], threads=0)
    return sc, cam, fr, g, o


def test_march_sloshing_1080p_full(slosh):
    """Every one of the 2,073,600 pixels (394,543 started) bit-exact against the oracle."""
    sc, cam, fr, g, o = slosh
    assert int((g["start_depth"] < 1).sum()) > 390_000
    assert_same(g, o)
    assert (g["position"][:, 3] == 1).sum() > 190_000


def test_tolerances_vs_fp64_sloshing_1080p(fmlib, ctx, slosh):
    """The headline frame against the FP64 re-evaluation of the same march, every started pixel:
    hit masks identical except where |rho - iso| <= 1e-3 iso, hit depth within 1e-4 of the scene
    extent and normals within 0.5 degrees on at least 99.9% of the hits."""
    sc, cam, fr, g, _ = slosh
    z = g["start_depth"]
    # the mask is decided at the first sample with rho >= iso (bisection only refines the hit):
    # the densities there, FP32 and FP64, come from the marches without bisection
    o32_0 = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 0, z, threads=0, want_colour=False)
    o64_0 = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 0, z, threads=0, precision=64, want_colour=False)
    hg = g["position"][:, 3] == 1
    assert np.array_equal(hg, o32_0["position"][:, 3] == 1)
    h64 = o64_0["position"][:, 3] == 1
    for sel, rho in ((hg & ~h64, o32_0["rho"]), (h64 & ~hg, o64_0["rho"])):
        assert np.all(np.abs(rho[sel] - sc.iso) <= 1e-3 * sc.iso)
    o64 = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 8, z, threads=0, precision=64, want_colour=False)
    h64 = o64["position"][:, 3] == 1
    both = hg & h64
    ext = float(np.max(sc.xyz.max(0) - sc.xyz.min(0)))
    derr = np.abs(g["depth"][both].astype(np.float64) - o64["depth"][both])
    assert np.mean(derr <= 1e-4 * ext) >= 0.999
    n1 = g["normal"][both, :3].astype(np.float64)
    n2 = o64["normal"][both, :3].astype(np.float64)
    cosang = np.sum(n1 * n2, 1) / np.linalg.norm(n1, axis=1) / np.linalg.norm(n2, axis=1)
    ang = np.degrees(np.arccos(np.clip(cosang, -1, 1)))
    assert np.mean(ang <= 0.5) >= 0.999


def test_skip_exact_equals_skip_off_full_size(fmlib, ctx):
    """FM_SKIP_EXACT steps over cells whose density bound is below iso: same bits as no skipping."""
    sc = scenes.sloshing()
    cam = sc.cameras[0]
    a = gpu_render(fmlib, ctx, sc, cam, 8, skip=0)
    b = gpu_render(fmlib, ctx, sc, cam, 8, skip=1)
    assert_same(a, b)


# ---- golden vectors from the reference's own RayMarcher -----------------------

class _Cam:
    def __init__(self, z):
        self.view, self.proj, self.inv_proj_view = z["view"], z["proj"], z["inv_proj_view"]
        self.position, self.width, self.height = z["cam_pos"], int(z["width"]), int(z["height"])

    @property
    def n_pixels(self):
        return self.width * self.height


@pytest.mark.skipif(not GOLDEN, reason="no golden vectors")
@pytest.mark.parametrize("external", [True, False])
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_march_matches_reference_golden(fmlib, ctx, path, external):
    z = dict(np.load(path))
    cam = _Cam(z)
    sc = scenes.Scene("golden", z["xyz"], float(z["support"]), float(z["iso"]), float(z["step"]), int(z["max_steps"]), 0)
    skip = 2 if int(z["box_mode"]) == 1 else 0
    g = gpu_render(fmlib, ctx, sc, cam, 0, skip, external=z["start_depth"] if external else None)
    last = cam.n_pixels - 1  # never marched by the reference
    for k in ("position", "normal"):
        x = g[k].copy()
        x[last] = 0
        assert np.array_equal(bits(x), bits(z["ref_" + k])), k


# ---- tolerances against the FP64 re-evaluation ----------------------------------

def test_tolerances_vs_fp64(fmlib, ctx):
    """The 640x480 dam break against the FP64 re-evaluation, every started pixel."""
    sc = scenes.dam_break()
    cam = sc.cameras[0]
    fr = O.build_frame(sc.xyz, sc.support)
    # hit mask at the march samples (no bisection): decided by rho >= iso at the first crossing
    g0 = gpu_render(fmlib, ctx, sc, cam, 0)
    pix = np.nonzero(g0["start_depth"] < 1)[0]
    o32 = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 0, g0["start_depth"], pixels=pix)
    o64 = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 0, g0["start_depth"], pixels=pix, precision=64)
    hg = g0["position"][pix, 3] == 1
    assert np.array_equal(hg, o32["position"][pix, 3] == 1)
    h64 = o64["position"][pix, 3] == 1
    for sel, rho in ((hg & ~h64, o32["rho"][pix]), (h64 & ~hg, o64["rho"][pix])):
        assert np.all(np.abs(rho[sel] - sc.iso) <= 1e-3 * sc.iso)
    # depth and normal after 8 bisections
    g = gpu_render(fmlib, ctx, sc, cam, 8)
    o64 = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 8, g["start_depth"], pixels=pix, precision=64)
    hg = g["position"][pix, 3] == 1
    h64 = o64["position"][pix, 3] == 1
    both = hg & h64
    ext = float(np.max(sc.xyz.max(0) - sc.xyz.min(0)))
    derr = np.abs(g["depth"][pix][both] - o64["depth"][pix][both])
    assert np.quantile(derr, 0.999) <= 1e-4 * ext
    n1 = g["normal"][pix][both, :3].astype(np.float64)
    n2 = o64["normal"][pix][both, :3].astype(np.float64)
    cosang = np.sum(n1 * n2, 1) / np.linalg.norm(n1, axis=1) / np.linalg.norm(n2, axis=1)
    ang = np.degrees(np.arccos(np.clip(cosang, -1, 1)))
    assert np.quantile(ang, 0.999) <= 0.5


# ---- full-size properties ----------------------------------------------------------

def test_sloshing_properties(slosh):
    sc, cam, fr, g, _ = slosh
    hit = g["position"][:, 3] == 1
    assert hit.sum() > 150000
    n = g["normal"][hit, :3]
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-5)
    assert np.all(g["position"][~hit] == 0) and np.all(g["normal"][~hit] == 0) and np.all(g["depth"][~hit] == 0)
    assert np.all(np.isfinite(g["colour"]))
    # every hit point is inside the iso surface (FP32 canonical sum = what the GPU evaluated)
    idx = np.nonzero(hit)[0]
    rho = O.density(fr, g["position"][idx, :3], precision=32)
    assert np.all(rho >= sc.iso)
    # hit distance equals |p - camera|
    d = np.linalg.norm(g["position"][idx, :3].astype(np.float64) - cam.position.astype(np.float64), axis=1)
    assert np.allclose(g["depth"][idx], d, rtol=1e-6)


def test_device_outputs_match_host_outputs(fmlib, ctx):
    torch = pytest.importorskip("torch")
    sc = scenes.small_scene(seed=30, n=6000, width=100, height=80)
    cam = sc.cameras[0]
    h = gpu_render(fmlib, ctx, sc, cam, 8, skip=1)
    s = fmlib.Scene(ctx, torch.from_numpy(sc.xyz).cuda(), sc.support)
    npx = cam.n_pixels
    dev = {k: torch.zeros((npx, 4) if k in ("position", "normal", "colour") else (npx,), device="cuda")
           for k in ("position", "normal", "depth", "colour", "start_depth")}
    fmlib.march(s, cam, fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 8, 1), dev["position"], dev["normal"],
                dev["depth"], dev["colour"], dev["start_depth"])
    ctx.sync()
    for k in dev:
        assert np.array_equal(bits(dev[k].cpu().numpy()), bits(h[k])), k


def test_stats_match_oracle_counts(fmlib, ctx):
    sc = scenes.small_scene(seed=31, n=6000, width=80, height=60)
    cam = sc.cameras[0]
    ctx.set_stats(True)
    try:
        g = gpu_render(fmlib, ctx, sc, cam, 8, skip=0)
        st = ctx.stats()
    finally:
        ctx.set_stats(False)
    fr = O.build_frame(sc.xyz, sc.support)
    o = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 8, g["start_depth"], threads=0)
    hits = int((o["position"][:, 3] == 1).sum())
    assert st["hits"] == hits
    assert st["rays"] == cam.n_pixels
    assert st["started"] == int((g["start_depth"] < 1).sum())
    # the oracle counts march + bisection evaluations; the GPU also counts the normal pass
    assert st["evals"] == int(o["evals"].sum()) + hits


def test_raymarcher_prepare_start_exit(fmlib, ctx):
    """The reference-shaped host interface: Prepare(settings, camera, frame, positions, normals, depth)."""
    sc = scenes.small_scene(seed=32, n=5000, width=64, height=48)
    cam = sc.cameras[0]
    rm = fmlib.RayMarcher(0)
    s = fmlib.Scene(rm.ctx, sc.xyz, sc.support)
    depth = fmlib.splat_depth(s, cam)
    pos = np.zeros((cam.n_pixels, 4), np.float32)
    nrm = np.zeros((cam.n_pixels, 4), np.float32)
    rm.prepare(fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 0), cam, s, pos, nrm, depth)
    rm.start()
    rm.exit()
    assert rm.is_done()
    fr = O.build_frame(sc.xyz, sc.support)
    o = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 0, depth, threads=0)
    assert np.array_equal(bits(pos), bits(o["position"])) and np.array_equal(bits(nrm), bits(o["normal"]))


def test_march_rejects_bad_params(fmlib, ctx):
    sc = scenes.small_scene(seed=33, n=2000, width=16, height=16)
    cam = sc.cameras[0]
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    out = np.zeros((cam.n_pixels, 4), np.float32)
    for bad in (fmlib.MarchParams(sc.iso, 0.0, 10), fmlib.MarchParams(sc.iso, sc.step, -1),
                fmlib.MarchParams(float("nan"), sc.step, 10), fmlib.MarchParams(sc.iso, sc.step, 10, 65),
                fmlib.MarchParams(sc.iso, sc.step, 10, 0, 7)):
        with pytest.raises(fmlib.FmError) as e:
            fmlib.march(s, cam, bad, position=out)
        assert e.value.code == fmlib.FM_ERR_INVALID
    import copy
    c2 = copy.copy(cam)
    c2.width = 0
    with pytest.raises(fmlib.FmError):
        fmlib.march(s, c2, fmlib.MarchParams(sc.iso, sc.step, 10), position=out)


def test_density_probe_bitwise(fmlib, ctx):
    """fm_density (DiskRenderer::ComputeDensity) equals the oracle's FP32 density bit for bit."""
    sc = scenes.small_scene(seed=12, n=20000, width=64, height=48)
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    rng = np.random.default_rng(0)
    pts = np.concatenate([sc.xyz[rng.choice(sc.n, 3000, replace=False)] + rng.normal(0, sc.support / 3, (3000, 3)),
                          rng.uniform(-0.5, 1.5, (1000, 3))]).astype(np.float32)
    got = fmlib.density(s, pts)
    fr = O.build_frame(sc.xyz, sc.support)
    ref = O.density(fr, pts).astype(np.float32)
    assert np.array_equal(bits(got), bits(ref))
    assert (got > 0).sum() > 2500
    s.close()


def test_bound_table_on_reuse(fmlib, ctx):
    """The scene's first exact-skip march builds both levels of the bound table (4x4x4 boxes, then the
    shell boxes refined into eighths); later marches of the same build reuse it: the oracle's bits
    every time, the same samples skipped and evaluated every time, and fewer evaluations than with the
    skip off."""
    sc = scenes.small_scene(seed=23, n=20000, width=128, height=96)
    cam = sc.cameras[0]
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    p = fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 8, fmlib.FM_SKIP_EXACT)
    p_off = fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 8, fmlib.FM_SKIP_OFF)
    ctx.set_stats(True)
    try:
        runs = []
        for _ in range(3):
            runs.append((fmlib.render(s, cam, p), ctx.stats()))
        fmlib.render(s, cam, p_off)
        st_off = ctx.stats()
    finally:
        ctx.set_stats(False)
    fr = O.build_frame(sc.xyz, sc.support)
    o = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 8, O.splat(sc.xyz, sc.support, cam))
    for g, _ in runs:
        for k in ("position", "normal", "depth", "colour"):
            assert np.array_equal(bits(g[k]), bits(o[k])), k
    (_, st1), (_, st2), (_, st3) = runs
    assert st1["skipped"] > 0 and st1["evals"] < st_off["evals"]
    assert (st1["skipped"], st1["evals"]) == (st2["skipped"], st2["evals"]) == (st3["skipped"], st3["evals"])
    s.close()


def test_bound_table_follows_iso(fmlib, ctx):
    """The bound table stops summing a cell once every box reached the iso density of the march that
    built it (+inf there), and refines the boxes whose bound lies between that iso and +inf: marches at
    that iso or a lower one reuse it, a march at a higher iso builds it again.  Every march equals the
    march without skipping bit for bit; a march at the table's own iso skips at least as many samples
    as one at that iso reading a table built for a higher iso."""
    sc = scenes.small_scene(seed=29, n=20000, width=128, height=96)
    cam = sc.cameras[0]
    ctx.set_stats(True)
    own = {}
    try:
        for iso in (sc.iso, 0.5 * sc.iso, 2.0 * sc.iso):
            s = fmlib.Scene(ctx, sc.xyz, sc.support)
            p = fmlib.MarchParams(iso, sc.step, sc.max_steps, 8, fmlib.FM_SKIP_EXACT)
            for _ in range(2):  # built at this iso, then refined
                fmlib.render(s, cam, p)
            own[iso] = ctx.stats()["skipped"]
            s.close()
        s = fmlib.Scene(ctx, sc.xyz, sc.support)
        # tables: built at iso and refined, reused (iso / 2), built at 2 iso and refined, reused (iso),
        # built at 3 iso, reused (iso / 2, 2 iso)
        for iso in (sc.iso, sc.iso, 0.5 * sc.iso, 2.0 * sc.iso, 2.0 * sc.iso, sc.iso, 3.0 * sc.iso, 0.5 * sc.iso,
                    2.0 * sc.iso):
            ref = fmlib.render(s, cam, fmlib.MarchParams(iso, sc.step, sc.max_steps, 8, fmlib.FM_SKIP_OFF))
            got = fmlib.render(s, cam, fmlib.MarchParams(iso, sc.step, sc.max_steps, 8, fmlib.FM_SKIP_EXACT))
            st = ctx.stats()
            for k in ("position", "normal", "depth", "colour"):
                assert np.array_equal(bits(got[k]), bits(ref[k])), (iso, k)
            if iso in own:
                assert st["skipped"] <= own[iso], iso
        assert own[sc.iso] > 0
        s.close()
    finally:
        ctx.set_stats(False)


def test_outputs_in_library_pinned_memory(fmlib, ctx):
    """Outputs in fm_host_alloc memory are written by the kernels directly (no copy after the
    march); they equal the staged outputs of pageable buffers, also for a view inside a larger
    block and with only some outputs pinned."""
    sc = scenes.small_scene(seed=13, n=15000, width=150, height=90)
    cam = sc.cameras[0]
    npx = cam.width * cam.height
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    p = fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 8, fmlib.FM_SKIP_EXACT)
    want = fmlib.render(s, cam, p)
    big = ctx.host_array((npx + 100, 4))  # the outputs start 64 pixels into the block
    pin = {"position": big[64:64 + npx], "normal": ctx.host_array((npx, 4)), "depth": ctx.host_array((npx,)),
           "colour": np.zeros((npx, 4), np.float32)}
    for v in pin.values():
        v[...] = -1.0
    fmlib.march(s, cam, p, pin["position"], pin["normal"], pin["depth"], pin["colour"])
    for k in pin:
        assert np.array_equal(bits(pin[k]), bits(want[k])), k
    # every host buffer in the library's memory: the call returns at once and
    # fm_sync completes it
    allp = {k: ctx.host_array(v.shape) for k, v in want.items()}
    for v in allp.values():
        v[...] = -1.0
    fmlib.march(s, cam, p, allp["position"], allp["normal"], allp["depth"], allp["colour"], allp["start_depth"])
    ctx.sync()
    for k in allp:
        assert np.array_equal(bits(allp[k]), bits(want[k])), k
    s.close()
