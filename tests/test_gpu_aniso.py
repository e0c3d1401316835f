"""The anisotropic march (RayMarcher.cpp:346-423) on the GPU against the oracle.

The oracle's restatement is pinned against the reference's own
PerPixel_Anisotropic (tests/test_oracle.py).  The GPU reduces its WPCA sums
over the warp in a different order than the oracle's sequential loop, so the
comparison is to rounding: hit masks identical except where the density at the
hit sample is within 1e-3 of iso, the same hit samples (bisection 0), normals
within 0.5 degrees, refined hit depths within 1e-4 of the scene extent.
"""

import numpy as np
import pytest

import oracle as O
from fluidmarch import scenes

pytestmark = pytest.mark.gpu

ANISO = (2.0, 0.5, 2.0, 2000.0, 1)


def aniso_iso(fr, xyz):
    inner = xyz[(xyz[:, 1] < 0.2) & (xyz[:, 0] > 0.3) & (xyz[:, 0] < 0.7) & (xyz[:, 2] > 0.3) & (xyz[:, 2] < 0.7)]
    return float(np.float32(0.5 * np.median(O.density_aniso(fr, inner[:200], ANISO))))


def angles(a, b):
    c = np.sum(a * b, 1) / np.linalg.norm(a, axis=1) / np.linalg.norm(b, axis=1)
    return np.degrees(np.arccos(np.clip(c, -1, 1)))


@pytest.mark.parametrize("n,w,h,bisect,skip", [(3000, 48, 36, 0, 0), (12000, 64, 48, 0, 2), (12000, 64, 48, 8, 0)])
def test_aniso_march_vs_oracle(fmlib, ctx, n, w, h, bisect, skip):
    sc = scenes.small_scene(seed=5, n=n, width=w, height=h, max_steps=120)
    cam = sc.cameras[0]
    fr = O.build_frame(sc.xyz, sc.support)
    iso = aniso_iso(fr, sc.xyz)
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    ctx.set_anisotropy(*ANISO)
    p = fmlib.MarchParams(iso, sc.step, sc.max_steps, bisect, skip, anisotropic=True)
    g = fmlib.render(s, cam, p)
    depth = O.splat(sc.xyz, sc.support, cam)
    assert np.array_equal(g["start_depth"], depth)
    o = O.march_aniso(fr, cam, iso, sc.step, sc.max_steps, bisect, depth, ANISO, skip_mode=skip)
    hg, ho = g["depth"] > 0, o["depth"] > 0
    assert ho.sum() > 200
    bad = np.nonzero(hg != ho)[0]
    if bad.size:
        # a mismatch must sit on a sample whose density is within 1e-3 of iso
        pts = np.where(hg[bad, None], g["position"][bad, :3], o["position"][bad, :3])
        rho = O.density_aniso(fr, pts, ANISO)
        assert np.all(np.abs(rho - iso) <= 1e-3 * iso), (bad, rho, iso)
    assert bad.size <= max(2, ho.sum() // 500)
    both = hg & ho
    extent = float((sc.xyz.max(0) - sc.xyz.min(0)).max())
    if bisect == 0:
        same = np.all(g["position"][both] == o["position"][both], axis=1)
        assert same.mean() > 0.999
    else:
        assert np.percentile(np.abs(g["depth"][both] - o["depth"][both]), 99.9) <= 1e-4 * extent
    assert np.percentile(angles(g["normal"][both, :3], o["normal"][both, :3]), 99.9) < 0.5
    s.close()


@pytest.mark.parametrize("bisect", [0, 8])
def test_aniso_exact_skip_equals_no_skip(fmlib, ctx, bisect):
    """FM_SKIP_EXACT steps over samples whose bound box has no particle within the support radius
    (anisotropic density exactly 0): every output equals the march without skipping, bit for bit,
    when the march builds the bound table (both levels) and when a later march reuses it."""
    sc = scenes.small_scene(seed=8, n=12000, width=72, height=54, max_steps=160)
    cam = sc.cameras[0]
    fr = O.build_frame(sc.xyz, sc.support)
    iso = aniso_iso(fr, sc.xyz)
    ctx.set_anisotropy(*ANISO)
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    off = fmlib.render(s, cam, fmlib.MarchParams(iso, sc.step, sc.max_steps, bisect, fmlib.FM_SKIP_OFF,
                                                 anisotropic=True))
    p = fmlib.MarchParams(iso, sc.step, sc.max_steps, bisect, fmlib.FM_SKIP_EXACT, anisotropic=True)
    ctx.set_stats(True)
    try:
        first = fmlib.render(s, cam, p)  # the scene's first exact march builds the table
        st_1 = ctx.stats()
        again = fmlib.render(s, cam, p)  # the next one reuses it
        st_2 = ctx.stats()
    finally:
        ctx.set_stats(False)
    for got in (first, again):
        for k in ("position", "normal", "depth", "colour"):
            assert np.array_equal(got[k].view(np.uint32), off[k].view(np.uint32)), k
    assert (off["depth"] > 0).sum() > 200
    assert st_1["skipped"] > 0 and st_2["skipped"] == st_1["skipped"]
    s.close()


def test_aniso_rejects_bad_combinations(fmlib, ctx):
    sc = scenes.small_scene(seed=6, n=2000, width=16, height=12)
    s = fmlib.Scene(ctx, sc.xyz, sc.support)
    with pytest.raises(fmlib.FmError):
        fmlib.render(s, sc.cameras[0], fmlib.MarchParams(1.0, sc.step, 10, 0, fmlib.FM_SKIP_EXACT, anisotropic=True,
                                                         proposal=True))
    with pytest.raises(fmlib.FmError):
        ctx.set_anisotropy(3.0)
    with pytest.raises(fmlib.FmError):
        ctx.set_anisotropy(k_s=-1.0)
    ctx.set_anisotropy(*ANISO)
    s.close()
