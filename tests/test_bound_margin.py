"""The exact skip's density bound, restated on the CPU and checked against the oracle's density.

The skip steps over a sample when the bound of its bound box (a quarter cell per axis) is below the
iso density, so it is exact only if no sample located in a box has a density above the box's bound.
This restates the bound table of grid_build.cu (k_cell_bound4) in numpy FP32: per box, W at each
27-neighbourhood particle's distance to the box grown by the slack, summed (numpy's pairwise order,
not the kernel's: the margin is meant to cover any order) and inflated by the same margin; a cell
whose 64 sums all reach the iso density stores +inf.  Random samples (uniform in boxes, at box
corners and at the particles themselves), located as the march locates them, must have an FP32
oracle density no larger than their box's bound.
"""

import numpy as np
import pytest

import oracle as O
from fluidmarch import scenes

EPS = np.float32(5.9604645e-8)  # 2^-24


def w_in(q2, h, hinv, sig):
    """CubicSplineKernel::W for q2 < h^2, FP32 as the kernels evaluate it (Kernel.cpp:16-32)."""
    f = np.float32
    q = np.sqrt(q2.astype(f)).astype(f) * f(hinv)
    qm = f(1) - q
    a = f(sig) * (((f(2) * qm) * qm) * qm)
    b = f(sig) * (f(6) * (((q * q) * q) - (q * q)) + f(1))
    return np.where(q >= f(0.5), a, b).astype(f)


def bound_table(fr, thr):
    f = np.float32
    g = fr.grid
    dims = [int(g.dims[a]) for a in range(3)]
    gmin = np.array(g.min[:], f)
    gmax = np.array(g.max[:], f)
    cell = f(g.cell)
    h = f(fr.support)
    h2 = h * h
    hinv = f(1) / h
    sig = f(8) / (((f(np.pi) * h) * h) * h)
    amax = max(np.abs(gmin).max(), np.abs(gmax).max())
    slack = f(1e-4) * h + f(1e-6) * f(amax)
    pts = fr.sorted[:, :3]
    start = fr.start
    ncells = dims[0] * dims[1] * dims[2]
    out = np.zeros((ncells, 64), f)
    ib = np.arange(4, dtype=f)
    for c in range(ncells):
        cx, cy, cz = c % dims[0], (c // dims[0]) % dims[1], c // (dims[0] * dims[1])
        idx = []
        for z in range(max(cz - 1, 0), min(cz + 1, dims[2] - 1) + 1):
            for y in range(max(cy - 1, 0), min(cy + 1, dims[1] - 1) + 1):
                r = (z * dims[1] + y) * dims[0]
                b, e = start[r + max(cx - 1, 0)], start[r + min(cx + 1, dims[0] - 1) + 1]
                idx.append(np.arange(b, e))
        idx = np.concatenate(idx)
        n = f(len(idx))
        if len(idx) == 0:
            continue
        q = pts[idx]
        dd = []
        for a, cc in enumerate((cx, cy, cz)):
            lo = gmin[a] + (f(cc) + f(0.25) * ib) * cell - slack
            hi = gmin[a] + (f(cc) + f(0.25) * (ib + f(1))) * cell + slack
            d = np.maximum(np.maximum(lo[None, :] - q[:, a:a + 1], q[:, a:a + 1] - hi[None, :]), f(0))
            dd.append((d * d).astype(f))
        # box b = ix + 4 iy + 16 iz
        d2 = ((dd[0][:, None, None, :] + dd[1][:, None, :, None]) + dd[2][:, :, None, None]).reshape(len(idx), 64)
        w = np.where(d2 < h2, w_in(np.minimum(d2, h2), h, hinv, sig), f(0)).astype(f)
        acc = w.sum(axis=0, dtype=f)
        up = acc * (f(1) + f(16) * EPS) * (f(1) + f(4) * n * EPS) + f(32) * n * EPS * sig
        out[c] = np.where(acc == 0, f(0), up)
        if np.all(acc >= f(thr)):
            out[c] = np.inf
    return out, dims, gmin, g


def box_of(pts, dims, gmin, g):
    """The bound box a sample falls in, as the march locates it (locate + box_bound)."""
    f = np.float32
    fl = np.floor((pts - gmin[None, :]) * f(g.inv)).astype(f)
    u = ((pts - gmin[None, :]) * f(g.inv)).astype(f) - fl
    c = fl.astype(np.int64)
    inside = np.all((c >= 0) & (c < np.array(dims)[None, :]), axis=1)
    bi = np.minimum((f(4) * u).astype(np.int64), 3)
    cell = c[:, 0] + c[:, 1] * dims[0] + c[:, 2] * dims[0] * dims[1]
    return inside, cell, bi[:, 0] + 4 * bi[:, 1] + 16 * bi[:, 2]


@pytest.mark.parametrize("seed,n", [(3, 3000), (4, 6000)])
def test_bound_covers_every_sample(seed, n):
    sc = scenes.small_scene(seed=seed, n=n)
    fr = O.build_frame(sc.xyz, sc.support)
    table, dims, gmin, g = bound_table(fr, sc.iso)
    rng = np.random.default_rng(seed)
    f = np.float32
    cell = f(g.cell)
    # samples: uniform inside random boxes of non-empty neighbourhoods, box corners, particles
    live = np.nonzero(np.any(table != 0, axis=1))[0]
    cs = rng.choice(live, 4000)
    bs = rng.integers(0, 64, 4000)
    cc = np.stack([cs % dims[0], (cs // dims[0]) % dims[1], cs // (dims[0] * dims[1])], 1).astype(f)
    bb = np.stack([bs & 3, (bs >> 2) & 3, bs >> 4], 1).astype(f)
    base = gmin[None, :] + (cc + f(0.25) * bb) * cell
    samples = [base + rng.random((4000, 3)).astype(f) * f(0.25) * cell,
               base + rng.integers(0, 2, (4000, 3)).astype(f) * f(0.25) * cell,
               sc.xyz[rng.choice(sc.n, 2000)].astype(f)]
    pts = np.concatenate(samples).astype(f)
    inside, cix, bix = box_of(pts, dims, gmin, g)
    pts, cix, bix = pts[inside], cix[inside], bix[inside]
    rho = O.density(fr, pts, 32)
    bound = table[cix, bix].astype(np.float64)
    assert np.all(rho <= bound), (rho - bound).max()
    # the bound is a useful one: many samples are skippable, and finite bounds are not far off
    assert np.mean(bound < sc.iso) > 0.1
    fin = np.isfinite(bound) & (rho > 0)
    assert np.median(bound[fin] / rho[fin]) < 8.0


def test_reached_cells_are_never_skipped():
    """+inf is stored only for cells whose 64 sums all reach the iso density; each of those boxes'
    finite bound would be at least the iso density too, so the skip decisions do not change."""
    sc = scenes.small_scene(seed=5, n=5000)
    fr = O.build_frame(sc.xyz, sc.support)
    full, _, _, _ = bound_table(fr, np.inf)
    stop, _, _, _ = bound_table(fr, sc.iso)
    reached = np.isinf(stop).all(axis=1)
    assert reached.any() and (~reached).any()
    assert np.all(full[reached] >= sc.iso)
    assert np.array_equal(stop[~reached], full[~reached])
    assert np.array_equal(full < sc.iso, stop < sc.iso)


def test_bound_holds_at_the_nearest_point_of_each_box():
    """The tight case: a sample at a box's point nearest to a lone particle (and a few ulps around
    it) has the density the bound takes for that particle, up to rounding; the slack and the margin
    must keep the bound above it."""
    f = np.float32
    rng = np.random.default_rng(9)
    xyz = rng.uniform(0.2, 0.8, (6, 3)).astype(f)
    support = 0.05
    fr = O.build_frame(xyz, support)
    table, dims, gmin, g = bound_table(fr, np.inf)
    cell = f(g.cell)
    pts = []
    for c in range(table.shape[0]):
        if not np.any(table[c] > 0):
            continue
        cc = np.array([c % dims[0], (c // dims[0]) % dims[1], c // (dims[0] * dims[1])], f)
        for b in range(64):
            bb = np.array([b & 3, (b >> 2) & 3, b >> 4], f)
            lo = gmin + (cc + f(0.25) * bb) * cell
            hi = gmin + (cc + f(0.25) * (bb + f(1))) * cell
            for p in xyz:
                q = np.minimum(np.maximum(p, lo), hi).astype(f)
                for k in (-2, 0, 2):
                    pts.append(np.nextafter(q, q + f(k)) if k else q)
    pts = np.array(pts, f)
    inside, cix, bix = box_of(pts, dims, gmin, g)
    pts, cix, bix = pts[inside], cix[inside], bix[inside]
    rho = O.density(fr, pts, 32)
    bound = table[cix, bix].astype(np.float64)
    assert np.all(rho <= bound), (rho - bound).max()
    tight = rho > 0
    assert tight.sum() > 1000 and (rho[tight] / bound[tight]).max() > 0.99
