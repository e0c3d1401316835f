"""The exact skip's density bound, restated on the CPU and checked against the oracle's density.

The skip steps over a sample when the bound of its bound box is below the iso density, so it is
exact only if no sample located in a box has a density above the box's bound.  This restates the
bound tables of grid_build.cu in numpy FP32: per box, W at each 27-neighbourhood particle's distance
to the box grown by the slack, summed (numpy's pairwise order, not the kernel's: the margin is meant
to cover any order) and inflated by the same margin.  The first level (k_cell_bound4) has 4x4x4
boxes per cell and stores +inf for a cell whose 64 sums all reach the iso density; the table the
march reads (k_cell_refine8) has 8x8x8 boxes, each inheriting its 4x4x4 box's bound except under the
"shell" boxes (iso <= bound < +inf), whose eighths get their own sums.  Random samples (uniform in
boxes, at box corners and at the particles themselves), located as the march locates them, must
have an FP32 oracle density no larger than their box's bound.
"""

import numpy as np
import pytest

import oracle as O
from fluidmarch import scenes

EPS = np.float32(5.9604645e-8)  # 2^-24
_I8 = np.arange(512)
PARENT8 = ((_I8 & 7) >> 1) + 4 * (((_I8 >> 3) & 7) >> 1) + 16 * ((_I8 >> 6) >> 1)  # 4x4x4 box of each 8x8x8 box


def w_in(q2, h, hinv, sig):
    """CubicSplineKernel::W for q2 < h^2, FP32 as the kernels evaluate it (Kernel.cpp:16-32)."""
    f = np.float32
    q = np.sqrt(q2.astype(f)).astype(f) * f(hinv)
    qm = f(1) - q
    a = f(sig) * (((f(2) * qm) * qm) * qm)
    b = f(sig) * (f(6) * (((q * q) * q) - (q * q)) + f(1))
    return np.where(q >= f(0.5), a, b).astype(f)


def bound_table(fr, thr, div=4):
    """Bounds of div x div x div boxes per cell (box b = ix + div iy + div^2 iz); with div 4 and a finite
    thr, +inf for cells whose sums all reach thr (k_cell_bound4)."""
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
    nb = div ** 3
    out = np.zeros((ncells, nb), f)
    ib = np.arange(div, dtype=f)
    frac = f(1.0 / div)
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
            lo = gmin[a] + (f(cc) + frac * ib) * cell - slack
            hi = gmin[a] + (f(cc) + frac * (ib + f(1))) * cell + slack
            d = np.maximum(np.maximum(lo[None, :] - q[:, a:a + 1], q[:, a:a + 1] - hi[None, :]), f(0))
            dd.append((d * d).astype(f))
        d2 = ((dd[0][:, None, None, :] + dd[1][:, None, :, None]) + dd[2][:, :, None, None]).reshape(len(idx), nb)
        w = np.where(d2 < h2, w_in(np.minimum(d2, h2), h, hinv, sig), f(0)).astype(f)
        acc = w.sum(axis=0, dtype=f)
        up = acc * (f(1) + f(16) * EPS) * (f(1) + f(4) * n * EPS) + f(32) * n * EPS * sig
        out[c] = np.where(acc == 0, f(0), up)
        if div == 4 and np.all(acc >= f(thr)):
            out[c] = np.inf
    return out, dims, gmin, g


def march_table(fr, thr):
    """The 8x8x8 table the march reads: the 4x4x4 table at thr, refined under its shell boxes."""
    coarse, dims, gmin, g = bound_table(fr, thr, 4)
    full8, _, _, _ = bound_table(fr, np.inf, 8)
    fine = coarse[:, PARENT8]
    shell = (fine >= np.float32(thr)) & np.isfinite(fine)
    fine = np.where(shell, full8, fine).astype(np.float32)
    return fine, coarse, dims, gmin, g


def box_of(pts, dims, gmin, g, div=8):
    """The bound box a sample falls in, as the march locates it (locate + box_bound)."""
    f = np.float32
    fl = np.floor((pts - gmin[None, :]) * f(g.inv)).astype(f)
    u = ((pts - gmin[None, :]) * f(g.inv)).astype(f) - fl
    c = fl.astype(np.int64)
    inside = np.all((c >= 0) & (c < np.array(dims)[None, :]), axis=1)
    bi = np.minimum((f(div) * u).astype(np.int64), div - 1)
    cell = c[:, 0] + c[:, 1] * dims[0] + c[:, 2] * dims[0] * dims[1]
    return inside, cell, bi[:, 0] + div * bi[:, 1] + div * div * bi[:, 2]


@pytest.mark.parametrize("seed,n", [(3, 3000), (4, 6000)])
def test_bound_covers_every_sample(seed, n):
    sc = scenes.small_scene(seed=seed, n=n)
    fr = O.build_frame(sc.xyz, sc.support)
    table, coarse, dims, gmin, g = march_table(fr, sc.iso)
    rng = np.random.default_rng(seed)
    f = np.float32
    cell = f(g.cell)
    # samples: uniform inside random boxes of non-empty neighbourhoods (half of them under shell
    # boxes, where the table holds refined sums), box corners, particles
    live = np.nonzero(np.any(table != 0, axis=1))[0]
    shell_c, shell_b = np.nonzero((table >= f(sc.iso)) & np.isfinite(table) & (table != coarse[:, PARENT8]))
    assert shell_c.size > 100
    pick = rng.integers(0, shell_c.size, 2000)
    cs = np.concatenate([rng.choice(live, 2000), shell_c[pick]])
    bs = np.concatenate([rng.integers(0, 512, 2000), shell_b[pick]])
    cc = np.stack([cs % dims[0], (cs // dims[0]) % dims[1], cs // (dims[0] * dims[1])], 1).astype(f)
    bb = np.stack([bs & 7, (bs >> 3) & 7, bs >> 6], 1).astype(f)
    base = gmin[None, :] + (cc + f(0.125) * bb) * cell
    samples = [base + rng.random((4000, 3)).astype(f) * f(0.125) * cell,
               base + rng.integers(0, 2, (4000, 3)).astype(f) * f(0.125) * cell,
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
    # the refined table skips a sub-box only where its own full sum is below iso, and never where
    # its 4x4x4 box would not have been skipped less: it is at least as tight and no less exact
    fine, coarse, _, _, _ = march_table(fr, sc.iso)
    full8, _, _, _ = bound_table(fr, np.inf, 8)
    assert np.all((fine < sc.iso) <= (full8 < sc.iso))
    assert np.all((coarse[:, PARENT8] < sc.iso) <= (fine < sc.iso))
    assert np.sum(fine < sc.iso) > np.sum(coarse[:, PARENT8] < sc.iso)


def test_bound_holds_at_the_nearest_point_of_each_box():
    """The tight case: a sample at a box's point nearest to a lone particle (and a few ulps around
    it) has the density the bound takes for that particle, up to rounding; the slack and the margin
    must keep the bound above it."""
    f = np.float32
    rng = np.random.default_rng(9)
    xyz = rng.uniform(0.2, 0.8, (6, 3)).astype(f)
    support = 0.05
    fr = O.build_frame(xyz, support)
    table, dims, gmin, g = bound_table(fr, np.inf, 8)
    cell = f(g.cell)
    pts = []
    for c in range(table.shape[0]):
        if not np.any(table[c] > 0):
            continue
        cc = np.array([c % dims[0], (c // dims[0]) % dims[1], c // (dims[0] * dims[1])], f)
        for b in np.nonzero(table[c] > 0)[0]:
            bb = np.array([b & 7, (b >> 3) & 7, b >> 6], f)
            lo = gmin + (cc + f(0.125) * bb) * cell
            hi = gmin + (cc + f(0.125) * (bb + f(1))) * cell
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
