"""GPU grid build: bit-exact against the oracle (cells, stable order, cell table)."""

import numpy as np
import pytest

import oracle as O
from fluidmarch import scenes

pytestmark = pytest.mark.gpu


def check_grid(fm, ctx, xyz, H, stride=3):
    fr = O.build_frame(xyz, H)
    data = xyz if stride == 3 else np.ascontiguousarray(np.concatenate([xyz, np.ones((xyz.shape[0], stride - 3), np.float32)], 1))
    sc = fm.Scene(ctx, data, H, stride=stride)
    g = sc.grid()
    assert g["dims"] == fr.dims
    assert np.array_equal(g["min"].view(np.uint32), np.array(fr.grid.min[:], np.float32).view(np.uint32))
    assert np.array_equal(g["max"].view(np.uint32), np.array(fr.grid.max[:], np.float32).view(np.uint32))
    d = sc.download()
    assert np.array_equal(d["cell"], fr.cells)
    assert np.array_equal(d["perm"], fr.perm)
    assert np.array_equal(d["start"], fr.start)
    assert np.array_equal(d["sorted"].view(np.uint32), fr.sorted.view(np.uint32))
    sc.close()
    return g


@pytest.mark.parametrize("n", [1, 2, 31, 2049, 5000])
def test_grid_small(fmlib, ctx, n):
    sc = scenes.small_scene(seed=n, n=max(n, 200))
    check_grid(fmlib, ctx, np.ascontiguousarray(sc.xyz[:n]), sc.support)


def test_grid_dam_break(fmlib, ctx):
    sc = scenes.dam_break()
    check_grid(fmlib, ctx, sc.xyz, sc.support)


def test_grid_sloshing_1m(fmlib, ctx):
    """The 1M-particle sloshing frame: every cell index and the sort order bit-exact."""
    sc = scenes.sloshing()
    g = check_grid(fmlib, ctx, sc.xyz, sc.support)
    assert g["n_particles"] == 1_000_000


def test_grid_stride4_negative_coordinates(fmlib, ctx):
    rng = np.random.default_rng(1)
    xyz = rng.uniform(-3.0, -1.0, size=(10000, 3)).astype(np.float32)
    check_grid(fmlib, ctx, xyz, 0.13, stride=4)


def test_grid_all_in_one_cell_and_duplicates(fmlib, ctx):
    rng = np.random.default_rng(2)
    xyz = np.repeat(rng.uniform(0.0, 0.01, size=(100, 3)).astype(np.float32), 50, axis=0)
    check_grid(fmlib, ctx, xyz, 0.5)


def test_grid_many_cells(fmlib, ctx):
    """More than 2^16 cells (636k), sparse: most sub-cells hold 0 or 1 particle."""
    rng = np.random.default_rng(3)
    xyz = rng.uniform(0.0, 1.0, size=(300000, 3)).astype(np.float32)
    g = check_grid(fmlib, ctx, xyz, 0.012)
    assert g["n_cells"] > (1 << 16)


def test_grid_over_a_million_cells(fmlib, ctx):
    """1.4M cells: 11.5M sub-cell keys, more scan tiles than one add pass sums directly (the scan
    takes its recursive path)."""
    rng = np.random.default_rng(13)
    xyz = rng.uniform(0.0, 1.0, size=(200000, 3)).astype(np.float32)
    g = check_grid(fmlib, ctx, xyz, 0.009)
    assert 8 * g["n_cells"] + 1 > 2048 * 4096


def test_grid_segment_lengths(fmlib, ctx):
    """Sub-cells holding 1 .. 64 particles (sorted by one warp), 257, 4,000 and 60,000 (sorted by a
    block, radix passes over the input indices), in scrambled input order."""
    rng = np.random.default_rng(4)
    parts = [rng.uniform(0.0, 2.0, (20000, 3))]
    for m in (33, 64, 257, 4000):
        parts.append(rng.uniform(0.0, 2.0, 3) + rng.uniform(0.0, 0.01, (m, 3)))
    parts.append(np.repeat(rng.uniform(0.0, 2.0, (1, 3)), 60000, axis=0))
    xyz = np.concatenate(parts).astype(np.float32)
    rng.shuffle(xyz)
    fr = O.build_frame(xyz, 0.1)
    seg = np.diff(fr.sub_start)
    assert seg.max() >= 60000 and np.sum((seg > 64) & (seg < 60000)) >= 2 and np.sum((seg > 32) & (seg <= 64)) >= 2
    check_grid(fmlib, ctx, xyz, 0.1)


def test_scene_update_rebuilds(fmlib, ctx):
    a = scenes.small_scene(seed=1, n=4000)
    b = scenes.small_scene(seed=2, n=3500)
    sc = fmlib.Scene(ctx, a.xyz, a.support)
    sc.update(b.xyz)
    fr = O.build_frame(b.xyz, a.support)
    d = sc.download()
    assert np.array_equal(d["perm"], fr.perm) and np.array_equal(d["start"], fr.start)


def _check_scene(sc, xyz, H):
    fr = O.build_frame(xyz, H)
    g = sc.grid()
    assert g["dims"] == fr.dims and g["n_cells"] == int(np.prod(fr.dims))
    assert np.array_equal(g["min"].view(np.uint32), np.array(fr.grid.min[:], np.float32).view(np.uint32))
    assert np.array_equal(g["max"].view(np.uint32), np.array(fr.grid.max[:], np.float32).view(np.uint32))
    d = sc.download()
    assert np.array_equal(d["cell"], fr.cells)
    assert np.array_equal(d["perm"], fr.perm)
    assert np.array_equal(d["start"], fr.start)
    assert np.array_equal(d["sorted"].view(np.uint32), fr.sorted.view(np.uint32))


def test_scene_update_grow_shrink_and_failed_update(fmlib, ctx):
    """One scene through updates whose grids need more cells than its tables hold (the build grows
    them and runs again), fewer cells (the larger tables are reused), a rejected update (an infinite
    coordinate) and valid updates after it, plus a second scene of the same context in between:
    every build bit-exact to the oracle."""
    rng = np.random.default_rng(11)
    H = 0.05
    small = rng.uniform(0.0, 0.5, (30000, 3)).astype(np.float32)  # the scene's particle capacity
    big = rng.uniform(-0.5, 1.5, (30000, 3)).astype(np.float32)
    mid = rng.uniform(0.2, 1.0, (25000, 3)).astype(np.float32)
    sc = fmlib.Scene(ctx, small, H)
    _check_scene(sc, small, H)
    sc.update(big)  # more cells than the first build allocated
    _check_scene(sc, big, H)
    sc.update(mid)  # fewer cells
    _check_scene(sc, mid, H)
    bad = mid.copy()
    bad[123, 2] = np.inf
    with pytest.raises(fmlib.FmError) as e:
        sc.update(bad)
    assert e.value.code == fmlib.FM_ERR_INVALID
    other = fmlib.Scene(ctx, big[:7000], 0.02)  # another scene on the same scratch
    _check_scene(other, big[:7000], 0.02)
    other.close()
    sc.update(small)
    _check_scene(sc, small, H)
    sc.update(big[:29999])  # 3n not a multiple of 4: the float4 pass's tail
    _check_scene(sc, big[:29999], H)
    sc.close()


def test_scene_update_unaligned_device_positions(fmlib, ctx):
    """Device positions at an address that is not 16-byte aligned (one-float offset) take the
    scalar bounds pass; the same positions aligned take the float4 pass; both bit-exact."""
    torch = pytest.importorskip("torch")
    sc0 = scenes.small_scene(seed=12, n=9000)
    xyz = np.ascontiguousarray(sc0.xyz)
    n = xyz.shape[0]
    flat = torch.zeros(3 * n + 4, dtype=torch.float32, device="cuda")
    flat[1:1 + 3 * n] = torch.from_numpy(xyz.reshape(-1)).cuda()
    off = flat[1:1 + 3 * n].view(n, 3)
    assert off.data_ptr() % 16 == 4
    s = fmlib.Scene(ctx, off, sc0.support)
    _check_scene(s, xyz, sc0.support)
    al = torch.from_numpy(xyz).cuda()
    s.update(al)
    _check_scene(s, xyz, sc0.support)
    s.update(off)
    _check_scene(s, xyz, sc0.support)
    s.close()


def test_scene_from_device_memory(fmlib, ctx):
    torch = pytest.importorskip("torch")
    sc = scenes.small_scene(seed=6, n=6000)
    t = torch.from_numpy(sc.xyz).cuda()
    s = fmlib.Scene(ctx, t, sc.support)
    fr = O.build_frame(sc.xyz, sc.support)
    assert np.array_equal(s.download()["perm"], fr.perm)


def test_scene_upload_entry(fmlib, ctx):
    """fm_scene_upload (host positions) builds the same grid as fm_scene_create."""
    import ctypes as C

    sc = scenes.small_scene(seed=7, n=5000)
    h = C.c_void_p()
    xyz = np.ascontiguousarray(sc.xyz)
    assert ctx.L.fm_scene_upload(ctx.h, xyz.ctypes.data, xyz.shape[0], 3, sc.support, C.byref(h)) == fmlib.FM_OK
    s = fmlib.Scene.wrap(ctx, h, sc.support)
    fr = O.build_frame(sc.xyz, sc.support)
    d = s.download()
    assert np.array_equal(d["perm"], fr.perm) and np.array_equal(d["start"], fr.start)
    assert ctx.L.fm_scene_upload(ctx.h, xyz.ctypes.data, xyz.shape[0], -3, sc.support, C.byref(h)) != fmlib.FM_OK
    s.close()


def test_rejects_bad_input(fmlib, ctx):
    xyz = np.zeros((10, 3), np.float32)
    xyz[3, 1] = np.nan
    with pytest.raises(fmlib.FmError) as e:
        fmlib.Scene(ctx, xyz, 0.1)
    assert e.value.code == fmlib.FM_ERR_INVALID
    with pytest.raises(fmlib.FmError):
        fmlib.Scene(ctx, np.zeros((0, 3), np.float32), 0.1)
    with pytest.raises(fmlib.FmError):
        fmlib.Scene(ctx, np.zeros((4, 3), np.float32), -1.0)
    xyz = np.array([[0, 0, 0], [1e6, 1e6, 1e6]], np.float32)
    with pytest.raises(fmlib.FmError):  # 2^28 cell cap
        fmlib.Scene(ctx, xyz, 1e-3)
