"""fm_grid_build_noalloc: the grid build for callers that cannot allocate.

Some callers must not call cudaMalloc (a renderer that reserves its memory up
front, a plugin inside a host application's memory budget).  For them the
library has one entry point that allocates nothing: the caller passes the
input and every output buffer, and the build's scratch lives in a fixed device
array inside the library.  These tests call it through the C ABI several times
in a row (each call finds the previous call's leftovers in the shared scratch)
and check that its output equals, bit for bit, what the regular entry point
(fm_scene_create) builds for the same particles, for sort keys of three, two
and one radix pass.  The file is named so that pytest collects it last.
"""

import ctypes

import numpy as np
import pytest

from fluidmarch import scenes

pytestmark = pytest.mark.gpu


def _build_noalloc(fmlib, torch, xyz_np, support, capacity=None):
    L = fmlib.load()
    n = xyz_np.shape[0]
    xyz = torch.from_numpy(xyz_np).cuda()
    sorted_xyzw = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    cell = torch.zeros(n, dtype=torch.int32, device="cuda")
    perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    if capacity is None:
        capacity = 8 * 400_000 + 1
    sub = torch.zeros(capacity, dtype=torch.int32, device="cuda")
    info = fmlib.CGridInfo()
    torch.cuda.synchronize()
    rc = L.fm_grid_build_noalloc(xyz.data_ptr(), n, 3, float(support), sorted_xyzw.data_ptr(), cell.data_ptr(),
                                 perm.data_ptr(), sub.data_ptr(), capacity, ctypes.byref(info), None)
    torch.cuda.synchronize()
    return rc, info, sorted_xyzw, cell, perm, sub


def _cases():
    """(xyz, support): sort keys of three 8-bit radix passes (a 300k-particle sloshing frame on the 1M
    frame's grid, 8 * n_cells > 2^16), two (a 120k-particle frame with its scaled support radius, and a
    small scene) and one (a cluster inside 3x3x3 cells)."""
    out = []
    sc = scenes.sloshing(seed=101, n=300_000, h=0.02, width=8, height=8)
    out.append((sc.xyz, sc.support))
    sc = scenes.sloshing(seed=102, n=120_000, h=0.02 * (1_000_000 / 120_000) ** (1 / 3), width=8, height=8)
    out.append((sc.xyz, sc.support))
    sc = scenes.small_scene(seed=104, n=30_000)
    out.append((sc.xyz, sc.support))
    rng = np.random.default_rng(105)
    out.append((rng.uniform(0.0, 0.09, (5000, 3)).astype(np.float32), 0.1))
    return out


def test_noalloc_grid_build_matches_scene_create(fmlib, ctx):
    torch = pytest.importorskip("torch")
    # calls in a row, different sizes: each sees the previous one's scratch contents
    passes = set()
    for xyz, support in _cases():
        sc = scenes.Scene("noalloc", xyz, support, 1.0, 0.01, 8, 0)
        rc, info, srt, cell, perm, sub = _build_noalloc(fmlib, torch, sc.xyz, sc.support)
        assert rc == fmlib.FM_OK
        passes.add((max(1, (8 * int(info.n_cells) - 1).bit_length()) + 7) // 8)
        ref = fmlib.Scene(ctx, sc.xyz, sc.support)
        g = ref.grid()
        d = ref.download()
        ref.close()
        assert tuple(info.dims) == g["dims"] and int(info.n_cells) == g["n_cells"]
        assert np.array_equal(np.array(info.min[:], np.float32).view(np.uint32), g["min"].view(np.uint32))
        assert np.array_equal(cell.cpu().numpy().view(np.uint32), d["cell"])
        assert np.array_equal(perm.cpu().numpy().view(np.uint32), d["perm"])
        assert np.array_equal(srt.cpu().numpy().view(np.uint32), d["sorted"].view(np.uint32))
        starts = sub.cpu().numpy().view(np.uint32)[: 8 * g["n_cells"] + 1 : 8]
        assert np.array_equal(starts, d["start"])
    assert passes == {1, 2, 3}


def test_noalloc_rejects_sizes_beyond_its_limits(fmlib, ctx):
    torch = pytest.importorskip("torch")
    sc = scenes.small_scene(seed=103, n=20_000)
    # a sub-cell table that is too small: rejected, with the needed size reported
    rc, info, *_ = _build_noalloc(fmlib, torch, sc.xyz, sc.support, capacity=16)
    assert rc == fmlib.FM_ERR_INVALID and int(info.n_cells) > 2
    # more particles than the scratch array is sized for
    big = np.zeros(((1 << 21) + 1, 3), np.float32)
    rc, *_ = _build_noalloc(fmlib, torch, big, 0.1, capacity=9)
    assert rc == fmlib.FM_ERR_INVALID
    # more cells than it is sized for: a unit cube at a support radius of 0.005 (~8 M cells)
    rng = np.random.default_rng(106)
    spread = rng.uniform(0.0, 1.0, (1000, 3)).astype(np.float32)
    rc, info, *_ = _build_noalloc(fmlib, torch, spread, 0.005, capacity=9)
    assert rc == fmlib.FM_ERR_INVALID and int(info.n_cells) > (1 << 21)


def test_noalloc_rejects_host_pointers(fmlib, ctx):
    """Buffers the GPU cannot use as device memory are refused before any launch."""
    torch = pytest.importorskip("torch")
    L = fmlib.load()
    sc = scenes.small_scene(seed=107, n=2000)
    n = sc.n
    xyz = torch.from_numpy(sc.xyz).cuda()
    srt = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    cell = torch.zeros(n, dtype=torch.int32, device="cuda")
    perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    host_sub = np.zeros(8 * 400_000 + 1, np.uint32)
    info = fmlib.CGridInfo()
    torch.cuda.synchronize()
    rc = L.fm_grid_build_noalloc(xyz.data_ptr(), n, 3, float(sc.support), srt.data_ptr(), cell.data_ptr(),
                                 perm.data_ptr(), host_sub.ctypes.data, host_sub.size, ctypes.byref(info), None)
    assert rc == fmlib.FM_ERR_INVALID
    rc = L.fm_grid_build_noalloc(sc.xyz.ctypes.data, n, 3, float(sc.support), srt.data_ptr(), cell.data_ptr(),
                                 perm.data_ptr(), host_sub.ctypes.data, host_sub.size, ctypes.byref(info), None)
    assert rc == fmlib.FM_ERR_INVALID
