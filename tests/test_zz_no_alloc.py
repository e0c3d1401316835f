"""fm_grid_build_noalloc: the grid build for callers that cannot allocate.

Some callers must not call cudaMalloc (a renderer that reserves its memory up
front, a plugin inside a host application's memory budget, work recorded into
a CUDA graph).  For them the library has one entry point that allocates
nothing: the caller passes the input and every output buffer, and the build's
scratch lives in a fixed device array inside the library.  This test calls it
through the C ABI twice in a row (the second call finds the first call's
leftovers in the shared scratch) and checks that its output equals, bit for
bit, what the regular entry point (fm_scene_create) builds for the same
particles.  The file is named so that pytest collects it last.
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


def test_noalloc_grid_build_matches_scene_create(fmlib, ctx):
    torch = pytest.importorskip("torch")
    # two calls in a row, different sizes: the second sees the first one's scratch contents
    for seed, n in ((101, 300_000), (102, 120_000)):
        sc = scenes.sloshing(seed=seed, n=n, h=0.02 * (1_000_000 / n) ** (1 / 3), width=8, height=8)
        rc, info, srt, cell, perm, sub = _build_noalloc(fmlib, torch, sc.xyz, sc.support)
        assert rc == fmlib.FM_OK
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
