"""The C-ABI library builds for sm_103a, loads, and exports every entry point
that include/fluidmarch.h declares.  No compute calls: this runs without a GPU."""

import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from fluidmarch import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fluidmarch.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(fm_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("fm_create", "fm_destroy", "fm_scene_create", "fm_march", "fm_splat_depth", "fm_sync"):
        assert must in names


def test_library_exports_every_declared_symbol(fmlib):
    path = fmlib.LIB_PATH
    lib = ctypes.CDLL(path)
    for name in declared_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    for name in declared_functions():
        assert re.search(rf"\bT {name}\b", out), name
    assert set(fmlib.EXPORTS) == set(declared_functions())


def test_library_is_built_for_sm103a(fmlib):
    out = subprocess.run(["cuobjdump", "--list-elf", fmlib.LIB_PATH], capture_output=True, text=True).stdout
    assert "sm_103a" in out


def test_version(fmlib):
    assert fmlib.load().fm_version() >= 10000


def test_invalid_arguments_without_device(fmlib):
    """Argument checks come before any device work."""
    L = fmlib.load()
    assert L.fm_create(None, 0) == fmlib.FM_ERR_INVALID
    assert L.fm_scene_create(None, None, 0, 3, 0.1, 0, None) == fmlib.FM_ERR_INVALID
    assert L.fm_march(None, None, None, None, None, 0, None) == fmlib.FM_ERR_INVALID
    assert L.fm_last_error(None) == b"no context"
    assert L.fm_last_error_string(None) == b"no context"
    assert L.fm_scene_upload(None, None, 0, 3, 0.1, None) == fmlib.FM_ERR_INVALID
    assert L.fm_selftest_wait_timeout(None, 1) == fmlib.FM_ERR_INVALID
    assert L.fm_trainer_set_state(None, None, 0) == fmlib.FM_ERR_INVALID


def test_no_device_reports_cuda_error(fmlib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert fmlib.load().fm_create(ctypes.byref(h), 0) == fmlib.FM_ERR_CUDA


def test_scene_generators_are_seeded():
    a = scenes.sloshing(seed=3, n=20000, width=32, height=24)
    b = scenes.sloshing(seed=3, n=20000, width=32, height=24)
    assert np.array_equal(a.xyz, b.xyz)
    assert a.n == 20000
    fluid_top = 0.4 + 0.08 + 0.03
    assert (a.xyz[:, 1] > fluid_top).sum() > 0.03 * a.n  # the spray fraction
    d = scenes.dam_break()
    assert d.n == 64000 and d.support == pytest.approx(0.1)
    assert d.iso == pytest.approx(0.5 * 64005.07, rel=1e-5)
    cams = scenes.batch_scenes(n_scenes=3, scale=0.02)
    assert len(cams) == 3 and all(1 <= len(s.cameras) <= 4 for s in cams)


def test_camera_matrices_are_consistent():
    cam = scenes.make_camera((1.8, 1.2, 1.8), (0.5, 0.3, 0.5), 640, 480)
    V = cam.view.reshape(4, 4).astype(np.float64).T  # row-major
    P = cam.proj.reshape(4, 4).astype(np.float64).T
    IPV = cam.inv_proj_view.reshape(4, 4).astype(np.float64).T
    assert np.allclose(IPV @ (P @ V), np.eye(4), atol=1e-5)
    # the target projects to the image centre, in front of the camera
    t = P @ V @ np.array([0.5, 0.3, 0.5, 1.0])
    assert abs(t[0] / t[3]) < 1e-6 and abs(t[1] / t[3]) < 1e-6 and 0 < t[2] / t[3] < 1
    # y is flipped (Camera3D.cpp:9): a point above the target has negative NDC y
    u = P @ V @ np.array([0.5, 0.5, 0.5, 1.0])
    assert u[1] / u[3] < 0


def test_committed_proposal_weights():
    """The trained proposal ships with its training record (no GPU needed to read it)."""
    from fluidmarch import proposal as PR

    params, meta = PR.load()
    assert params.dtype == np.float32 and params.size == 6402
    assert np.all(np.isfinite(params))
    assert meta["train_scenes"] >= 2000 and meta["heldout_scenes"] >= 200
    assert meta["heldout"]["covered"] > 0.9
