"""The C++ host interface (include/fluidmarch.hpp): a C++ program drives the
marcher through RayMarcher::Prepare / Start / IsDone / Exit like the
reference's renderer, and its outputs equal the oracle's bit for bit."""

import os
import subprocess

import numpy as np
import pytest

import oracle as O
from fluidmarch import scenes

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_raymarcher_adapter(fmlib, tmp_path):
    exe = tmp_path / "adapter"
    libdir = os.path.dirname(fmlib.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "raymarcher_adapter.cpp"), "-L", libdir, "-lfluidmarch",
                    "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    sc = scenes.small_scene(seed=41, n=5000, width=72, height=54, max_steps=200)
    cam = sc.cameras[0]
    depth = O.splat(sc.xyz, sc.support, cam)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([sc.n, cam.width, cam.height, sc.max_steps], np.int32).tofile(f)
        np.array([sc.support, sc.step, sc.iso], np.float32).tofile(f)
        for m in (cam.view, cam.proj, cam.inv_proj_view, cam.position):
            np.asarray(m, np.float32).tofile(f)
        sc.xyz.astype(np.float32).tofile(f)
        depth.astype(np.float32).tofile(f)
    out = tmp_path / "out.bin"
    subprocess.run([str(exe), str(inp), str(out)], check=True)
    res = np.fromfile(out, np.float32).reshape(2, cam.n_pixels, 4)
    fr = O.build_frame(sc.xyz, sc.support)
    o = O.march(fr, cam, sc.iso, sc.step, sc.max_steps, 0, depth, threads=0)
    assert np.array_equal(res[0].view(np.uint32), o["position"].view(np.uint32))
    assert np.array_equal(res[1].view(np.uint32), o["normal"].view(np.uint32))
    assert (res[0][:, 3] == 1).sum() > 100
