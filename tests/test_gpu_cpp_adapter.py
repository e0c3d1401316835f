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


def test_cpp_dataset_autoplay(fmlib, ctx, tmp_path):
    """fluidmarch::Dataset loads a BGEO series at construction (Frames, MaxParticles, Loaded) and a
    RayMarcher plays it frame by frame; every frame equals the oracle's march of its particles."""
    from fluidmarch import bgeo

    exe = tmp_path / "dataset"
    libdir = os.path.dirname(fmlib.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "dataset_adapter.cpp"), "-L", libdir, "-lfluidmarch",
                    "-Wl,-rpath," + libdir, "-o", str(exe)], check=True)
    base = scenes.small_scene(seed=51, n=5000, width=64, height=48, max_steps=200)
    cam = base.cameras[0]
    prefix = str(tmp_path / "ParticleData_Fluid_")
    frames = []
    for i, n in enumerate((5000, 3500, 6500), start=1):
        sc = scenes.small_scene(seed=60 + i, n=n, width=64, height=48, max_steps=200)
        frames.append(sc.xyz)
        bgeo.write(f"{prefix}{i}.bgeo", sc.xyz, compressed=i != 2)
    depth = O.splat(frames[0], base.support, cam)
    inp = tmp_path / "cam.bin"
    with open(inp, "wb") as f:
        np.array([cam.width, cam.height, base.max_steps], np.int32).tofile(f)
        np.array([base.support, base.step, base.iso], np.float32).tofile(f)
        for m in (cam.view, cam.proj, cam.inv_proj_view, cam.position):
            np.asarray(m, np.float32).tofile(f)
        depth.astype(np.float32).tofile(f)
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), prefix, str(inp), str(out), "cube"], check=True, capture_output=True, text=True)
    assert r.stdout.split() == ["cube", "1001", "1001", "1"]
    data = open(out, "rb").read()
    nf = int(np.frombuffer(data[:4], np.int32)[0])
    maxp = int(np.frombuffer(data[4:12], np.int64)[0])
    assert nf == 3 and maxp == 6500
    pos = np.frombuffer(data[12:], np.float32).reshape(nf, cam.n_pixels, 4)
    hits = 0
    for i in range(nf):
        fr = O.build_frame(frames[i], base.support)
        o = O.march(fr, cam, base.iso, base.step, base.max_steps, 0, depth, threads=0)
        assert np.array_equal(pos[i].view(np.uint32), o["position"].view(np.uint32)), i
        hits += int((pos[i][:, 3] == 1).sum())
    assert hits > 100
