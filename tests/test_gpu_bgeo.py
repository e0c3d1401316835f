"""Particle files into scenes on the GPU.

A scene loaded from a BGEO file (host decode, device byte-swap gather, grid
build) equals the scene built from the same positions, bit for bit; a series
played frame by frame (autoplay) renders every frame as that frame's own scene
renders it, including frames that outgrow the scene.
"""

import numpy as np
import pytest

from fluidmarch import bgeo, scenes

pytestmark = pytest.mark.gpu


def same_grid(a, b):
    da, db = a.download(), b.download()
    for k in ("cell", "perm", "start"):
        assert np.array_equal(da[k], db[k]), k
    assert np.array_equal(da["sorted"].view(np.uint32), db["sorted"].view(np.uint32))


@pytest.mark.parametrize("compressed", [True, False])
def test_scene_from_file(fmlib, ctx, tmp_path, compressed):
    sc = scenes.small_scene(seed=71, n=20000, width=96, height=64)
    rng = np.random.default_rng(2)
    path = str(tmp_path / "frame.bgeo")
    bgeo.write(path, sc.xyz, {"v": ("vector", rng.normal(size=(sc.xyz.shape[0], 3))),
                              "id": ("int", np.arange(sc.xyz.shape[0]))}, compressed=compressed)
    s_file = bgeo.load_scene(ctx, path, sc.support)
    s_mem = fmlib.Scene(ctx, sc.xyz, sc.support)
    same_grid(s_file, s_mem)
    p = fmlib.MarchParams(sc.iso, sc.step, sc.max_steps, 8, fmlib.FM_SKIP_EXACT)
    a = fmlib.render(s_file, sc.cameras[0], p)
    b = fmlib.render(s_mem, sc.cameras[0], p)
    for k in a:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k
    s_file.close()
    s_mem.close()


def test_scene_from_bad_file(fmlib, ctx, tmp_path):
    path = str(tmp_path / "bad.bgeo")
    with open(path, "wb") as f:
        f.write(b"Bgeo" + bytes(20))
    with pytest.raises(fmlib.FmError):
        bgeo.load_scene(ctx, path, 0.05)
    empty = str(tmp_path / "empty.bgeo")
    bgeo.write(empty, np.zeros((0, 3), np.float32))
    with pytest.raises(fmlib.FmError):
        bgeo.load_scene(ctx, empty, 0.05)


def test_autoplay_series(fmlib, ctx, tmp_path):
    counts = [6000, 4000, 9000, 9000, 2000]  # frame 3 outgrows the scene made from frame 1
    prefix = str(tmp_path / "ParticleData_Fluid_")
    frames = []
    for i, n in enumerate(counts, start=1):
        sc = scenes.small_scene(seed=300 + i, n=n, width=80, height=60)
        frames.append(sc)
        bgeo.write(f"{prefix}{i}.bgeo", sc.xyz, compressed=i % 2 == 0)
    support = frames[0].support
    cam = frames[0].cameras[0]
    p = fmlib.MarchParams(frames[0].iso, frames[0].step, frames[0].max_steps, 8, fmlib.FM_SKIP_EXACT)
    ds = bgeo.Dataset(prefix, ".bgeo", -1, threads=2)
    assert len(ds) == len(counts) and ds.max_particles() == max(counts)
    seen = []
    for i, out in ds.autoplay(ctx, cam, p, support):
        own = fmlib.Scene(ctx, frames[i].xyz, support)
        want = fmlib.render(own, cam, p)
        for k in out:
            assert np.array_equal(out[k].view(np.uint32), want[k].view(np.uint32)), (i, k)
        same_grid(ds.scene, own)
        own.close()
        seen.append(i)
    assert seen == list(range(len(counts)))
    ds.close()
