"""Write the golden vectors in this directory from the reference's own marcher.

Runs the reference translation units (RayMarcher.cpp, Kernel.cpp,
ThreadPool.cpp, Dataset.cpp, compiled unmodified by oracle/Makefile into
oracle/_ref/libfmref.so) on small seeded scenes and stores inputs and outputs:

    xyz, support, iso, step, max_steps, camera matrices, start depth (the
    splat depth the reference consumes), box_mode, and the reference's
    positions and normals (vec4 per pixel).

Needs the reference tree (oracle/_ref is built only where it exists).  The
fixtures are committed; the tests only read them.

    python tests/golden/make_golden.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "bachelor-thesis_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
from fluidmarch import scenes  # noqa: E402


def small_dam(seed=11, width=64, height=48):
    """16^3 jittered lattice at the dam-break spacing (0.025) and H = 0.1."""
    rng = np.random.default_rng(seed)
    s = 0.025
    i = np.arange(16, dtype=np.float64) * s
    x, y, z = np.meshgrid(i, i, i, indexing="ij")
    base = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    xyz = (base + rng.uniform(-0.1 * s, 0.1 * s, size=base.shape)).astype(np.float32)
    H = np.float32(0.1)
    iso = np.float32(0.5 * scenes.lattice_rest_density(s, float(H)))
    cam = scenes.make_camera((0.9, 0.6, 0.9), (0.2, 0.15, 0.2), width, height)
    return xyz, float(H), float(iso), float(np.float32(0.0125)), 256, cam


def small_slosh(seed=12, width=64, height=48):
    sc = scenes.small_scene(seed=seed, n=3000, width=width, height=height, max_steps=192)
    return sc.xyz, sc.support, sc.iso, sc.step, sc.max_steps, sc.cameras[0]


def write(name, xyz, H, iso, step, max_steps, cam, box_mode):
    depth = oracle.splat(xyz, H, cam)
    r = oracle.ref_march(xyz, H, cam, depth, max_steps, step, iso, box_mode=box_mode)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, xyz=xyz, support=np.float32(H), iso=np.float32(iso), step=np.float32(step),
                        max_steps=np.int32(max_steps), view=cam.view, proj=cam.proj, inv_proj_view=cam.inv_proj_view,
                        cam_pos=cam.position, width=np.int32(cam.width), height=np.int32(cam.height),
                        start_depth=depth, box_mode=np.int32(box_mode), ref_position=r["position"],
                        ref_normal=r["normal"], ref_sorted=r["sorted"], ref_grid=r["grid"])
    hits = int((r["position"][:, 3] == 1).sum())
    print(f"{path}: {xyz.shape[0]} particles, {cam.width}x{cam.height}, box_mode {box_mode}, {hits} hits")


def main():
    oracle.build_oracle(ref=True)
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/libfmref.so was not built (reference tree absent)")
    write("dam16_skipoff", *small_dam(), box_mode=0)
    write("dam16_refskip", *small_dam(), box_mode=1)
    write("slosh3k_skipoff", *small_slosh(), box_mode=0)
    write("slosh3k_refskip", *small_slosh(), box_mode=1)


if __name__ == "__main__":
    main()
