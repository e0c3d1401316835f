"""Seeded synthetic particle scenes and pinhole cameras.

The reference renders SPlisHSPlasH BGEO frames (src/main.cpp:40, read by
src/app/Dataset.cpp:169-227); those datasets are not available, so every scene
here is generated from a seed with numpy's PCG64 (identical on x86_64 and
aarch64).  Cameras follow the reference's conventions: glm left-handed view
(src/engine/camera/CameraController3D.cpp:70-84, GLM_FORCE_LEFT_HANDED in
src/engine/hzpch.h:22-24), perspective with depth 0..1 and the y axis flipped
by scale(1, -1, 1) (src/engine/camera/Camera3D.cpp:5-20), 60 degree vertical
field of view, near 0.1, far 1000 (AdvancedRenderer.cpp:117-121).

Matrices are float32, column-major (glm layout: m[col*4 + row]).

Configurations (the reference's smoothing length h is half the support radius;
the reference's kernel radius ``ParticleRadius`` is the support radius H = 2h):

* ``dam_break``     64,000 particles, 40^3 lattice, spacing 0.025, jitter
                    U(+-0.1 spacing), H = 0.1, 640x480, step 0.25h, 512 steps.
* ``sloshing``      1,000,000 particles: 950k below the surface
                    y = 0.4 + 0.08 sin(2 pi x) cos(3 pi z) + N(0, 0.005), 50k
                    spray above it up to y = 0.9; H = 0.04, 1920x1080, step
                    0.25h, 1024 steps.
* ``batch``         64 sloshing-family scenes, N log-uniform in [50k, 2M],
                    h = 0.02 (1M/N)^(1/3), 1-4 cameras each on a radius-1.8
                    circle, resolutions from {640x480, 1280x720, 1920x1080}.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "Camera", "Scene", "look_at_lh", "perspective_lh_zo", "make_camera", "dam_break", "sloshing",
    "lattice_rest_density", "batch_scenes", "small_scene",
]


def look_at_lh(eye, center, up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """glm::lookAtLH as a column-major float64 4x4 (returned as [col][row])."""
    eye = np.asarray(eye, np.float64)
    center = np.asarray(center, np.float64)
    up = np.asarray(up, np.float64)
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(up, f)
    s /= np.linalg.norm(s)
    u = np.cross(f, s)
    m = np.eye(4)
    m[0, 0], m[1, 0], m[2, 0] = s
    m[0, 1], m[1, 1], m[2, 1] = u
    m[0, 2], m[1, 2], m[2, 2] = f
    m[3, 0] = -np.dot(s, eye)
    m[3, 1] = -np.dot(u, eye)
    m[3, 2] = -np.dot(f, eye)
    return m


def perspective_lh_zo(fovy: float, aspect: float, near: float, far: float, flip_y: bool = True) -> np.ndarray:
    """glm::perspectiveLH_ZO, then scale(1, -1, 1) (Camera3D.cpp:9)."""
    t = math.tan(fovy / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = 1.0 / (aspect * t)
    m[1, 1] = 1.0 / t
    m[2, 2] = far / (far - near)
    m[2, 3] = 1.0
    m[3, 2] = -(far * near) / (far - near)
    if flip_y:
        m[1, :] *= -1.0
    return m


def _colmajor(m: np.ndarray) -> np.ndarray:
    # m is indexed [col][row]; flatten col-major
    return np.ascontiguousarray(m.reshape(16), dtype=np.float32)


@dataclass
class Camera:
    """Pinhole camera in the reference's conventions (float32 matrices)."""

    view: np.ndarray          # (16,) float32, column-major
    proj: np.ndarray          # (16,) float32
    inv_proj_view: np.ndarray  # (16,) float32
    position: np.ndarray      # (3,) float32
    width: int
    height: int

    @property
    def n_pixels(self) -> int:
        return self.width * self.height


def make_camera(eye, target, width: int, height: int, fovy_deg: float = 60.0, near: float = 0.1,
                far: float = 1000.0) -> Camera:
    v = look_at_lh(eye, target)
    p = perspective_lh_zo(math.radians(fovy_deg), width / height, near, far)
    # [col][row] storage: (P*V)[c][r] = sum_k P[k][r] V[c][k]
    pv = np.einsum("kr,ck->cr", p, v)
    # inverse in row-major terms: M_rowmajor = pv.T
    inv = np.linalg.inv(pv.T).T
    return Camera(_colmajor(v), _colmajor(p), _colmajor(inv), np.asarray(eye, np.float32), int(width), int(height))


@dataclass
class Scene:
    """Particles plus the march settings of one configuration."""

    name: str
    xyz: np.ndarray            # (N, 3) float32
    support: float             # kernel/support radius H = 2h (the reference's ParticleRadius)
    iso: float                 # iso density (0.5 x lattice rest density)
    step: float                # march step size
    max_steps: int
    bisect: int
    cameras: list = field(default_factory=list)

    @property
    def n(self) -> int:
        return int(self.xyz.shape[0])


def _w_cubic(r: np.ndarray, H: float) -> np.ndarray:
    q = r / H
    sig = 8.0 / (math.pi * H ** 3)
    w = np.where(q < 0.5, 6.0 * (q ** 3 - q ** 2) + 1.0, 2.0 * (1.0 - q) ** 3)
    return np.where(q < 1.0, sig * w, 0.0)


def lattice_rest_density(spacing: float, H: float) -> float:
    """Rest density rho_0 = sum_j W(|x_j|) over an infinite cubic lattice at a site (FP64)."""
    k = int(math.ceil(H / spacing)) + 1
    g = np.arange(-k, k + 1) * spacing
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    r = np.sqrt(x * x + y * y + z * z)
    return float(_w_cubic(r, H).sum())


def dam_break(seed: int = 0, width: int = 640, height: int = 480) -> Scene:
    """64,000-particle jittered lattice (40^3, spacing 0.025) at the origin, H = 0.1."""
    rng = np.random.default_rng(seed)
    s = 0.025
    i = np.arange(40, dtype=np.float64) * s
    x, y, z = np.meshgrid(i, i, i, indexing="ij")
    base = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    jit = rng.uniform(-0.1 * s, 0.1 * s, size=base.shape)
    xyz = (base + jit).astype(np.float32)
    h = 0.05
    H = 2 * h
    rho0 = lattice_rest_density(s, H)
    cam = make_camera((1.8, 1.2, 1.8), (0.5, 0.3, 0.5), width, height)
    return Scene("dam_break", xyz, float(np.float32(H)), float(np.float32(0.5 * rho0)), float(np.float32(0.25 * h)),
                 512, 8, [cam])


def _surface(x, z):
    return 0.4 + 0.08 * np.sin(2 * np.pi * x) * np.cos(3 * np.pi * z)


def _sloshing_xyz(rng: np.random.Generator, n: int) -> np.ndarray:
    n_fluid = int(round(0.95 * n))
    n_spray = n - n_fluid
    out = []
    got = 0
    while got < n_fluid:
        m = max(1024, int((n_fluid - got) * 1.35))
        p = rng.uniform((0.0, 0.0, 0.0), (1.0, 0.5, 1.0), size=(m, 3))
        top = _surface(p[:, 0], p[:, 2]) + rng.normal(0.0, 0.005, size=m)
        p = p[p[:, 1] < top]
        out.append(p[: n_fluid - got])
        got += out[-1].shape[0]
    got = 0
    while got < n_spray:
        m = max(1024, int((n_spray - got) * 2.2))
        p = rng.uniform((0.0, 0.0, 0.0), (1.0, 0.9, 1.0), size=(m, 3))
        p = p[p[:, 1] > _surface(p[:, 0], p[:, 2])]
        out.append(p[: n_spray - got])
        got += out[-1].shape[0]
    return np.concatenate(out, axis=0).astype(np.float32)


def sloshing(seed: int = 1000, n: int = 1_000_000, h: float = 0.02, width: int = 1920, height: int = 1080,
             max_steps: int = 1024, bisect: int = 8) -> Scene:
    """Sloshing surface: 95% fluid below a sin/cos surface, 5% spray above it."""
    rng = np.random.default_rng(seed)
    xyz = _sloshing_xyz(rng, n)
    H = 2 * h
    spacing = (0.4 / (0.95 * n)) ** (1.0 / 3.0)
    rho0 = lattice_rest_density(spacing, H)
    cam = make_camera((1.8, 1.2, 1.8), (0.5, 0.3, 0.5), width, height)
    return Scene("sloshing", xyz, float(np.float32(H)), float(np.float32(0.5 * rho0)), float(np.float32(0.25 * h)),
                 max_steps, bisect, [cam])


def small_scene(seed: int = 7, n: int = 4000, width: int = 96, height: int = 72, bisect: int = 8,
                max_steps: int = 256) -> Scene:
    """A small sloshing-family scene for fast parity tests (same layout, scaled h)."""
    h = 0.02 * (1_000_000 / n) ** (1.0 / 3.0)
    return sloshing(seed=seed, n=n, h=h, width=width, height=height, max_steps=max_steps, bisect=bisect)


def batch_scenes(seed: int = 2000, n_scenes: int = 64, n_min: int = 50_000, n_max: int = 2_000_000,
                 max_steps: int = 1024, bisect: int = 8, scale: float = 1.0) -> list:
    """The batched configuration: scenes of the sloshing family with 1-4 views each.

    Particle counts are log-uniform in [n_min, n_max] and h = 0.02 (1M/N)^(1/3),
    so every scene has the same particles per kernel support.  ``scale`` < 1
    shrinks particle counts and resolutions together for quick tests.
    """
    rng = np.random.default_rng(seed)
    res = [(640, 480), (1280, 720), (1920, 1080)]
    out = []
    for s in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max))) * scale))
        n = max(n, 200)
        h = 0.02 * (1_000_000 / n) ** (1.0 / 3.0)
        sc = sloshing(seed=seed + 1 + s, n=n, h=h, width=8, height=8, max_steps=max_steps, bisect=bisect)
        cams = []
        for _ in range(int(rng.integers(1, 5))):
            ang = rng.uniform(0, 2 * math.pi)
            w, hgt = res[int(rng.integers(0, 3))]
            if scale != 1.0:
                w, hgt = max(16, int(w * scale)), max(12, int(hgt * scale))
            eye = (0.5 + 1.8 * math.cos(ang), 1.2, 0.5 + 1.8 * math.sin(ang))
            cams.append(make_camera(eye, (0.5, 0.3, 0.5), w, hgt))
        sc.cameras = cams
        sc.name = f"batch{s}"
        out.append(sc)
    return out
