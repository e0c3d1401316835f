"""ctypes wrapper for the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Loads ``oracle/liboracle.so`` (the CPU restatement, fm_oracle.cpp) and, when it
was built, ``oracle/_ref/libfmref.so`` (the reference's own RayMarcher
translation units, see ref_harness.cpp).  Only the tests, the smoke check and
the CPU-baseline leg of bench.py import this module.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libfmref.so")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")


class OrcCamera(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("proj", C.c_float * 16), ("inv_proj_view", C.c_float * 16),
                ("position", C.c_float * 3), ("width", C.c_int32), ("height", C.c_int32)]


class OrcGrid(C.Structure):
    _fields_ = [("min", C.c_float * 3), ("max", C.c_float * 3), ("cell", C.c_float), ("inv", C.c_float),
                ("dims", C.c_int32 * 3), ("pad", C.c_int32)]


class OrcParams(C.Structure):
    _fields_ = [("iso", C.c_float), ("step", C.c_float), ("max_steps", C.c_int32), ("bisect_iters", C.c_int32),
                ("skip_mode", C.c_int32), ("flags", C.c_int32)]


class OrcAniso(C.Structure):
    _fields_ = [("radius_mult", C.c_float), ("k_n", C.c_float), ("k_r", C.c_float), ("k_s", C.c_float),
                ("n_eps", C.c_int32), ("pad", C.c_int32)]


def build_oracle(ref: bool = True) -> None:
    """Compile liboracle.so (and oracle/_ref when the reference tree exists)."""
    target = "all" if ref else "oracle"
    subprocess.run(["make", "-C", HERE, "--no-print-directory", target], check=True,
                   stdout=subprocess.DEVNULL)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build_oracle(ref=False)
        L = C.CDLL(LIB_PATH)
        L.orc_W.restype = C.c_float
        L.orc_W.argtypes = [C.c_float] * 4
        L.orc_sigma.restype = C.c_float
        L.orc_sigma.argtypes = [C.c_float]
        L.orc_cos_poly.restype = C.c_float
        L.orc_cos_poly.argtypes = [C.c_float]
        L.orc_gradW.argtypes = [C.c_float] * 4 + [_f32p]
        L.orc_grid_params.argtypes = [_f32p, C.c_int64, C.c_int32, C.c_float, C.POINTER(OrcGrid)]
        L.orc_cells.argtypes = [_f32p, C.c_int64, C.c_int32, C.POINTER(OrcGrid), _u32p, _u32p]
        L.orc_sort.argtypes = [_u32p, C.c_int64, C.c_int64, _u32p, _u32p]
        L.orc_ref_flags.argtypes = [_u32p, C.POINTER(OrcGrid), C.c_float, C.c_void_p]
        L.orc_splat.argtypes = [_f32p, C.c_int64, C.c_int32, C.c_float, C.POINTER(OrcCamera), _f32p]
        L.orc_march.argtypes = [_f32p, _u32p, C.POINTER(OrcGrid), C.c_float, C.c_void_p, C.POINTER(OrcCamera),
                                C.POINTER(OrcParams), _f32p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32,
                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_march_ivl.argtypes = L.orc_march.argtypes + [C.c_void_p]
        L.orc_density_aniso.argtypes = [_f32p, _u32p, C.POINTER(OrcGrid), C.c_float, C.POINTER(OrcAniso), _f32p,
                                        C.c_int64, _f32p]
        L.orc_march_aniso.argtypes = [_f32p, _u32p, C.POINTER(OrcGrid), C.c_float, C.c_void_p, C.POINTER(OrcCamera),
                                      C.POINTER(OrcParams), C.POINTER(OrcAniso), _f32p, C.c_void_p, C.c_int64,
                                      C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_density.argtypes = [_f32p, _u32p, C.POINTER(OrcGrid), C.c_float, _f32p, C.c_int64, C.c_int32,
                                  np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")]
        L.orc_gauss_weights.argtypes = [C.c_int32, _f32p]
        L.orc_depth_blur.argtypes = [_f32p, _f32p, C.c_int32, C.c_int32, C.c_int32, C.c_float]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_PATH)
        R.ref_march.restype = C.c_double
        R.ref_march.argtypes = [_f32p, C.c_int64, C.c_float, _f32p, _f32p, C.c_int32, C.c_int32, _f32p, C.c_int32,
                                C.c_float, C.c_float, C.c_int32, _f32p, _f32p, C.c_void_p, C.c_void_p, C.c_void_p]
        R.ref_march_any.restype = C.c_double
        R.ref_march_any.argtypes = R.ref_march.argtypes + [C.c_int32, C.c_float, C.c_float, C.c_float, C.c_float,
                                                           C.c_int32]
        R.ref_W.restype = C.c_float
        R.ref_W.argtypes = [C.c_float] * 4
        R.ref_gradW.argtypes = [C.c_float] * 4 + [_f32p]
        R.ref_query_cells.argtypes = [_f32p, C.c_int64, C.c_float, _f32p, C.c_int64,
                                      np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")]
        R.ref_bgeo_positions.restype = C.c_int64
        R.ref_bgeo_positions.argtypes = [C.c_char_p, C.c_void_p, C.c_int64]
        R.ref_bgeo_write.argtypes = [C.c_char_p, _f32p, C.c_int64, C.c_int32]
        R.ref_dataset_load.restype = C.c_int32
        R.ref_dataset_load.argtypes = [C.c_char_p, C.c_char_p, C.c_int32, C.c_float, C.c_void_p, C.c_int32,
                                       C.POINTER(C.c_int64), C.c_void_p, C.c_int64]
        _ref = R
    return _ref


def camera_struct(cam) -> OrcCamera:
    c = OrcCamera()
    c.view[:] = [float(x) for x in cam.view]
    c.proj[:] = [float(x) for x in cam.proj]
    c.inv_proj_view[:] = [float(x) for x in cam.inv_proj_view]
    c.position[:] = [float(x) for x in cam.position]
    c.width = cam.width
    c.height = cam.height
    return c


@dataclass
class Frame:
    """Oracle grid build: cell table and cell-sorted particles."""

    grid: OrcGrid
    cells: np.ndarray    # (N,) uint32 cell of each input particle
    perm: np.ndarray     # (N,) uint32 input index of each sorted particle
    start: np.ndarray    # (ncells+1,) uint32 sorted range of each cell
    sorted: np.ndarray   # (N, 4) float32 cell-sorted xyz (w = 0)
    support: float
    sub_start: np.ndarray = None

    @property
    def dims(self):
        return tuple(self.grid.dims)

    @property
    def ncells(self) -> int:
        d = self.grid.dims
        return int(d[0]) * int(d[1]) * int(d[2])


def build_frame(xyz: np.ndarray, support: float) -> Frame:
    L = lib()
    xyz = np.ascontiguousarray(xyz, np.float32)
    n = xyz.shape[0]
    g = OrcGrid()
    if L.orc_grid_params(xyz, n, 3, support, C.byref(g)) != 0:
        raise ValueError("oracle grid: invalid input")
    cells = np.empty(n, np.uint32)
    keys = np.empty(n, np.uint32)
    L.orc_cells(xyz, n, 3, C.byref(g), cells, keys)
    ncells = int(g.dims[0]) * int(g.dims[1]) * int(g.dims[2])
    perm = np.empty(n, np.uint32)
    sub_start = np.empty(8 * ncells + 1, np.uint32)
    L.orc_sort(keys, n, 8 * ncells, perm, sub_start)
    start = np.ascontiguousarray(sub_start[::8])
    srt = np.zeros((n, 4), np.float32)
    srt[:, :3] = xyz[perm]
    return Frame(g, cells, perm, start, srt, float(support), sub_start)


def ref_flags(frame: Frame) -> np.ndarray:
    out = np.zeros(frame.ncells, np.uint8)
    lib().orc_ref_flags(frame.start, C.byref(frame.grid), frame.support, out.ctypes.data)
    return out


def splat(xyz: np.ndarray, support: float, cam) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, np.float32)
    out = np.empty(cam.width * cam.height, np.float32)
    cs = camera_struct(cam)
    lib().orc_splat(xyz, xyz.shape[0], 3, support, C.byref(cs), out)
    return out


def march(frame: Frame, cam, iso: float, step: float, max_steps: int, bisect: int, depth: np.ndarray,
          skip_mode: int = 0, pixels=None, threads: int = 0, precision: int = 32, want_colour: bool = True,
          intervals=None):
    """March all pixels (or the given pixel indices).  Returns a dict of arrays.

    intervals: optional (W*H, 2) int32 proposed intervals (ks, kf) of the
    learned march (fm_oracle.cpp march_pixel)."""
    L = lib()
    npx = cam.width * cam.height
    P = OrcParams(float(iso), float(step), int(max_steps), int(bisect), int(skip_mode), 0)
    cs = camera_struct(cam)
    pos = np.zeros((npx, 4), np.float32)
    nrm = np.zeros((npx, 4), np.float32)
    dep = np.zeros(npx, np.float32)
    col = np.zeros((npx, 4), np.float32)
    evals = np.zeros(npx, np.int32)
    cand = np.zeros(npx, np.int64)
    rho = np.zeros(npx, np.float64)
    flags = ref_flags(frame) if skip_mode == 2 else None
    pix = None
    npix = 0
    if pixels is not None:
        pix = np.ascontiguousarray(pixels, np.int64)
        npix = pix.shape[0]
    ivl = None if intervals is None else np.ascontiguousarray(intervals, np.int32).reshape(npx, 2)
    L.orc_march_ivl(np.ascontiguousarray(frame.sorted.reshape(-1)), frame.start, C.byref(frame.grid), frame.support,
                    flags.ctypes.data if flags is not None else None, C.byref(cs), C.byref(P),
                    np.ascontiguousarray(depth, np.float32), pix.ctypes.data if pix is not None else None, npix,
                    int(threads), int(precision), pos.ctypes.data, nrm.ctypes.data, dep.ctypes.data,
                    col.ctypes.data if want_colour else None, evals.ctypes.data, cand.ctypes.data, rho.ctypes.data,
                    ivl.ctypes.data if ivl is not None else None)
    return {"position": pos, "normal": nrm, "depth": dep, "colour": col, "evals": evals, "candidates": cand,
            "rho": rho}


def march_aniso(frame: Frame, cam, iso: float, step: float, max_steps: int, bisect: int, depth: np.ndarray,
                aniso=(2.0, 0.5, 2.0, 2000.0, 1), skip_mode: int = 0, pixels=None, threads: int = 0):
    """The anisotropic march (fm_oracle.cpp march_pixel_aniso); aniso = (radius_mult, k_n, k_r, k_s, n_eps)."""
    L = lib()
    npx = cam.width * cam.height
    P = OrcParams(float(iso), float(step), int(max_steps), int(bisect), int(skip_mode), 0)
    A = OrcAniso(float(aniso[0]), float(aniso[1]), float(aniso[2]), float(aniso[3]), int(aniso[4]), 0)
    cs = camera_struct(cam)
    pos = np.zeros((npx, 4), np.float32)
    nrm = np.zeros((npx, 4), np.float32)
    dep = np.zeros(npx, np.float32)
    evals = np.zeros(npx, np.int32)
    flags = ref_flags(frame) if skip_mode == 2 else None
    pix = None
    npix = 0
    if pixels is not None:
        pix = np.ascontiguousarray(pixels, np.int64)
        npix = pix.shape[0]
    L.orc_march_aniso(np.ascontiguousarray(frame.sorted.reshape(-1)), frame.start, C.byref(frame.grid),
                      frame.support, flags.ctypes.data if flags is not None else None, C.byref(cs), C.byref(P),
                      C.byref(A), np.ascontiguousarray(depth, np.float32), pix.ctypes.data if pix is not None else None,
                      npix, int(threads), pos.ctypes.data, nrm.ctypes.data, dep.ctypes.data, evals.ctypes.data)
    return {"position": pos, "normal": nrm, "depth": dep, "evals": evals}


def density_aniso(frame: Frame, pts: np.ndarray, aniso=(2.0, 0.5, 2.0, 2000.0, 1)) -> np.ndarray:
    pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
    out = np.empty(pts.shape[0], np.float32)
    A = OrcAniso(float(aniso[0]), float(aniso[1]), float(aniso[2]), float(aniso[3]), int(aniso[4]), 0)
    lib().orc_density_aniso(np.ascontiguousarray(frame.sorted.reshape(-1)), frame.start, C.byref(frame.grid),
                            frame.support, C.byref(A), pts, pts.shape[0], out)
    return out


def density(frame: Frame, pts: np.ndarray, precision: int = 32) -> np.ndarray:
    pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
    out = np.empty(pts.shape[0], np.float64)
    lib().orc_density(np.ascontiguousarray(frame.sorted.reshape(-1)), frame.start, C.byref(frame.grid),
                      frame.support, pts, pts.shape[0], int(precision), out)
    return out


def ref_march(xyz: np.ndarray, support: float, cam, depth: np.ndarray, max_steps: int, step: float, iso: float,
              box_mode: int = 0, aniso=None):
    """Run the reference's own RayMarcher (Oracle A) on the whole image.

    aniso: None (isotropic) or (radius_mult, k_n, k_r, k_s, n_eps) for the
    reference's anisotropic marcher."""
    R = ref()
    xyz = np.ascontiguousarray(xyz, np.float32)
    npx = cam.width * cam.height
    pos = np.zeros((npx, 4), np.float32)
    nrm = np.zeros((npx, 4), np.float32)
    srt = np.zeros((xyz.shape[0], 3), np.float32)
    grid = np.zeros(7, np.float32)
    build_s = C.c_double(0.0)
    an = (0, 2.0, 0.5, 2.0, 2000.0, 1) if aniso is None else (1,) + tuple(aniso)
    secs = R.ref_march_any(xyz, xyz.shape[0], support, np.ascontiguousarray(cam.inv_proj_view, np.float32),
                           np.ascontiguousarray(cam.position, np.float32), cam.width, cam.height,
                           np.ascontiguousarray(depth, np.float32), int(max_steps), float(step), float(iso),
                           int(box_mode), pos, nrm, srt.ctypes.data, grid.ctypes.data, C.byref(build_s),
                           int(an[0]), float(an[1]), float(an[2]), float(an[3]), float(an[4]), int(an[5]))
    if secs < 0:
        raise RuntimeError("reference march rejected its input")
    return {"position": pos, "normal": nrm, "sorted": srt, "grid": grid, "seconds": secs,
            "build_seconds": build_s.value}


def ref_bgeo_positions(path: str) -> np.ndarray:
    """Positions of a particle file as the reference reads it (Partio::read + Dataset::ReadFile)."""
    R = ref()
    n = R.ref_bgeo_positions(path.encode(), None, 0)
    if n < 0:
        raise IOError(f"Partio could not read {path}")
    out = np.zeros((n, 3), np.float32)
    R.ref_bgeo_positions(path.encode(), out.ctypes.data, n)
    return out


def ref_bgeo_write(path: str, xyz: np.ndarray, compressed: bool) -> None:
    """A particle file written by the reference's Partio."""
    x = np.ascontiguousarray(xyz, np.float32).reshape(-1)
    ref().ref_bgeo_write(path.encode(), x, x.size // 3, int(compressed))


def ref_dataset_load(prefix: str, suffix: str, count: int, radius: float, cap_points: int):
    """(frames, counts, max_particles, xyz of all frames) of the reference's Dataset constructor, or None."""
    R = ref()
    counts = np.zeros(4096, np.int64)
    mp = C.c_int64()
    xyz = np.zeros((cap_points, 3), np.float32)
    nf = R.ref_dataset_load(prefix.encode(), suffix.encode(), int(count), float(radius), counts.ctypes.data,
                            counts.size, C.byref(mp), xyz.ctypes.data, xyz.size)
    if nf < 0:
        return None
    return nf, counts[:nf].copy(), int(mp.value), xyz


def gauss_weights(n: int) -> np.ndarray:
    """ComputeGaussKernel's (n + 1) x (n + 1) weights (GaussRenderPass.cpp:24-57)."""
    out = np.zeros((n + 1) * (n + 1), np.float32)
    lib().orc_gauss_weights(int(n), out)
    return out.reshape(n + 1, n + 1)


def depth_blur(depth: np.ndarray, width: int, height: int, n: int = 8, spread: float = 1.0) -> np.ndarray:
    """The depth Gaussian blur of gauss.frag restated in FP32 (fm_oracle.cpp orc_depth_blur)."""
    src = np.ascontiguousarray(depth, np.float32).reshape(-1)
    out = np.zeros(width * height, np.float32)
    lib().orc_depth_blur(src, out, int(width), int(height), int(n), float(spread))
    return out

