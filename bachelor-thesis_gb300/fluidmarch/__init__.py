"""Python binding of libfluidmarch (ctypes over the C ABI in include/fluidmarch.h).

The classes mirror the reference's host interface for the march:

* :class:`Context`      ~ ``RayMarcher`` (RayMarcher.h:28-77): owns a CUDA stream.
* :class:`Scene`        ~ ``Frame`` (Dataset.h:37-65): particles + uniform grid.
* :class:`RayMarcher`   ~ ``RayMarcher::Prepare/Start/IsDone/Exit`` on top of the
                          two above, with the reference's ``VisualizationSettings``.

Arrays are numpy (host memory) or any object exposing ``data_ptr()`` (device
memory, e.g. a torch CUDA tensor).  Every call goes through the CUDA library;
there is no CPU fallback: if the library or a GPU is missing, calls raise.
"""

from __future__ import annotations

import ctypes as C
import os
import weakref
from dataclasses import dataclass

import numpy as np

from . import scenes  # noqa: F401  (re-export)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfluidmarch.so")

FM_OK, FM_ERR_INVALID, FM_ERR_CUDA, FM_ERR_TIMEOUT, FM_ERR_OOM, FM_ERR_DEVICE = 0, 1, 2, 3, 4, 5
FM_MEM_HOST, FM_MEM_DEVICE = 0, 1
FM_SKIP_OFF, FM_SKIP_EXACT, FM_SKIP_REFERENCE = 0, 1, 2
FM_MARCH_EXTERNAL_DEPTH = 1
FM_MARCH_PROPOSAL = 2
FM_MARCH_ANISOTROPIC = 4
FM_PROPOSAL_FEATURES = 32
FM_PROPOSAL_PARAMS = 6402

EXPORTS = [
    "fm_version", "fm_create", "fm_destroy", "fm_last_error", "fm_last_error_string", "fm_scene_upload", "fm_stream", "fm_sync", "fm_query", "fm_host_alloc",
    "fm_host_free", "fm_scene_create", "fm_scene_update", "fm_scene_destroy", "fm_scene_grid", "fm_scene_download",
    "fm_splat_depth", "fm_march", "fm_set_stats", "fm_march_stats_get", "fm_grid_build_noalloc",
    "fm_set_tile_config", "fm_get_tile_config", "fm_batch_create", "fm_batch_run", "fm_batch_refresh",
    "fm_batch_autotune", "fm_batch_info_get", "fm_batch_destroy", "fm_march_batch",
    "fm_proposal_create", "fm_proposal_destroy", "fm_set_proposal", "fm_proposal_features", "fm_proposal_intervals",
    "fm_judge", "fm_set_judge", "fm_judge_frames", "fm_trainer_create", "fm_trainer_destroy", "fm_trainer_step", "fm_trainer_predict",
    "fm_trainer_params", "fm_density", "fm_set_anisotropy",
    "fm_trainer_get_state", "fm_trainer_set_state", "fm_selftest_wait_timeout", "fm_depth_blur", "fm_bgeo_read", "fm_gunzip", "fm_scene_create_bgeo", "fm_dataset_open", "fm_dataset_frames", "fm_dataset_path",
    "fm_dataset_frame_info", "fm_dataset_max_particles", "fm_dataset_read", "fm_dataset_scene",
    "fm_dataset_last_error", "fm_dataset_close",
]


class FmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[fm error {code}] {msg}")
        self.code = code


class CCamera(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("proj", C.c_float * 16), ("inv_proj_view", C.c_float * 16),
                ("position", C.c_float * 3), ("width", C.c_int32), ("height", C.c_int32)]


class _HostBlock:
    """Frees an fm_host_alloc block when the array over it goes away."""

    def __init__(self, ctx, p: int):
        self.ctx, self.p = ctx, p

    def __del__(self):
        try:
            if self.p:
                self.ctx.L.fm_host_free(getattr(self.ctx, "h", None), C.c_void_p(self.p))
        except Exception:
            pass


class CBgeoInfo(C.Structure):
    _fields_ = [("points", C.c_uint64), ("record_words", C.c_uint32), ("attributes", C.c_uint32),
                ("file_bytes", C.c_uint64), ("data_bytes", C.c_uint64), ("compressed", C.c_int32),
                ("reserved", C.c_int32)]


class CMarchParams(C.Structure):
    _fields_ = [("iso_density", C.c_float), ("step_size", C.c_float), ("max_steps", C.c_int32),
                ("bisect_iters", C.c_int32), ("skip_mode", C.c_int32), ("flags", C.c_int32)]


class CFrameOut(C.Structure):
    _fields_ = [("position", C.c_void_p), ("normal", C.c_void_p), ("depth", C.c_void_p), ("colour", C.c_void_p),
                ("start_depth", C.c_void_p)]


class CGridInfo(C.Structure):
    _fields_ = [("min", C.c_float * 3), ("max", C.c_float * 3), ("cell_width", C.c_float),
                ("inv_cell_width", C.c_float), ("dims", C.c_int32 * 3), ("pad", C.c_int32),
                ("n_particles", C.c_uint64), ("n_cells", C.c_uint64)]


class CMarchStats(C.Structure):
    _fields_ = [("rays", C.c_uint64), ("started", C.c_uint64), ("hits", C.c_uint64), ("evals", C.c_uint64),
                ("candidates", C.c_uint64), ("skipped", C.c_uint64), ("tested", C.c_uint64),
                ("streamed", C.c_uint64), ("deferred", C.c_uint64), ("proposed", C.c_uint64),
                ("fallbacks", C.c_uint64), ("regrouped", C.c_uint64)]


class CJudge(C.Structure):
    _fields_ = [("pixels", C.c_uint64), ("hits_ref", C.c_uint64), ("hits_test", C.c_uint64),
                ("mask_mismatch", C.c_uint64), ("within_tol", C.c_uint64), ("max_err", C.c_float), ("tol", C.c_float)]


class CFrameJudge(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("sampled", C.c_uint64), ("hits_ref", C.c_uint64), ("hits_test", C.c_uint64),
                ("mask_mismatch", C.c_uint64), ("within_tol", C.c_uint64), ("max_err", C.c_float), ("tol", C.c_float)]


class CAniso(C.Structure):
    _fields_ = [("radius_mult", C.c_float), ("k_n", C.c_float), ("k_r", C.c_float), ("k_s", C.c_float),
                ("n_eps", C.c_int32), ("reserved", C.c_int32)]


class CTileConfig(C.Structure):
    _fields_ = [("tile_width", C.c_int32), ("tiles_per_claim", C.c_int32), ("defer_iters", C.c_int32),
                ("long_queue", C.c_int32), ("defer_lanes", C.c_int32), ("regroup_iters", C.c_int32)]


class CView(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", CCamera), ("params", CMarchParams), ("out", CFrameOut)]


class CBatchInfo(C.Structure):
    _fields_ = [("n_views", C.c_int32), ("graph_nodes", C.c_int32), ("pixels", C.c_uint64),
                ("particles", C.c_uint64), ("tiles", C.c_uint64), ("config", CTileConfig)]


_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load libfluidmarch.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} missing: run __graft_entry__.build() (the CUDA library is required)")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.fm_version.restype = C.c_int
    L.fm_create.argtypes = [C.POINTER(vp), C.c_int]
    L.fm_destroy.argtypes = [vp]
    L.fm_destroy.restype = None
    L.fm_last_error.argtypes = [vp]
    L.fm_last_error.restype = C.c_char_p
    L.fm_last_error_string.argtypes = [vp]
    L.fm_last_error_string.restype = C.c_char_p
    L.fm_scene_upload.argtypes = [vp, vp, C.c_uint64, C.c_int32, C.c_float, C.POINTER(vp)]
    L.fm_stream.argtypes = [vp]
    L.fm_stream.restype = vp
    L.fm_sync.argtypes = [vp, C.c_int]
    L.fm_query.argtypes = [vp]
    L.fm_host_alloc.argtypes = [vp, C.c_size_t, C.POINTER(vp)]
    L.fm_host_free.argtypes = [vp, vp]
    L.fm_host_free.restype = None
    L.fm_scene_create.argtypes = [vp, vp, C.c_uint64, C.c_uint32, C.c_float, C.c_int, C.POINTER(vp)]
    L.fm_scene_update.argtypes = [vp, vp, C.c_uint64, C.c_uint32, C.c_int]
    L.fm_scene_destroy.argtypes = [vp]
    L.fm_scene_destroy.restype = None
    L.fm_scene_grid.argtypes = [vp, C.POINTER(CGridInfo)]
    L.fm_scene_download.argtypes = [vp, vp, vp, vp, vp]
    L.fm_splat_depth.argtypes = [vp, vp, C.POINTER(CCamera), vp, C.c_int, vp]
    L.fm_march.argtypes = [vp, vp, C.POINTER(CCamera), C.POINTER(CMarchParams), C.POINTER(CFrameOut), C.c_int, vp]
    L.fm_set_stats.argtypes = [vp, C.c_int]
    L.fm_march_stats_get.argtypes = [vp, C.POINTER(CMarchStats)]
    L.fm_grid_build_noalloc.argtypes = [vp, C.c_uint64, C.c_uint32, C.c_float, vp, vp, vp, vp, C.c_uint64,
                                        C.POINTER(CGridInfo), vp]
    L.fm_density.argtypes = [vp, vp, vp, C.c_uint64, C.c_uint32, vp, C.c_int, vp]
    L.fm_set_anisotropy.argtypes = [vp, C.POINTER(CAniso)]
    L.fm_set_tile_config.argtypes = [vp, C.POINTER(CTileConfig)]
    L.fm_get_tile_config.argtypes = [vp, C.POINTER(CTileConfig)]
    L.fm_batch_create.argtypes = [vp, C.POINTER(CView), C.c_int32, C.POINTER(CTileConfig), C.POINTER(vp)]
    L.fm_batch_run.argtypes = [vp, vp]
    L.fm_batch_refresh.argtypes = [vp]
    L.fm_batch_autotune.argtypes = [vp, C.POINTER(CTileConfig), C.c_int32, C.c_int32, C.POINTER(CTileConfig),
                                    C.POINTER(C.c_float)]
    L.fm_batch_info_get.argtypes = [vp, C.POINTER(CBatchInfo)]
    L.fm_batch_destroy.argtypes = [vp]
    L.fm_batch_destroy.restype = None
    L.fm_march_batch.argtypes = [vp, C.POINTER(CView), C.c_int32, vp]
    L.fm_proposal_create.argtypes = [vp, vp, C.c_float, C.c_float, C.c_float, C.POINTER(vp)]
    L.fm_proposal_destroy.argtypes = [vp]
    L.fm_proposal_destroy.restype = None
    L.fm_set_proposal.argtypes = [vp, vp]
    L.fm_proposal_features.argtypes = [vp, vp, C.POINTER(CCamera), vp, vp, vp, vp]
    L.fm_proposal_intervals.argtypes = [vp, vp, C.POINTER(CCamera), C.POINTER(CMarchParams), vp, vp, vp, vp]
    L.fm_judge.argtypes = [vp, vp, vp, C.c_uint64, C.c_float, C.POINTER(CJudge), vp]
    L.fm_set_judge.argtypes = [vp, C.c_uint32, C.c_float]
    L.fm_judge_frames.argtypes = [vp, C.POINTER(CFrameJudge), C.c_int]
    L.fm_trainer_create.argtypes = [vp, C.c_uint64, vp, C.POINTER(vp)]
    L.fm_trainer_destroy.argtypes = [vp]
    L.fm_trainer_destroy.restype = None
    L.fm_trainer_step.argtypes = [vp, vp, vp, C.c_uint32, C.c_float, C.c_float, C.c_float, C.POINTER(C.c_float)]
    L.fm_trainer_predict.argtypes = [vp, vp, C.c_uint32, vp]
    L.fm_trainer_params.argtypes = [vp, vp]
    L.fm_trainer_get_state.argtypes = [vp, vp, C.POINTER(C.c_int64)]
    L.fm_selftest_wait_timeout.argtypes = [vp, C.c_uint32]
    L.fm_depth_blur.argtypes = [vp, vp, vp, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_int, vp]
    L.fm_trainer_set_state.argtypes = [vp, vp, C.c_int64]
    L.fm_bgeo_read.argtypes = [C.c_char_p, vp, C.c_uint64, C.POINTER(CBgeoInfo), C.c_char_p, C.c_uint64]
    L.fm_gunzip.argtypes = [vp, C.c_uint64, vp, C.c_uint64, C.POINTER(C.c_uint64)]
    L.fm_scene_create_bgeo.argtypes = [vp, C.c_char_p, C.c_float, C.POINTER(vp)]
    L.fm_dataset_open.argtypes = [C.c_char_p, C.c_char_p, C.c_int32, C.c_int32, C.POINTER(vp), C.c_char_p, C.c_uint64]
    L.fm_dataset_frames.argtypes = [vp]
    L.fm_dataset_frames.restype = C.c_int32
    L.fm_dataset_path.argtypes = [vp, C.c_int32]
    L.fm_dataset_path.restype = C.c_char_p
    L.fm_dataset_frame_info.argtypes = [vp, C.c_int32, C.POINTER(CBgeoInfo)]
    L.fm_dataset_max_particles.argtypes = [vp, C.POINTER(C.c_uint64)]
    L.fm_dataset_read.argtypes = [vp, C.c_int32, vp, C.c_uint64, C.POINTER(C.c_uint64)]
    L.fm_dataset_scene.argtypes = [vp, vp, C.c_int32, C.c_float, C.POINTER(vp)]
    L.fm_dataset_last_error.argtypes = [vp]
    L.fm_dataset_last_error.restype = C.c_char_p
    L.fm_dataset_close.argtypes = [vp]
    L.fm_dataset_close.restype = None
    _lib = L
    return L


def _ptr(a):
    """(address, memkind) of a numpy array or a device tensor."""
    if a is None:
        return None, None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be C-contiguous")
        return a.ctypes.data, FM_MEM_HOST
    if hasattr(a, "data_ptr"):
        dev = getattr(a, "is_cuda", True)
        return a.data_ptr(), (FM_MEM_DEVICE if dev else FM_MEM_HOST)
    raise TypeError(f"unsupported array type {type(a)}")


def camera_struct(cam) -> CCamera:
    c = CCamera()
    c.view[:] = [float(x) for x in np.asarray(cam.view, np.float32)]
    c.proj[:] = [float(x) for x in np.asarray(cam.proj, np.float32)]
    c.inv_proj_view[:] = [float(x) for x in np.asarray(cam.inv_proj_view, np.float32)]
    c.position[:] = [float(x) for x in np.asarray(cam.position, np.float32)]
    c.width, c.height = int(cam.width), int(cam.height)
    return c


class Context:
    """A device context (``RayMarcher()`` in the reference)."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = C.c_void_p()
        rc = self.L.fm_create(C.byref(h), int(device))
        if rc != FM_OK:
            raise FmError(rc, f"fm_create(device={device}) failed")
        self.h = h
        self._scenes = weakref.WeakSet()
        self._batches = weakref.WeakSet()
        self._proposals = weakref.WeakSet()
        self._trainers = weakref.WeakSet()

    def check(self, rc: int):
        if rc != FM_OK:
            raise FmError(rc, self.L.fm_last_error(self.h).decode())

    @property
    def stream(self) -> int:
        return self.L.fm_stream(self.h) or 0

    def sync(self, timeout_ms: int = -1):
        self.check(self.L.fm_sync(self.h, int(timeout_ms)))

    def query(self) -> bool:
        r = self.L.fm_query(self.h)
        if r < 0:
            raise FmError(-r, self.L.fm_last_error(self.h).decode())
        return r == 1

    def set_stats(self, on: bool):
        self.check(self.L.fm_set_stats(self.h, 1 if on else 0))

    def stats(self) -> dict:
        s = CMarchStats()
        self.check(self.L.fm_march_stats_get(self.h, C.byref(s)))
        return {k: int(getattr(s, k)) for k, _ in CMarchStats._fields_}

    def set_tile_config(self, tile_width: int = 8, tiles_per_claim: int = 1, defer_iters: int = 0,
                        long_queue: int = 0, defer_lanes: int = 2, regroup_iters: int = 0):
        """Work split of single-view marches (results do not depend on it)."""
        c = CTileConfig(int(tile_width), int(tiles_per_claim), int(defer_iters), int(long_queue), int(defer_lanes),
                        int(regroup_iters))
        self.check(self.L.fm_set_tile_config(self.h, C.byref(c)))

    def set_judge(self, stride: int, tol: float):
        """Judge every learned march: the plain march of a 1-in-`stride` pixel sample, compared on the
        device (hit masks, hit distances within `tol`); stride 0 turns it off."""
        self.check(self.L.fm_set_judge(self.h, int(stride), float(tol)))

    def judge_frames(self, reset: bool = False) -> dict:
        """What the per-frame judge accumulated since the last reset."""
        r = CFrameJudge()
        self.check(self.L.fm_judge_frames(self.h, C.byref(r), 1 if reset else 0))
        return {k: (float(getattr(r, k)) if k in ("max_err", "tol") else int(getattr(r, k))) for k, _ in
                CFrameJudge._fields_}

    def host_array(self, shape, dtype=np.float32) -> np.ndarray:
        """A numpy array in page-locked host memory of this context (fm_host_alloc).

        March outputs placed in such arrays are written by the kernels directly,
        without a copy after the march; the block is freed with the array."""
        dt = np.dtype(dtype)
        nbytes = max(1, int(np.prod(shape)) * dt.itemsize)
        p = C.c_void_p()
        self.check(self.L.fm_host_alloc(self.h, nbytes, C.byref(p)))
        buf = (C.c_char * nbytes).from_address(p.value)
        buf._fm_block = _HostBlock(self, p.value)
        return np.frombuffer(buf, dt, count=int(np.prod(shape))).reshape(shape)

    def set_anisotropy(self, radius_mult: float = 2.0, k_n: float = 0.5, k_r: float = 2.0, k_s: float = 2000.0,
                       n_eps: int = 1):
        """Kernels of the anisotropic march (VisualizationSettings k_n, k_r, k_s, N_eps)."""
        a = CAniso(float(radius_mult), float(k_n), float(k_r), float(k_s), int(n_eps), 0)
        self.check(self.L.fm_set_anisotropy(self.h, C.byref(a)))

    def tile_config(self) -> dict:
        c = CTileConfig()
        self.check(self.L.fm_get_tile_config(self.h, C.byref(c)))
        return _tile_dict(c)

    def close(self):
        """Destroy the context; its batches and scenes that are still open are closed first."""
        if getattr(self, "h", None):
            for b in list(self._batches):
                b.close()
            for t in list(self._trainers):
                t.close()
            for p in list(self._proposals):
                p.close()
            for sc in list(self._scenes):
                sc.close()
            self.L.fm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    """Particles plus their uniform grid (``Frame`` in the reference)."""

    def __init__(self, ctx: Context, xyz, support: float, stride: int = 3):
        self.ctx = ctx
        p, mem = _ptr(xyz)
        n = int(xyz.shape[0])
        h = C.c_void_p()
        ctx.check(ctx.L.fm_scene_create(ctx.h, p, n, int(stride), float(support), mem, C.byref(h)))
        self.h = h
        self.support = float(support)
        ctx._scenes.add(self)

    @classmethod
    def wrap(cls, ctx: Context, handle, support: float) -> "Scene":
        """A Scene object for a handle the library created (particle files, datasets)."""
        s = cls.__new__(cls)
        s.ctx = ctx
        s.h = handle if isinstance(handle, C.c_void_p) else C.c_void_p(handle)
        s.support = float(support)
        ctx._scenes.add(s)
        return s

    def update(self, xyz, stride: int = 3):
        p, mem = _ptr(xyz)
        self.ctx.check(self.ctx.L.fm_scene_update(self.h, p, int(xyz.shape[0]), int(stride), mem))

    def grid(self) -> dict:
        g = CGridInfo()
        self.ctx.check(self.ctx.L.fm_scene_grid(self.h, C.byref(g)))
        return {"min": np.array(g.min[:], np.float32), "max": np.array(g.max[:], np.float32),
                "cell_width": g.cell_width, "inv_cell_width": g.inv_cell_width, "dims": tuple(g.dims[:]),
                "n_particles": int(g.n_particles), "n_cells": int(g.n_cells)}

    def download(self) -> dict:
        g = self.grid()
        n, nc = g["n_particles"], g["n_cells"]
        cell = np.empty(n, np.uint32)
        perm = np.empty(n, np.uint32)
        start = np.empty(nc + 1, np.uint32)
        pts = np.empty((n, 4), np.float32)
        self.ctx.check(self.ctx.L.fm_scene_download(self.h, cell.ctypes.data, perm.ctypes.data, start.ctypes.data,
                                                    pts.ctypes.data))
        return {"cell": cell, "perm": perm, "start": start, "sorted": pts}

    def close(self):
        if getattr(self, "h", None):
            if getattr(self.ctx, "h", None):  # a closed context already freed its scenes
                self.ctx.L.fm_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class MarchParams:
    """``VisualizationSettings`` fields of the isotropic march, plus bisection and skip mode."""

    iso: float
    step: float
    max_steps: int
    bisect: int = 0
    skip_mode: int = FM_SKIP_OFF
    external_depth: bool = False
    proposal: bool = False
    anisotropic: bool = False

    def cstruct(self) -> CMarchParams:
        flags = (FM_MARCH_EXTERNAL_DEPTH if self.external_depth else 0) | (FM_MARCH_PROPOSAL if self.proposal else 0)
        flags |= FM_MARCH_ANISOTROPIC if self.anisotropic else 0
        return CMarchParams(float(self.iso), float(self.step), int(self.max_steps), int(self.bisect),
                            int(self.skip_mode), flags)


def density(scene: Scene, xyz, out=None, stride: int = 3, stream=None):
    """SPH density at points (DiskRenderer::ComputeDensity); numpy in -> numpy out unless ``out`` is given."""
    ctx = scene.ctx
    n = int(xyz.shape[0])
    if out is None:
        out = np.empty(n, np.float32)
    p, mem = _ptr(xyz)
    q, mem2 = _ptr(out)
    if mem != mem2:
        raise ValueError("points and output must both be host or both be device buffers")
    ctx.check(ctx.L.fm_density(ctx.h, scene.h, p, n, int(stride), q, mem, stream))
    return out


def splat_depth(scene: Scene, cam, out=None, stream=None):
    """Depth pass: returns a (H*W,) float32 buffer cleared to 1.0 (numpy unless ``out`` is given)."""
    ctx = scene.ctx
    if out is None:
        out = np.empty(cam.width * cam.height, np.float32)
    p, mem = _ptr(out)
    cs = camera_struct(cam)
    ctx.check(ctx.L.fm_splat_depth(ctx.h, scene.h, C.byref(cs), p, mem, stream))
    return out


def march(scene: Scene, cam, params: MarchParams, position=None, normal=None, depth=None, colour=None,
          start_depth=None, stream=None):
    """Render one view.  Outputs are the given buffers (all host or all device).

    Asynchronous for device buffers and for host buffers that all come from
    ``Context.host_array`` (call ``ctx.sync()`` before reading them); other host
    buffers are written when the call returns."""
    ctx = scene.ctx
    bufs = [position, normal, depth, colour, start_depth]
    mems = {m for m in (_ptr(b)[1] for b in bufs) if m is not None}
    if len(mems) > 1:
        raise ValueError("outputs must all be host or all be device buffers")
    mem = mems.pop() if mems else FM_MEM_HOST
    o = CFrameOut(*[_ptr(b)[0] for b in bufs])
    cs = camera_struct(cam)
    ps = params.cstruct()
    ctx.check(ctx.L.fm_march(ctx.h, scene.h, C.byref(cs), C.byref(ps), C.byref(o), mem, stream))


def depth_blur(ctx: Context, depth, width: int, height: int, n: int = 8, spread: float = 1.0, out=None,
               stream=None):
    """The depth Gaussian blur pass (GaussRenderPass / gauss.frag); numpy in -> numpy out unless out is given."""
    if out is None:
        out = np.empty(width * height, np.float32)
    p, mem = _ptr(depth)
    q, mem2 = _ptr(out)
    if mem != mem2:
        raise ValueError("depth and output must both be host or both be device buffers")
    ctx.check(ctx.L.fm_depth_blur(ctx.h, p, q, int(width), int(height), int(n), float(spread), mem, stream))
    return out


def render(scene: Scene, cam, params: MarchParams, want_start: bool = True) -> dict:
    """Convenience: march one view into fresh numpy buffers."""
    npx = cam.width * cam.height
    out = {"position": np.zeros((npx, 4), np.float32), "normal": np.zeros((npx, 4), np.float32),
           "depth": np.zeros(npx, np.float32), "colour": np.zeros((npx, 4), np.float32)}
    if want_start:
        out["start_depth"] = np.zeros(npx, np.float32)
    march(scene, cam, params, out["position"], out["normal"], out["depth"], out["colour"], out.get("start_depth"))
    return out


def _tile_dict(c: CTileConfig) -> dict:
    return {"tile_width": int(c.tile_width), "tiles_per_claim": int(c.tiles_per_claim),
            "defer_iters": int(c.defer_iters), "long_queue": int(c.long_queue), "defer_lanes": int(c.defer_lanes),
            "regroup_iters": int(c.regroup_iters)}


def _tile_struct(d: dict) -> CTileConfig:
    return CTileConfig(int(d["tile_width"]), int(d.get("tiles_per_claim", 1)), int(d.get("defer_iters", 0)),
                       int(d.get("long_queue", 0)), int(d.get("defer_lanes", 2)), int(d.get("regroup_iters", 0)))


@dataclass
class View:
    """One view of a batch: scene, camera, march settings and DEVICE output buffers."""

    scene: Scene
    camera: object
    params: MarchParams
    position: object = None
    normal: object = None
    depth: object = None
    colour: object = None
    start_depth: object = None

    def cstruct(self) -> CView:
        if self.params.external_depth:
            raise ValueError("batched views are splatted: external_depth must be False")
        ptrs = []
        for b in (self.position, self.normal, self.depth, self.colour, self.start_depth):
            p, mem = _ptr(b)
            if p is not None and mem != FM_MEM_DEVICE:
                raise ValueError("batch outputs must be device buffers")
            ptrs.append(p)
        return CView(self.scene.h, camera_struct(self.camera), self.params.cstruct(), CFrameOut(*ptrs))


class Batch:
    """Many views of many scenes rendered by one launch per pass under a CUDA graph."""

    def __init__(self, ctx: Context, views: list, tile_config: dict | None = None):
        self.ctx = ctx
        self.views = list(views)  # keeps the scenes and buffers alive
        arr = (CView * len(views))(*[v.cstruct() for v in views])
        cfg = None
        if tile_config is not None:
            cfg = C.byref(_tile_struct(tile_config))
        h = C.c_void_p()
        ctx.check(ctx.L.fm_batch_create(ctx.h, arr, len(views), cfg, C.byref(h)))
        self.h = h
        ctx._batches.add(self)

    def run(self, stream=None):
        self.ctx.check(self.ctx.L.fm_batch_run(self.h, stream))

    def refresh(self):
        self.ctx.check(self.ctx.L.fm_batch_refresh(self.h))

    def autotune(self, reps: int = 2, candidates: list | None = None) -> tuple:
        best = CTileConfig()
        ms = C.c_float()
        if candidates:
            arr = (CTileConfig * len(candidates))(*[_tile_struct(c) for c in candidates])
            rc = self.ctx.L.fm_batch_autotune(self.h, arr, len(candidates), int(reps), C.byref(best), C.byref(ms))
        else:
            rc = self.ctx.L.fm_batch_autotune(self.h, None, 0, int(reps), C.byref(best), C.byref(ms))
        self.ctx.check(rc)
        return _tile_dict(best), float(ms.value)

    def info(self) -> dict:
        i = CBatchInfo()
        self.ctx.check(self.ctx.L.fm_batch_info_get(self.h, C.byref(i)))
        return {"n_views": int(i.n_views), "graph_nodes": int(i.graph_nodes), "pixels": int(i.pixels),
                "particles": int(i.particles), "tiles": int(i.tiles), "config": _tile_dict(i.config)}

    def close(self):
        if getattr(self, "h", None):
            if getattr(self.ctx, "h", None):  # a closed context already freed its batches
                self.ctx.L.fm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Proposal:
    """Learned hit-interval proposal (MLP parameters on the device)."""

    def __init__(self, ctx: Context, params, margin_lo: float = 0.0, margin_hi: float = 0.0, min_near: float = 0.0):
        self.ctx = ctx
        p = np.ascontiguousarray(params, np.float32).reshape(-1)
        if p.size != FM_PROPOSAL_PARAMS:
            raise ValueError(f"expected {FM_PROPOSAL_PARAMS} parameters, got {p.size}")
        h = C.c_void_p()
        ctx.check(ctx.L.fm_proposal_create(ctx.h, p.ctypes.data, float(margin_lo), float(margin_hi), float(min_near),
                                           C.byref(h)))
        self.h = h
        self.params = p
        ctx._proposals.add(self)

    def close(self):
        if getattr(self, "h", None):
            if getattr(self.ctx, "h", None):
                self.ctx.L.fm_proposal_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_proposal(ctx: Context, p):
    ctx.check(ctx.L.fm_set_proposal(ctx.h, p.h if p is not None else None))
    ctx._active_proposal = p


def proposal_features(scene: Scene, cam, start_depth, features, t0=None, stream=None):
    """Features of every pixel's ray into device buffers (W*H x 32 floats, W*H floats)."""
    ctx = scene.ctx
    cs = camera_struct(cam)
    ctx.check(ctx.L.fm_proposal_features(ctx.h, scene.h, C.byref(cs), _ptr(start_depth)[0], _ptr(features)[0],
                                         _ptr(t0)[0], stream))


def proposal_intervals(scene: Scene, cam, params: MarchParams, start_depth, intervals, near_far=None, stream=None):
    ctx = scene.ctx
    cs = camera_struct(cam)
    ps = params.cstruct()
    ctx.check(ctx.L.fm_proposal_intervals(ctx.h, scene.h, C.byref(cs), C.byref(ps), _ptr(start_depth)[0],
                                          _ptr(intervals)[0], _ptr(near_far)[0], stream))


def judge(ctx: Context, depth_ref, depth_test, tol: float, stream=None) -> dict:
    """Hit-mask mismatches and depth errors of depth_test against depth_ref (device buffers)."""
    r = CJudge()
    n = int(depth_ref.numel()) if hasattr(depth_ref, "numel") else int(depth_ref.size)
    ctx.check(ctx.L.fm_judge(ctx.h, _ptr(depth_ref)[0], _ptr(depth_test)[0], n, float(tol), C.byref(r), stream))
    return {k: (float(getattr(r, k)) if k in ("max_err", "tol") else int(getattr(r, k))) for k, _ in CJudge._fields_}


class Trainer:
    """FP32 trainer of the proposal MLP (forward, backward, Adam kernels)."""

    def __init__(self, ctx: Context, seed: int = 0, init=None):
        self.ctx = ctx
        h = C.c_void_p()
        ip = None
        if init is not None:
            self._init = np.ascontiguousarray(init, np.float32).reshape(-1)
            ip = self._init.ctypes.data
        ctx.check(ctx.L.fm_trainer_create(ctx.h, int(seed), ip, C.byref(h)))
        self.h = h
        ctx._trainers.add(self)

    def step(self, features, targets, n: int, lr: float, tau_lo: float, tau_hi: float, want_loss: bool = False):
        loss = C.c_float()
        self.ctx.check(self.ctx.L.fm_trainer_step(self.h, _ptr(features)[0], _ptr(targets)[0], int(n), float(lr),
                                                  float(tau_lo), float(tau_hi),
                                                  C.byref(loss) if want_loss else None))
        return float(loss.value) if want_loss else None

    def predict(self, features, n: int, out):
        self.ctx.check(self.ctx.L.fm_trainer_predict(self.h, _ptr(features)[0], int(n), _ptr(out)[0]))

    def params(self) -> np.ndarray:
        p = np.empty(FM_PROPOSAL_PARAMS, np.float32)
        self.ctx.check(self.ctx.L.fm_trainer_params(self.h, p.ctypes.data))
        return p

    def state(self) -> tuple:
        """(3 x FM_PROPOSAL_PARAMS state: parameters, Adam first and second moments; Adam step)."""
        s = np.empty(3 * FM_PROPOSAL_PARAMS, np.float32)
        step = C.c_int64()
        self.ctx.check(self.ctx.L.fm_trainer_get_state(self.h, s.ctypes.data, C.byref(step)))
        return s, int(step.value)

    def set_state(self, state, step: int):
        s = np.ascontiguousarray(state, np.float32).reshape(-1)
        if s.size != 3 * FM_PROPOSAL_PARAMS:
            raise ValueError(f"expected {3 * FM_PROPOSAL_PARAMS} floats, got {s.size}")
        self.ctx.check(self.ctx.L.fm_trainer_set_state(self.h, s.ctypes.data, int(step)))

    def close(self):
        if getattr(self, "h", None):
            if getattr(self.ctx, "h", None):
                self.ctx.L.fm_trainer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def march_batch(ctx: Context, views: list, stream=None):
    """One-shot batch: create, run, wait, destroy."""
    arr = (CView * len(views))(*[v.cstruct() for v in views])
    ctx.check(ctx.L.fm_march_batch(ctx.h, arr, len(views), stream))


class RayMarcher:
    """Mirror of the reference's ``RayMarcher`` host class (RayMarcher.h:28-77).

    ``prepare(settings, camera, scene, positions, normals, depth)`` takes the
    same arguments as ``RayMarcher::Prepare`` (RayMarcher.cpp:76-100): the
    depth buffer is the ray-start (splat) depth the reference consumes; the
    marcher writes positions and normals.  ``start()`` launches on the
    context's stream, ``is_done()`` polls it, ``exit()`` waits.
    """

    def __init__(self, device: int = 0):
        self.ctx = Context(device)
        self._args = None

    def prepare(self, settings: MarchParams, camera, scene: Scene, positions, normals, depth):
        if positions is None or normals is None or depth is None:
            raise ValueError("positions, normals and depth buffers are required")
        if scene.ctx is not self.ctx:
            raise ValueError("the scene belongs to another context")
        self._args = (settings, camera, scene, positions, normals, depth)

    def start(self):
        if self._args is None:
            raise RuntimeError("prepare() first")
        settings, camera, scene, positions, normals, depth = self._args
        p = MarchParams(settings.iso, settings.step, settings.max_steps, settings.bisect, settings.skip_mode, True)
        march(scene, camera, p, position=positions, normal=normals, start_depth=depth,
              stream=None)

    def is_done(self) -> bool:
        return self.ctx.query()

    def exit(self):
        self.ctx.sync()
