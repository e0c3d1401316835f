"""Particle files: classic BGEO frames (the reference's dataset format) and numbered series.

* ``write``       a classic BGEO (version 5) file: positions plus optional point
                  attributes (float, int, vector, indexed string), plain or
                  gzip-compressed; the layout Partio writes
                  (vendor/partio/src/io/BGEO.cpp writeBGEO: big-endian header,
                  attribute definitions with zero defaults, one record per point
                  with w = 1, no primitives, no detail attributes, then 0x00 0xff);
* ``read``        positions of a file through the library's host reader (``fm_bgeo_read``);
* ``load_scene``  a scene straight from a file (``fm_scene_create_bgeo``);
* ``Dataset``     a series prefix + i + suffix (``Dataset::Dataset``, Dataset.cpp:169-227) whose
                  frames host threads decode ahead; ``autoplay`` marches every frame in order, the
                  next one once the previous march finished (AdvancedRenderer.cpp:281-297).
"""

from __future__ import annotations

import ctypes as C
import gzip
import io
import struct

import numpy as np

import fluidmarch as fm

TYPES = {"float": 0, "int": 1, "vector": 5, "indexed": 4}


def _hstr(s: str) -> bytes:
    b = s.encode()
    return struct.pack(">H", len(b)) + b


def encode(xyz, attributes: dict | None = None) -> bytes:
    """The uncompressed bytes of a BGEO file.

    attributes: name -> (kind, values[, strings]) with kind in TYPES; values is
    an (n, size) array (float32 for float / vector, int32 for int and indexed
    string indices); strings is the table of an indexed string attribute.
    """
    xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    n = xyz.shape[0]
    attributes = attributes or {}
    head = [b"Bgeo", b"V", struct.pack(">9i", 5, n, 0, 0, 0, len(attributes), 0, 0, 0)]
    cols = [xyz.view(np.uint32), np.full((n, 1), np.float32(1.0)).view(np.uint32)]
    for name, spec in attributes.items():
        kind, values = spec[0], spec[1]
        t = TYPES[kind]
        vals = np.asarray(values).reshape(n, -1)
        size = vals.shape[1]
        head.append(_hstr(name) + struct.pack(">Hi", size, t))
        if t == 4:
            strings = spec[2]
            head.append(struct.pack(">i", len(strings)) + b"".join(_hstr(s) for s in strings))
        else:
            head.append(b"\0" * (4 * size))
        dt = np.int32 if t in (1, 4) else np.float32
        cols.append(np.ascontiguousarray(vals, dt).view(np.uint32))
    rec = np.concatenate(cols, axis=1).astype(">u4")
    return b"".join(head) + rec.tobytes() + b"\x00\xff"


def write(path: str, xyz, attributes: dict | None = None, compressed: bool = True, level: int = 6) -> None:
    data = encode(xyz, attributes)
    if compressed:
        buf = io.BytesIO()
        with gzip.GzipFile(fileobj=buf, mode="wb", compresslevel=level, mtime=0) as g:
            g.write(data)
        data = buf.getvalue()
    with open(path, "wb") as f:
        f.write(data)


def _info(ci: fm.CBgeoInfo) -> dict:
    return {"points": int(ci.points), "record_words": int(ci.record_words), "attributes": int(ci.attributes),
            "file_bytes": int(ci.file_bytes), "data_bytes": int(ci.data_bytes), "compressed": bool(ci.compressed)}


def info(path: str) -> dict:
    """Header of a file (no decoding of the point data)."""
    L = fm.load()
    ci = fm.CBgeoInfo()
    err = C.create_string_buffer(512)
    rc = L.fm_bgeo_read(path.encode(), None, 0, C.byref(ci), err, 512)
    if rc != fm.FM_OK:
        raise fm.FmError(rc, err.value.decode())
    return _info(ci)


def read(path: str) -> np.ndarray:
    """(n, 3) float32 positions of a file, read on the host by the library."""
    n = info(path)["points"]
    L = fm.load()
    out = np.empty((n, 3), np.float32)
    err = C.create_string_buffer(512)
    rc = L.fm_bgeo_read(path.encode(), out.ctypes.data, n, None, err, 512)
    if rc != fm.FM_OK:
        raise fm.FmError(rc, err.value.decode())
    return out


def gunzip(data: bytes) -> bytes:
    """The library's gzip decoder (first member, CRC-32 and length checked)."""
    L = fm.load()
    n = C.c_uint64()
    src = C.create_string_buffer(data, len(data))
    # the member's size field (last 4 bytes) sizes the buffer; DEFLATE expands
    # at most ~1032:1, which bounds a corrupt field
    cap = min(int.from_bytes(data[-4:], "little"), 1032 * len(data) + 65536) if len(data) >= 4 else 0
    out = C.create_string_buffer(max(1, cap))
    rc = L.fm_gunzip(src, len(data), out, cap, C.byref(n))
    if rc != fm.FM_OK and n.value > cap:  # decoded, but larger than the size field said
        cap = n.value
        out = C.create_string_buffer(cap)
        rc = L.fm_gunzip(src, len(data), out, cap, C.byref(n))
    if rc != fm.FM_OK:
        raise fm.FmError(rc, "gzip decoding failed")
    return out.raw[:n.value]


def load_scene(ctx: fm.Context, path: str, support: float) -> fm.Scene:
    h = C.c_void_p()
    ctx.check(ctx.L.fm_scene_create_bgeo(ctx.h, path.encode(), float(support), C.byref(h)))
    return fm.Scene.wrap(ctx, h, support)


class Dataset:
    """A numbered series of BGEO frames (``Dataset::Dataset``)."""

    def __init__(self, prefix: str, suffix: str = ".bgeo", count: int = -1, threads: int = 2):
        self.L = fm.load()
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = self.L.fm_dataset_open(prefix.encode(), suffix.encode(), int(count), int(threads), C.byref(h), err, 512)
        if rc != fm.FM_OK:
            raise fm.FmError(rc, err.value.decode())
        self.h = h
        self.scene = None

    def __len__(self) -> int:
        return int(self.L.fm_dataset_frames(self.h))

    def _check(self, rc: int):
        if rc != fm.FM_OK:
            raise fm.FmError(rc, (self.L.fm_dataset_last_error(self.h) or b"").decode())

    def path(self, i: int) -> str:
        p = self.L.fm_dataset_path(self.h, int(i))
        if p is None:
            raise IndexError(i)
        return p.decode()

    def frame_info(self, i: int) -> dict:
        ci = fm.CBgeoInfo()
        self._check(self.L.fm_dataset_frame_info(self.h, int(i), C.byref(ci)))
        return _info(ci)

    def max_particles(self) -> int:
        m = C.c_uint64()
        self._check(self.L.fm_dataset_max_particles(self.h, C.byref(m)))
        return int(m.value)

    def read(self, i: int) -> np.ndarray:
        n = C.c_uint64()
        self._check(self.L.fm_dataset_read(self.h, int(i), None, 0, C.byref(n)))
        out = np.empty((n.value, 3), np.float32)
        self._check(self.L.fm_dataset_read(self.h, int(i), out.ctypes.data, n.value, C.byref(n)))
        return out

    def load(self, ctx: fm.Context, i: int, support: float) -> fm.Scene:
        """Frame i as the dataset's scene (rebuilt in place when it fits, else replaced)."""
        h = C.c_void_p(self.scene.h.value if self.scene is not None and self.scene.h else None)
        ctx.check(ctx.L.fm_dataset_scene(self.h, ctx.h, int(i), float(support), C.byref(h)))
        if self.scene is None or self.scene.h is None or self.scene.h.value != h.value:
            if self.scene is not None:
                self.scene.h = None  # the library destroyed the old one
            self.scene = fm.Scene.wrap(ctx, h, support)
        return self.scene

    def autoplay(self, ctx: fm.Context, camera, params: fm.MarchParams, support: float, out: dict | None = None,
                 start: int = 0):
        """Yields (frame index, outputs) for frames start, start+1, ... up to the last one."""
        for i in range(start, len(self)):
            scene = self.load(ctx, i, support)
            if out is None:
                yield i, fm.render(scene, camera, params)
            else:
                fm.march(scene, camera, params, out["position"], out["normal"], out["depth"], out.get("colour"),
                         out.get("start_depth"))
                ctx.sync()  # outputs in the library's pinned memory are written asynchronously
                yield i, out

    def close(self):
        if getattr(self, "h", None):
            if self.scene is not None:
                self.scene.close()
                self.scene = None
            self.L.fm_dataset_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
