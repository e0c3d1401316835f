"""Particle files on the host: the gzip decoder, the BGEO reader and numbered series.

* The library's gzip / DEFLATE decoder against Python's zlib on stored, fixed
  and dynamic Huffman blocks, every gzip header field, corrupt and truncated
  streams.
* The BGEO reader against the reference's own reader (the vendored Partio,
  compiled into oracle/_ref): files written by this package and files written
  by Partio give the same position bits.
* Series: the frames and particle counts the reference's Dataset constructor
  finds for prefix + i + suffix, and the positions of every frame.

No GPU: these call the host entry points of the C ABI only.
"""

import gzip
import os
import struct
import zlib

import numpy as np
import pytest

import oracle as O
from fluidmarch import bgeo

REF = O.ref_available()
needs_ref = pytest.mark.skipif(not REF, reason="oracle/_ref (the reference's Partio) not built")


@pytest.fixture(scope="module")
def fm(fmlib):
    return fmlib


def payloads():
    rng = np.random.default_rng(1)
    text = b"".join(b"particle %d at %f\n" % (i, v) for i, v in enumerate(rng.normal(size=3000)))
    return {
        "empty": b"",
        "one": b"x",
        "random": rng.integers(0, 256, 100_000, dtype=np.uint8).tobytes(),
        "zeros": bytes(200_000),
        "text": text,
        "floats": rng.normal(size=40_000).astype(">f4").tobytes(),
        "runs": b"".join(bytes([i % 7]) * (i % 300 + 1) for i in range(800)),
    }


def gz(data, level=6, strategy=zlib.Z_DEFAULT_STRATEGY):
    c = zlib.compressobj(level, zlib.DEFLATED, 31, 9, strategy)
    return c.compress(data) + c.flush()


@pytest.mark.parametrize("name", list(payloads()))
@pytest.mark.parametrize("level,strategy", [(0, zlib.Z_DEFAULT_STRATEGY), (1, zlib.Z_DEFAULT_STRATEGY),
                                            (6, zlib.Z_DEFAULT_STRATEGY), (9, zlib.Z_DEFAULT_STRATEGY),
                                            (6, zlib.Z_FIXED), (6, zlib.Z_HUFFMAN_ONLY), (6, zlib.Z_RLE),
                                            (6, zlib.Z_FILTERED)])
def test_gunzip_matches_zlib(fm, name, level, strategy):
    data = payloads()[name]
    assert bgeo.gunzip(gz(data, level, strategy)) == data


def test_gunzip_header_fields(fm):
    data = payloads()["text"]
    c = zlib.compressobj(6, zlib.DEFLATED, -15)
    raw = c.compress(data) + c.flush()
    trailer = struct.pack("<II", zlib.crc32(data), len(data) & 0xFFFFFFFF)
    for flg, extra in [(0, b""), (8, b"name.bgeo\0"), (16, b"a comment\0"), (4, struct.pack("<H", 5) + b"abcde"),
                       (2, b"\x12\x34"), (8 | 16 | 4 | 2, struct.pack("<H", 3) + b"xyz" + b"n\0" + b"c\0" + b"\0\0")]:
        head = bytes([0x1F, 0x8B, 8, flg, 0, 0, 0, 0, 0, 3]) + extra
        assert bgeo.gunzip(head + raw + trailer) == data, flg


def test_gunzip_first_member_only(fm):
    a, b = payloads()["text"], payloads()["floats"]
    assert bgeo.gunzip(gzip.compress(a) + gzip.compress(b)) == a


def test_gunzip_rejects_corrupt_streams(fm):
    data = payloads()["random"]
    good = gz(data)
    bad_crc = good[:-8] + bytes([good[-8] ^ 1]) + good[-7:]
    bad_len = good[:-4] + struct.pack("<I", len(data) + 1)
    for bad in (bad_crc, bad_len, good[: len(good) // 2], good[:20], b"\x1f\x8b\x07" + good[3:],
                bytes([0x1F, 0x8B, 8, 0x20]) + good[4:], b"not gzip at all", b""):
        with pytest.raises(fm.FmError):
            bgeo.gunzip(bad)
    # a block of type 3 right after the header
    with pytest.raises(fm.FmError):
        bgeo.gunzip(bytes([0x1F, 0x8B, 8, 0, 0, 0, 0, 0, 0, 3, 0x07]) + bytes(16))


def sample_xyz(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 2, (n, 3)).astype(np.float32)
    if n > 4:
        x[1, 0] = np.float32(-0.0)
        x[2, 1] = np.float32(1e-42)  # subnormal
        x[3, 2] = np.uint32(0x7FC12345).view(np.float32)  # NaN with a payload
    return x


def attrs(n, seed):
    rng = np.random.default_rng(seed)
    return {"v": ("vector", rng.normal(size=(n, 3))), "id": ("int", np.arange(n)),
            "density": ("float", rng.uniform(900, 1100, n)),
            "kind": ("indexed", rng.integers(0, 3, n), ["fluid", "spray", "foam"])}


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("compressed", [True, False])
@pytest.mark.parametrize("with_attrs", [False, True])
def test_reader_round_trip(fm, tmp_path, compressed, with_attrs):
    n = 5000
    x = sample_xyz(n, 3)
    path = str(tmp_path / "f.bgeo")
    bgeo.write(path, x, attrs(n, 4) if with_attrs else None, compressed=compressed)
    got = bgeo.read(path)
    assert np.array_equal(bits(got), bits(x))
    inf = bgeo.info(path)
    assert inf["points"] == n and inf["compressed"] == compressed
    assert inf["record_words"] == (4 + 3 + 1 + 1 + 1 if with_attrs else 4)
    assert inf["attributes"] == (4 if with_attrs else 0)
    assert inf["file_bytes"] == os.path.getsize(path)


def test_reader_empty_file_and_big_header(fm, tmp_path):
    p0 = str(tmp_path / "empty.bgeo")
    bgeo.write(p0, np.zeros((0, 3), np.float32))
    assert bgeo.read(p0).shape == (0, 3)
    # a string table of ~1.6 MB: the header-only read has to grow its prefix
    n = 100
    strings = [f"label-{i:07d}-" + "x" * 40 for i in range(30000)]
    x = sample_xyz(n, 5)
    for compressed in (True, False):
        p = str(tmp_path / f"big{int(compressed)}.bgeo")
        bgeo.write(p, x, {"tag": ("indexed", np.arange(n) % 30000, strings)}, compressed=compressed)
        assert bgeo.info(p)["points"] == n
        assert np.array_equal(bits(bgeo.read(p)), bits(x))


def test_reader_errors(fm, tmp_path):
    x = sample_xyz(100, 6)
    good = bgeo.encode(x)
    cases = {
        "magic": b"Bgeq" + good[4:],
        "json": b"\x7fNSJ" + good[4:],
        "version": good[:5] + struct.pack(">i", 4) + good[9:],
        "truncated_points": good[: len(good) - 200],
        "truncated_header": good[:30],
        # a point attribute of Houdini type 2 (string), which Partio refuses
        "string_attr": b"Bgeo" + b"V" + struct.pack(">9i", 5, 100, 0, 0, 0, 1, 0, 0, 0) + b"\x00\x01s"
                       + struct.pack(">Hi", 1, 2) + bytes(4) + bytes(100 * 20),
    }
    for name, data in cases.items():
        p = str(tmp_path / f"{name}.bgeo")
        with open(p, "wb") as f:
            f.write(data)
        with pytest.raises(fm.FmError):
            bgeo.read(p)
        with open(p + ".gz.bgeo", "wb") as f:
            f.write(gzip.compress(data))
        with pytest.raises(fm.FmError):
            bgeo.read(p + ".gz.bgeo")
    with pytest.raises(fm.FmError):
        bgeo.read(str(tmp_path / "missing.bgeo"))


def test_header_read_rejects_short_point_block(fm, tmp_path):
    """A header that claims more points than the file holds fails at the header read already, plain
    or gzip (by the gzip member's size field, exact for a small file), so a loader sizes no buffer
    from it."""
    x = sample_xyz(100, 7)
    good = bgeo.encode(x)
    for name, data in {"plain": good[:-8], "gzip": gzip.compress(good[:-8])}.items():
        p = str(tmp_path / f"short_{name}.bgeo")
        with open(p, "wb") as f:
            f.write(data)
        with pytest.raises(fm.FmError, match="truncated"):
            bgeo.info(p)
    p = str(tmp_path / "whole.bgeo")
    with open(p, "wb") as f:
        f.write(gzip.compress(good))
    assert bgeo.info(p)["points"] == 100


@needs_ref
@pytest.mark.parametrize("compressed", [True, False])
def test_reader_matches_partio(fm, oracle_lib, tmp_path, compressed):
    """Files written here, read by the reference's Partio, and files written by Partio, read here."""
    n = 7000
    x = sample_xyz(n, 7)
    mine = str(tmp_path / "mine.bgeo")
    bgeo.write(mine, x, attrs(n, 8), compressed=compressed)
    assert np.array_equal(bits(O.ref_bgeo_positions(mine)), bits(bgeo.read(mine)))
    theirs = str(tmp_path / "theirs.bgeo")
    O.ref_bgeo_write(theirs, x, compressed)
    with open(theirs, "rb") as f:
        assert (f.read(2) == b"\x1f\x8b") == compressed
    assert np.array_equal(bits(bgeo.read(theirs)), bits(x))
    assert np.array_equal(bits(O.ref_bgeo_positions(theirs)), bits(x))


def write_series(tmp_path, counts, gap_at=None):
    prefix = str(tmp_path / "ParticleData_Fluid_")
    frames = []
    for i, n in enumerate(counts, start=1):
        x = sample_xyz(n, 100 + i) * np.float32(0.5) + np.float32(0.25)
        x[:4] = np.float32(0.5)  # finite (the reference builds a grid over each frame)
        frames.append(x)
        bgeo.write(f"{prefix}{i}.bgeo", x, compressed=i % 2 == 1)
    if gap_at is not None:  # a file after a missing index is never reached
        bgeo.write(f"{prefix}{gap_at}.bgeo", frames[0])
    return prefix, frames


@pytest.mark.parametrize("threads", [0, 2])
def test_dataset_series(fm, tmp_path, threads):
    prefix, frames = write_series(tmp_path, [1200, 800, 1500, 300, 900], gap_at=7)
    ds = bgeo.Dataset(prefix, ".bgeo", -1, threads)
    assert len(ds) == 5
    assert ds.path(0).endswith("ParticleData_Fluid_1.bgeo")
    assert ds.max_particles() == 1500
    assert [ds.frame_info(i)["points"] for i in range(5)] == [1200, 800, 1500, 300, 900]
    for order in (range(5), [3, 0, 4, 1, 2, 2]):
        for i in order:
            assert np.array_equal(bits(ds.read(i)), bits(frames[i])), i
    ds.close()
    assert len(bgeo.Dataset(prefix, ".bgeo", 3, threads)) == 3
    assert len(bgeo.Dataset(prefix, ".bgeo", 0, threads)) == 0
    assert len(bgeo.Dataset(prefix + "none_", ".bgeo", -1, threads)) == 0


@needs_ref
def test_dataset_matches_reference(fm, oracle_lib, tmp_path):
    prefix, frames = write_series(tmp_path, [700, 1100, 400], gap_at=5)
    for count in (-1, 2):
        r = O.ref_dataset_load(prefix, ".bgeo", count, 0.05, sum(len(f) for f in frames))
        assert r is not None
        nf, counts, maxp, xyz = r
        ds = bgeo.Dataset(prefix, ".bgeo", count, 1)
        assert nf == len(ds)
        assert list(counts) == [ds.frame_info(i)["points"] for i in range(nf)]
        assert maxp == ds.max_particles()
        at = 0
        for i in range(nf):
            # the reference's Frame keeps the particles in its search's spatial order: compare as sets
            ref_rows = np.sort(bits(xyz[at:at + counts[i]]).view([("a", "<u4"), ("b", "<u4"), ("c", "<u4")]),
                               axis=0)
            mine = np.sort(bits(ds.read(i)).view([("a", "<u4"), ("b", "<u4"), ("c", "<u4")]), axis=0)
            assert np.array_equal(ref_rows, mine), i
            at += counts[i]
        ds.close()


def test_dataset_concurrent_readers(fm, tmp_path):
    """Several host threads reading frames of one series in random orders while the decode-ahead
    threads work: every read returns its frame's positions."""
    import threading

    counts = [900, 1300, 700, 1100, 500, 1000, 800]
    prefix, frames = write_series(tmp_path, counts)
    ds = bgeo.Dataset(prefix, ".bgeo", -1, 3)
    errors = []

    def reader(seed):
        rng = np.random.default_rng(seed)
        try:
            for i in rng.integers(0, len(counts), 40):
                got = ds.read(int(i))
                if not np.array_equal(bits(got), bits(frames[i])):
                    errors.append(int(i))
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(repr(e))

    ts = [threading.Thread(target=reader, args=(s,)) for s in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    ds.close()
    assert not errors, errors[:5]


def test_decoders_survive_corrupt_input(fm, tmp_path):
    """Random byte flips and truncations of a gzip stream and of a BGEO file end in an error or
    some output, never in a crash or a hang."""
    rng = np.random.default_rng(11)
    data = payloads()["text"][:20000]
    good = gz(data)
    for _ in range(300):
        bad = bytearray(good)
        for _ in range(int(rng.integers(1, 6))):
            bad[int(rng.integers(10, len(bad)))] = int(rng.integers(0, 256))
        if rng.random() < 0.3:
            bad = bad[: int(rng.integers(10, len(bad)))]
        try:
            bgeo.gunzip(bytes(bad))
        except fm.FmError:
            pass
    x = sample_xyz(300, 12)
    raw = bgeo.encode(x, attrs(300, 13))
    p = str(tmp_path / "fuzz.bgeo")
    for k in range(200):
        bad = bytearray(raw)
        for _ in range(int(rng.integers(1, 4))):
            bad[int(rng.integers(0, min(len(bad), 400)))] = int(rng.integers(0, 256))
        with open(p, "wb") as f:
            f.write(gzip.compress(bytes(bad)) if k % 2 else bytes(bad))
        try:
            bgeo.read(p)
        except (fm.FmError, ValueError, MemoryError):
            pass
