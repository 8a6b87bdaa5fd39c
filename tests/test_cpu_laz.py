"""CPU tests of the LAZ reader and writer (include/cr_laz.h): the committed
fixtures whose point data LASzip wrote decode to their records and are
reproduced byte for byte by the product's writer; when the LASzip probe is
built (oracle/_ref), random formats, chunkings and records cross both ways;
partial decodes, the unchunked and interrupted-table layouts, and the error
statuses."""
import ctypes as C
import json
import struct
from pathlib import Path

import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import las
from helpers import LAZ_OFFSET, LAZ_SCALE, laszip_file, laz_box, laz_records
from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = json.loads((GOLDEN / "laz.json").read_text())["cases"]
needs_laszip = pytest.mark.skipif(not O.LAZREF.exists(), reason="LASzip probe not built (no reference tree)")


def product_laz(rec, n, fmt, bpp, chunk=L.LAZ_DEFAULT_CHUNK, var_chunk=0, threads=0):
    bmin, bmax = laz_box(rec, n, bpp)
    return las.laz_bytes(rec, n, LAZ_SCALE, LAZ_OFFSET, bmin, bmax, point_format=fmt, bytes_per_point=bpp,
                         chunk_size=chunk, var_chunk=var_chunk, threads=threads)


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_fixture_decodes_to_its_records(case):
    data = (GOLDEN / "laz" / f"{case['name']}.laz").read_bytes()
    assert O.fnv(np.frombuffer(data, np.uint8)) == case["file_fnv"]
    rec, bpp = laz_records(case["point_format"], case["points"], case["seed"], case["extra"])
    assert O.fnv(rec) == case["records_fnv"] and bpp == case["bytes_per_point"]
    f = las.LazFile(data)
    assert f.num_points == case["points"] and f.info.las.point_format == case["point_format"]
    layered = case["point_format"] >= 6
    assert f.info.chunk_size == case["chunk_size"]
    assert f.info.compressor == (L.LAZ_LAYERED_CHUNKED if layered else L.LAZ_POINTWISE_CHUNKED)
    for threads in (1, 3):
        assert np.array_equal(f.decode(threads=threads), rec)


@pytest.mark.parametrize("case", [c for c in CASES if c["point_format"] <= 3],
                         ids=[c["name"] for c in CASES if c["point_format"] <= 3])
def test_writer_reproduces_fixture_bytes(case):
    data = (GOLDEN / "laz" / f"{case['name']}.laz").read_bytes()
    rec, bpp = laz_records(case["point_format"], case["points"], case["seed"], case["extra"])
    mine = product_laz(rec, case["points"], case["point_format"], bpp, case["chunk_size"], case["var_chunk"])
    assert mine == data


@needs_laszip
@pytest.mark.parametrize("fmt", [0, 1, 2, 3])
@pytest.mark.parametrize("chunking", [(50000, 0), (777, 0), (-1, 3001), (1, 0)], ids=str)
def test_against_laszip_both_ways(fmt, chunking):
    chunk, var = chunking
    n = 9001 if chunk != 1 else 300
    rec, bpp = laz_records(fmt, n, 40 + fmt, extra=fmt % 2)
    ref = laszip_file(rec, n, fmt, bpp, chunk, var)
    assert np.array_equal(las.LazFile(ref).decode(threads=4), rec)
    assert product_laz(rec, n, fmt, bpp, chunk, var) == ref


@needs_laszip
@pytest.mark.parametrize("version", [3, 4])
@pytest.mark.parametrize("fmt", [6, 7, 8])
@pytest.mark.parametrize("chunking", [(50000, 0), (611, 0), (-1, 2711), (1, 0)], ids=str)
def test_layered_las14_against_laszip(fmt, chunking, version):
    """LAS 1.4 points through LASzip's layered coder, item versions 3 (its
    default) and 4 (its fix of the context hand-over): four scanner channels
    with switches, pulses sharing a GPS time, classes past 31, extra bytes."""
    chunk, var = chunking
    n = 9001 if chunk != 1 else 200
    rec, bpp = laz_records(fmt, n, 60 + fmt, extra=2 if fmt == 7 else 0)
    f = las.LazFile(laszip_file(rec, n, fmt, bpp, chunk, var, item_version=version))
    assert f.info.compressor == L.LAZ_LAYERED_CHUNKED and f.info.item_version[0] == version
    assert np.array_equal(f.decode(threads=4), rec)
    a, b = n // 7, n // 7 + n // 2
    assert np.array_equal(f.decode(a, b - a, threads=2), rec[a * bpp:b * bpp])


@needs_laszip
def test_layered_random_records():
    """Every byte of format-8 records random but the GPS time: every return,
    flag and channel combination, empty and full layers side by side."""
    rng = np.random.default_rng(23)
    n, fmt, bpp = 5000, 8, 40
    rec = rng.integers(0, 256, n * bpp, dtype=np.uint8)
    t = rec.reshape(n, bpp)
    t[:, 22:30] = rng.normal(4e5, 10.0, n).astype("<f8").view(np.uint8).reshape(n, 8)
    t[: n // 2, 36:38] = 7  # the NIR layer's first chunk stays empty
    f = las.LazFile(laszip_file(rec, n, fmt, bpp, 2500))
    assert np.array_equal(f.decode(), rec)


@needs_laszip
def test_unchunked_pointwise_stream():
    rec, bpp = laz_records(3, 7000, 9)
    ref = laszip_file(rec, 7000, 3, bpp, compressor=L.LAZ_POINTWISE)
    f = las.LazFile(ref)
    assert f.info.compressor == L.LAZ_POINTWISE and f.info.num_chunks == 1
    assert np.array_equal(f.decode(), rec)
    assert np.array_equal(f.decode(4000, 1234), rec[4000 * bpp:5234 * bpp])


@needs_laszip
def test_adversarial_records_cross_laszip():
    """Every byte random: all coder classes, GPS deltas beyond 32 bits, all
    return contexts; both decoders agree with the writers."""
    rng = np.random.default_rng(17)
    n, fmt, bpp = 6000, 3, 34
    rec = rng.integers(0, 256, n * bpp, dtype=np.uint8)
    t = rec.reshape(n, bpp)
    # finite GPS times avoid LASzip's undefined float-to-int cast of huge ratios
    t[:, 20:28] = rng.normal(1e5, 1e4, n).astype("<f8").view(np.uint8).reshape(n, 8)
    ref = laszip_file(rec, n, fmt, bpp, 2000)
    assert np.array_equal(las.LazFile(ref).decode(), rec)
    assert product_laz(rec, n, fmt, bpp, 2000) == ref


def test_round_trip_and_partial_decodes():
    rec, bpp = laz_records(2, 25000, 5)
    data = product_laz(rec, 25000, 2, bpp, chunk=3000)
    f = las.LazFile(data)
    assert f.info.num_chunks == 9
    for first, n in [(0, 1), (2999, 2), (3000, 3000), (100, 24900), (24999, 1), (5, 0)]:
        assert np.array_equal(f.decode(first, n, threads=2), rec[first * bpp:(first + n) * bpp])
    rng = np.random.default_rng(3)
    junk = rng.integers(0, 256, 4000 * 28, dtype=np.uint8)
    data = product_laz(junk, 4000, 1, 28, chunk=999)
    assert np.array_equal(las.LazFile(data).decode(), junk)


def test_empty_and_single_point_files():
    rec, bpp = laz_records(2, 1, 1)
    assert np.array_equal(las.LazFile(product_laz(rec, 1, 2, bpp)).decode(), rec)
    empty = las.laz_bytes(np.zeros(0, np.uint8), 0, LAZ_SCALE, LAZ_OFFSET, (0,) * 3, (1,) * 3)
    f = las.LazFile(empty)
    assert f.num_points == 0 and f.info.num_chunks == 0 and f.decode().size == 0


def test_interrupted_writer_decodes_in_order():
    """A chunk table pointer that points at itself (the writer stopped before
    writing its table): fixed-size chunks decode sequentially."""
    rec, bpp = laz_records(2, 7000, 6)
    data = bytearray(product_laz(rec, 7000, 2, bpp, chunk=2000))
    at = struct.unpack_from("<I", data, 96)[0]
    struct.pack_into("<q", data, at, at)
    f = las.LazFile(bytes(data))
    assert f.info.num_chunks == 0
    assert np.array_equal(f.decode(), rec)
    assert np.array_equal(f.decode(2500, 3000), rec[2500 * bpp:5500 * bpp])


def test_error_statuses():
    lib = L.load()
    rec, bpp = laz_records(2, 5000, 8)
    good = product_laz(rec, 5000, 2, bpp, chunk=1000)

    def status(data):
        buf = np.frombuffer(bytes(data), np.uint8)
        h, info = C.c_void_p(), L.LazInfo()
        st = lib.cr_laz_open(buf.ctypes.data, buf.size, C.byref(h), C.byref(info))
        if st == L.OK:
            out = np.zeros(5000 * bpp, np.uint8)
            st = lib.cr_laz_decode(h, 0, 5000, out.ctypes.data, 2)
            lib.cr_laz_close(h)
        return st

    assert status(good) == L.OK
    las_file = las._header(5000, LAZ_SCALE, LAZ_OFFSET, (0,) * 3, (1,) * 3, 2, bpp, (1, 2)) + rec.tobytes()
    assert status(las_file) == L.INVALID_ARG  # no LASzip VLR
    vlr_at = struct.unpack_from("<H", good, 94)[0] + 54
    bad = bytearray(good)
    struct.pack_into("<H", bad, vlr_at, 3)  # the layered compressor over point-wise items
    assert status(bad) == L.INVALID_ARG
    struct.pack_into("<H", bad, vlr_at, 4)  # no such compressor
    assert status(bad) == L.UNSUPPORTED
    bad = bytearray(good)
    struct.pack_into("<H", bad, vlr_at + 38, 1)  # POINT10 version 1
    assert status(bad) == L.UNSUPPORTED
    assert status(good[: len(good) - 40]) == L.CORRUPT  # chunk table cut
    bad = bytearray(good)
    mid = struct.unpack_from("<I", good, 96)[0] + 8 + 2000
    bad[mid:mid + 64] = bytes(64)  # a chunk's coder bytes zeroed
    assert status(bad) == L.CORRUPT
    assert lib.cr_laz_decode(None, 0, 1, None, 1) == L.INVALID_ARG
    bad = bytearray(good)
    struct.pack_into("<H", bad, vlr_at + 34, L.LAZ_ITEM_POINT14)  # a LAS 1.4 item in a point-wise stream
    struct.pack_into("<H", bad, vlr_at + 36, 30)
    struct.pack_into("<H", bad, vlr_at + 38, 3)
    assert status(bad) == L.INVALID_ARG
    vlen = C.c_int64()
    assert lib.cr_laz_vlr(6, 30, 50000, None, 0, C.byref(vlen)) == L.UNSUPPORTED
    assert lib.cr_laz_vlr(2, 20, 50000, None, 0, C.byref(vlen)) == L.INVALID_ARG


@pytest.mark.parametrize("case", ["fmt2_12k", "fmt7_extra3", "fmt8_variable"])
def test_corrupted_files_fail_cleanly(case):
    """Random byte flips and cuts anywhere in a file (header, VLR, chunk
    table, layer sizes, coder bytes): every open and decode returns a status
    or some records, never reads outside the file (the decoders and layer
    extents are clamped to it)."""
    lib = L.load()
    data = (GOLDEN / "laz" / f"{case}.laz").read_bytes()
    rng = np.random.default_rng(99)
    seen = set()
    for it in range(120):
        buf = bytearray(data)
        if it % 3 == 0:
            buf = buf[: int(rng.integers(1, len(buf)))]
        else:
            for _ in range(int(rng.integers(1, 8))):
                k = int(rng.integers(0, len(buf)))
                buf[k] = int(rng.integers(0, 256))
        arr = np.frombuffer(bytes(buf), np.uint8)
        h, info = C.c_void_p(), L.LazInfo()
        st = lib.cr_laz_open(arr.ctypes.data, arr.size, C.byref(h), C.byref(info))
        if st == L.OK:
            n = int(info.las.num_points)
            bpp = int(info.las.bytes_per_point)
            if 0 < n <= 200_000 and 0 < bpp <= 512:
                out = np.zeros(n * bpp, np.uint8)
                st = lib.cr_laz_decode(h, 0, n, out.ctypes.data, 2)
            lib.cr_laz_close(h)
        assert st in (L.OK, L.INVALID_ARG, L.UNSUPPORTED, L.CORRUPT)
        seen.add(st)
    assert L.CORRUPT in seen or L.INVALID_ARG in seen
