"""The GPU layout builder against the host one on inputs chosen to stress its
exact shortcuts: the batch AABB taken from the integer extremes, and the
30-bit quantisation evaluated in integer fixed point where its error bound
decides the cell, by the reciprocal or the division elsewhere
(LasLoaderSparse.cpp:84-199); the GPU Morton keys against the host sort
(Sort_Frugal/src/main.cpp:82-105).  The host paths evaluate the double chain
itself."""
import ctypes as C

import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import synth

pytestmark = pytest.mark.gpu


def records(xyz, rgb):
    n = len(xyz)
    rec = np.zeros((n, L.LAS_FORMAT2_BYTES), np.uint8)
    rec[:, :12] = np.ascontiguousarray(xyz, "<i4").view(np.uint8).reshape(n, 12)
    rec[:, 20:26] = np.ascontiguousarray(rgb, "<u2").view(np.uint8).reshape(n, 6)
    return rec.reshape(-1)


def georeferenced(rng, n, spans):
    """Integer coordinates of a UTM-like survey: batches of 10,240 points
    within per-batch spans (in scale units) around a moving base, so batch
    extents run from centimetres to kilometres at 1 mm resolution."""
    nb = n // 10240 + 1
    base = rng.integers(0, 2 * 10 ** 8, size=(nb, 3))
    span = rng.choice(spans, size=(nb, 3))
    xyz = np.repeat(base, 10240, axis=0)[:n] + (rng.random((n, 3)) * np.repeat(span, 10240, axis=0)[:n])
    return xyz.astype(np.int64)


@pytest.mark.parametrize("case", ["pow2", "random", "negative_scale", "flat", "utm", "utm_tiny_scale"])
def test_device_encoder_matches_host_on_boundaries(ctx, case):
    import torch
    rng = np.random.default_rng(3)
    n = 409_600 + 77
    scale = np.array([0.001, 0.01, 0.25])
    offset = np.array([1000.0, -50.0, 3.0])
    if case == "pow2":
        # exact coordinates and per batch extents of 2^k steps: (v - min) /
        # size * 2^30 is an integer for every point, so every point takes the
        # division (no integer may sit within the fast path's margin)
        scale, offset = np.array([0.25, 0.5, 2.0]), np.array([1000.0, -50.0, 3.0])
        k = rng.integers(1, 30, size=(n // 10240 + 1, 3))
        xyz = rng.integers(0, 2 ** 30, size=(n, 3)) % (2 ** np.repeat(k, 10240, axis=0)[:n])
        xyz[::10240] = 0
        xyz[5::10240] = 2 ** np.repeat(k, 10240, axis=0)[:n][5::10240]
    elif case == "random":
        xyz = rng.integers(-2 ** 31, 2 ** 31 - 1, size=(n, 3))
    elif case == "negative_scale":
        scale = -scale
        xyz = rng.integers(-10 ** 6, 10 ** 6, size=(n, 3))
    elif case == "flat":  # zero extent on one axis (0 / 0 quantises to 0) and duplicates
        xyz = rng.integers(0, 1000, size=(n, 3))
        xyz[:, 2] = 7
    elif case == "utm":
        # easting / northing offsets: the double chain's own rounding is
        # comparable to a 30-bit cell of the small batches, whose points take
        # the double chain; the wide ones take the integer form
        scale, offset = np.array([0.001, 0.001, 0.001]), np.array([500000.0, 5000000.0, 0.0])
        xyz = georeferenced(rng, n, [10, 10 ** 3, 10 ** 4, 10 ** 6, 10 ** 8])
    else:  # 0.1 um steps and a kilometre-scale offset, spans up to 2^31 steps
        scale, offset = np.array([1e-7, 1e-7, 1e-7]), np.array([1e6, -2e6, 123.456])
        xyz = georeferenced(rng, n, [100, 10 ** 5, 10 ** 7, 2 * 10 ** 9])
        xyz = np.clip(xyz - 10 ** 8, -2 ** 31, 2 ** 31 - 1)
    rgb = rng.integers(0, 65536, size=(n, 3))
    rec = records(xyz, rgb)
    hdr = L.LasHeader()
    hdr.scale[:], hdr.offset[:] = list(scale), list(offset)
    bmin = np.array([-3.5, 12.25, 0.0])
    if case.startswith("utm"):
        # the file's boxMin: its smallest coordinate on each axis
        bmin = (xyz.min(axis=0) * scale + offset)
    want = synth.encode_las(rec, n, hdr, box_min=bmin)
    lib = L.load()
    cloud = ctx.cloud(n, len(want[0]), 1)
    d = cloud.device_pointers()
    dev = torch.from_numpy(rec).cuda()
    sc, of, mn = (np.ascontiguousarray(x, np.float64) for x in (scale, offset, bmin))
    ctx.check(lib.cr_encode_las_device(ctx.handle, dev.data_ptr(), n, 26, 2, sc.ctypes.data,
                                       of.ctypes.data, mn.ctypes.data, 0, 0, d["batches"], d["low"],
                                       d["med"], d["hig"], d["rgba"], None), "encode")
    ctx.sync()
    assert np.array_equal(cloud.read(0).view(np.uint8), want[0].view(np.uint8)), "batches"
    for which, arr in zip((L.STREAM_LOW, L.STREAM_MED, L.STREAM_HIG, L.STREAM_RGBA), want[1:]):
        got = cloud.read(which)
        assert np.array_equal(got, arr), (which, int(np.argmax(got != arr)))
    cloud.close()


def test_gather_tail_and_odd_counts(ctx):
    """The Morton sort's warp-staged gather on counts that leave a partial
    warp, against the host sort."""
    import torch
    lib = L.load()
    for n in (33, 1000, 65_537):
        p = synth.synth_params(L.SYNTH_TERRAIN, 300.0, 5 + n)
        host, hh = synth.las_records_host(p, n, morton=False)
        rec = torch.from_numpy(host.copy()).cuda()
        ctx.check(lib.cr_morton_sort_device(ctx.handle, rec.data_ptr(), n, 26, C.byref(hh), None),
                  "sort")
        sorted_host, _ = synth.las_records_host(p, n, morton=True)
        assert np.array_equal(rec.cpu().numpy(), sorted_host), n


@pytest.mark.parametrize("case", ["utm", "utm_header_wider", "tiny_scale"])
def test_device_morton_keys_match_host_georeferenced(ctx, case):
    """GPU Morton sort (integer keys where the bound decides) == host sort
    (the double chain) for georeferenced headers: UTM offsets at 1 mm, a
    header box wider than the points, 0.1 um steps."""
    import torch
    rng = np.random.default_rng(11)
    n = 300_001
    scale, offset = np.array([0.001] * 3), np.array([500000.0, 5000000.0, 0.0])
    xyz = georeferenced(rng, n, [10, 10 ** 4, 10 ** 6])
    if case == "tiny_scale":
        scale, offset = np.array([1e-7] * 3), np.array([1e6, -2e6, 123.456])
        xyz = np.clip(georeferenced(rng, n, [100, 10 ** 7]) - 10 ** 8, -2 ** 31, 2 ** 31 - 1)
    rgb = rng.integers(0, 65536, size=(n, 3))
    rec = records(xyz, rgb)
    hdr = L.LasHeader()
    hdr.num_points, hdr.point_format, hdr.bytes_per_point = n, 2, 26
    hdr.scale[:], hdr.offset[:] = list(scale), list(offset)
    lo, hi = xyz.min(axis=0) * scale + offset, xyz.max(axis=0) * scale + offset
    if case == "utm_header_wider":
        lo, hi = lo - 37.25, hi + 1000.0
    hdr.min[:], hdr.max[:] = list(lo), list(hi)
    lib = L.load()
    dev = torch.from_numpy(rec.copy()).cuda()
    ctx.check(lib.cr_morton_sort_device(ctx.handle, dev.data_ptr(), n, 26, C.byref(hdr), None), "sort")
    host = rec.copy()
    assert lib.cr_morton_sort_host(host.ctypes.data, n, 26, C.byref(hdr)) == L.OK
    got = dev.cpu().numpy()
    assert np.array_equal(got, host), int(np.argmax(got != host))
