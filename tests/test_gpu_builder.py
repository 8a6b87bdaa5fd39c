"""The GPU layout builder against the host one on inputs chosen to stress its
exact shortcuts: the batch AABB taken from the integer extremes, and the
30-bit quantisation that multiplies by the AABB's reciprocal except where an
integer is within reach (LasLoaderSparse.cpp:84-199)."""
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


@pytest.mark.parametrize("case", ["pow2", "random", "negative_scale", "flat"])
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
    else:  # zero extent on one axis (0 / 0 quantises to 0) and duplicates
        xyz = rng.integers(0, 1000, size=(n, 3))
        xyz[:, 2] = 7
    rgb = rng.integers(0, 65536, size=(n, 3))
    rec = records(xyz, rgb)
    hdr = L.LasHeader()
    hdr.scale[:], hdr.offset[:] = list(scale), list(offset)
    bmin = np.array([-3.5, 12.25, 0.0])
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
