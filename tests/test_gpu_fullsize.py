"""Parity at the benchmark sizes: whole framebuffers of the CUDA path against
the oracle, bit for bit, on the full workloads -- the 1B-point terrain at
1920x1080 (loop_las with both payloads, loop_las_prefetch, HQS), the
100M-point terrain from all five flight poses at 2560x1440 and with HQS, the
1B frame and the five poses with CR_QUIRK_LITERAL_ARITH, and every view of the 64-view multi-view frame against its single-view render.
The clouds are generated on the GPU (the generator is bit-identical to the
host one) and read back for the oracle, which runs on all host cores."""
import os

import numpy as np
import pytest

import compute_rasterizer_gb300 as cr
from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import synth, workloads
from compute_rasterizer_gb300.multiview import MultiView
from helpers import QUIRKS, first_diff, gpu_raw, oracle_frame
from oracle import oracle as O

pytestmark = pytest.mark.gpu

THREADS = max(1, os.cpu_count() or 1)


def read_back(ctx, cloud):
    """Batch records and the four streams, each stream with the device's
    zeroed padding words, as the oracle reads them."""
    lib = L.load()
    n = cloud.n
    out = [cloud.read(0)]
    for which in (L.STREAM_LOW, L.STREAM_MED, L.STREAM_HIG, L.STREAM_RGBA):
        a = np.zeros(n + 64, np.uint32)
        ctx.check(lib.cr_cloud_read(ctx.handle, cloud.handle, which, a.ctypes.data, n * 4, None),
                  "stream read")
        out.append(a)
    ctx.sync()
    return out


def build(ctx, params, n):
    cloud, hdr = synth.build_cloud_device(ctx, params, n)
    return cloud, np.array(hdr.min[:]), np.array(hdr.max[:])


@pytest.fixture(scope="module")
def terrain_1b(ctx):
    cloud, bmin, bmax = build(ctx, synth.synth_params(L.SYNTH_TERRAIN, 10_000.0, 1), 1_000_000_000)
    yield cloud, bmin, bmax, read_back(ctx, cloud)
    cloud.close()


@pytest.mark.parametrize("method,payload", [(L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR),
                                            (L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX),
                                            (L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_COLOR)])
def test_terrain_1b_1080p(ctx, terrain_1b, method, payload):
    cloud, bmin, bmax, host = terrain_1b
    cam = workloads.terrain_frame(bmin, bmax, 1920, 1080)
    fb, params = gpu_raw(ctx, cloud, cam, method, payload)
    got = fb.read(L.FB_WORDS)
    fr = oracle_frame(cam, bmin[None], QUIRKS[method], payload)
    want = O.raster_batched(fr, host[0], cloud.n, *host[1:], threads=THREADS)
    assert np.array_equal(got, want), first_diff(got, want)
    ctx.resolve(cloud, params, fb)
    img = fb.read(L.FB_IMAGE)
    ref = (O.resolve_color(1920, 1080, want) if payload == L.PAYLOAD_COLOR
           else O.resolve_index(1920, 1080, want, host[4][:cloud.n]))
    assert np.array_equal(img, ref), first_diff(img, ref)
    assert (img != L.BACKGROUND).mean() > 0.3
    fb.close()


def test_terrain_1b_hqs(ctx, terrain_1b):
    cloud, bmin, bmax, host = terrain_1b
    cam = workloads.terrain_frame(bmin, bmax, 1920, 1080)
    fb, params = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS_HQS)
    fr = oracle_frame(cam, bmin[None], QUIRKS[L.METHOD_LOOP_LAS_HQS])
    depth, accum, img = O.hqs(fr, host[0], cloud.n, *host[1:])
    gd = fb.read(L.FB_DEPTH)
    assert np.array_equal(gd, depth), first_diff(gd, depth)
    ga = fb.read(L.FB_ACCUM)
    assert np.array_equal(ga, accum), first_diff(ga, accum)
    ctx.resolve(cloud, params, fb)
    assert np.array_equal(fb.read(L.FB_IMAGE), img)
    fb.close()


def test_terrain_1b_literal(ctx, terrain_1b):
    """CR_QUIRK_LITERAL_ARITH on the full frame, where nearly every batch takes
    the literal pair body (pair products, scalar sums, two-step division)."""
    cloud, bmin, bmax, host = terrain_1b
    cam = workloads.terrain_frame(bmin, bmax, 1920, 1080)
    m = L.METHOD_LOOP_LAS
    fb, _ = gpu_raw(ctx, cloud, cam, m, L.PAYLOAD_COLOR, quirks=QUIRKS[m] | L.QUIRK_LITERAL_ARITH)
    got = fb.read(L.FB_WORDS)
    with O.arith(O.ARITH_LITERAL):
        fr = oracle_frame(cam, bmin[None], QUIRKS[m], L.PAYLOAD_COLOR)
        want = O.raster_batched(fr, host[0], cloud.n, *host[1:], threads=THREADS)
    assert np.array_equal(got, want), first_diff(got, want)
    fb.close()


@pytest.fixture(scope="module")
def terrain_100m(ctx):
    cloud, bmin, bmax = build(ctx, synth.synth_params(L.SYNTH_TERRAIN, 1000.0, 2), 100_000_000)
    yield cloud, bmin, bmax, read_back(ctx, cloud)
    cloud.close()


def test_flight_path_100m_1440p(ctx, terrain_100m):
    cloud, bmin, bmax, host = terrain_100m
    levels = np.zeros(5, np.int64)
    for cam in workloads.flight_path(bmin, bmax):
        fb, params = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR)
        got = fb.read(L.FB_WORDS)
        fr = oracle_frame(cam, bmin[None], QUIRKS[L.METHOD_LOOP_LAS], L.PAYLOAD_COLOR)
        want = O.raster_batched(fr, host[0], cloud.n, *host[1:], threads=THREADS)
        assert np.array_equal(got, want), first_diff(got, want)
        levels += np.array(ctx.frame_stats(cloud, params).points_per_level[:])
        fb.close()
    assert levels[1] > 0 and levels[2:].sum() > 0  # 20-bit and 10-bit batches both drawn


def test_flight_path_100m_literal(ctx, terrain_100m):
    """The five flight poses and HQS from the first, with CR_QUIRK_LITERAL_ARITH."""
    cloud, bmin, bmax, host = terrain_100m
    poses = workloads.flight_path(bmin, bmax)
    m = L.METHOD_LOOP_LAS
    for cam in poses:
        fb, _ = gpu_raw(ctx, cloud, cam, m, L.PAYLOAD_INDEX, quirks=QUIRKS[m] | L.QUIRK_LITERAL_ARITH)
        got = fb.read(L.FB_WORDS)
        with O.arith(O.ARITH_LITERAL):
            fr = oracle_frame(cam, bmin[None], QUIRKS[m], L.PAYLOAD_INDEX)
            want = O.raster_batched(fr, host[0], cloud.n, *host[1:], threads=THREADS)
        assert np.array_equal(got, want), first_diff(got, want)
        fb.close()
    h = L.METHOD_LOOP_LAS_HQS
    fb, _ = gpu_raw(ctx, cloud, poses[0], h, quirks=QUIRKS[h] | L.QUIRK_LITERAL_ARITH)
    with O.arith(O.ARITH_LITERAL):
        fr = oracle_frame(poses[0], bmin[None], QUIRKS[h])
        depth, accum, _ = O.hqs(fr, host[0], cloud.n, *host[1:])
    gd, ga = fb.read(L.FB_DEPTH), fb.read(L.FB_ACCUM)
    assert np.array_equal(gd, depth), first_diff(gd, depth)
    assert np.array_equal(ga, accum), first_diff(ga, accum)
    fb.close()


def test_hqs_100m(ctx, terrain_100m):
    cloud, bmin, bmax, host = terrain_100m
    cam = workloads.flight_path(bmin, bmax)[0]
    fb, params = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS_HQS)
    fr = oracle_frame(cam, bmin[None], QUIRKS[L.METHOD_LOOP_LAS_HQS])
    depth, accum, img = O.hqs(fr, host[0], cloud.n, *host[1:])
    gd = fb.read(L.FB_DEPTH)
    assert np.array_equal(gd, depth), first_diff(gd, depth)
    ga = fb.read(L.FB_ACCUM)
    assert np.array_equal(ga, accum), first_diff(ga, accum)
    ctx.resolve(cloud, params, fb)
    assert np.array_equal(fb.read(L.FB_IMAGE), img)
    fb.close()


def test_multiview_64_full(ctx):
    """The 64-view frame of the multi-view benchmark (200M points): every view's
    framebuffer equals that view rendered alone."""
    cloud, bmin, bmax = build(ctx, workloads.multiview_cloud_params(), 200_000_000)
    cams = workloads.multiview_64(bmin, bmax)
    params = cr.default_params(L.METHOD_LOOP_LAS, payload=L.PAYLOAD_COLOR, resolve=0, clear_after=0)
    mv = MultiView(ctx, cloud, [(c[2], c[3]) for c in cams], params)
    mv.set_views([cr.make_view(*c) for c in cams])
    mv.clear()
    mv.render(True)
    ctx.sync()
    for i, cam in enumerate(cams):
        fb, _ = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR)
        want = fb.read(L.FB_WORDS)
        got = mv.read(i, L.FB_WORDS)
        assert np.array_equal(got, want), (i, first_diff(got, want))
        fb.close()
    mv.close()
    cloud.close()
