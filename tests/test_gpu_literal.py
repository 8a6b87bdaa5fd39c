"""CR_QUIRK_LITERAL_ARITH: the kernels evaluate the shader math as the GLSL
source writes it, and every framebuffer equals the oracle's literal
arithmetic mode bit for bit -- the mode that tests/test_cpu_shader_pin.py
pins to the reference's own shaders compiled as C++.  The batched methods
(both payloads, the prefetch addressing over files on every firstPoint % 4,
more than 8 files), HQS, the three 2021 plain methods, and loop_nodes, on
fixed and randomized clouds and cameras, and with every clip w beyond the
literal pair body's range; the multi-view plans and the server refuse the
quirk."""
import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import default_params, make_view, synth
from helpers import (QUIRKS, cameras, encoded, first_diff, gpu_raw, many_file_cameras,
                     many_file_cloud, oracle_frame)
from oracle import oracle as O

pytestmark = pytest.mark.gpu
LIT = L.QUIRK_LITERAL_ARITH


@pytest.fixture(scope="module")
def small(ctx):
    cl = encoded(n=62674, extent=200.0, seed=7)
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"],
                                  cl["box_min"])
    return cl, cloud


@pytest.mark.parametrize("camname", ["far", "near", "mid", "corner"])
@pytest.mark.parametrize("method,payload", [(L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX),
                                            (L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR),
                                            (L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_INDEX)])
def test_batched_literal(ctx, small, camname, method, payload):
    cl, cloud = small
    cam = cameras(cl)[camname]
    fb, _ = gpu_raw(ctx, cloud, cam, method, payload, quirks=QUIRKS[method] | LIT)
    got = fb.read(L.FB_WORDS)
    with O.arith(O.ARITH_LITERAL):
        fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[method], payload)
        want = O.raster_batched(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
    assert np.array_equal(got, want), first_diff(got, want)
    # the default contract differs (FMA and reciprocal) on the same frame
    fb2, _ = gpu_raw(ctx, cloud, cam, method, payload)
    assert not np.array_equal(fb2.read(L.FB_WORDS), got)
    fb.close()
    fb2.close()


@pytest.mark.parametrize("nfiles", [24, 300])
def test_batched_literal_many_files(ctx, nfiles):
    """Per-file records with the literal planes (host for the first 8 files,
    the GPU beyond), and loop_las_prefetch's uvec4 addressing over files on
    every firstPoint % 4."""
    cl = many_file_cloud(nfiles=nfiles, base=10241, spread=900)
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"],
                                  cl["box_min"])
    for camname, cam in many_file_cameras(cl).items():
        for method in (L.METHOD_LOOP_LAS, L.METHOD_LOOP_LAS_PREFETCH):
            fb, _ = gpu_raw(ctx, cloud, cam, method, quirks=QUIRKS[method] | LIT)
            got = fb.read(L.FB_WORDS)
            with O.arith(O.ARITH_LITERAL):
                fr = oracle_frame(cam, cl["box_min"], QUIRKS[method])
                want = O.raster_batched(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"],
                                        cl["rgba"])
            assert np.array_equal(got, want), (camname, method, first_diff(got, want))
            fb.close()
    cloud.close()


@pytest.mark.parametrize("camname", ["far", "near", "mid"])
def test_hqs_literal(ctx, small, camname):
    cl, cloud = small
    cam = cameras(cl)[camname]
    m = L.METHOD_LOOP_LAS_HQS
    fb, _ = gpu_raw(ctx, cloud, cam, m, quirks=QUIRKS[m] | LIT)
    with O.arith(O.ARITH_LITERAL):
        fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[m])
        depth, accum, _ = O.hqs(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
    assert np.array_equal(fb.read(L.FB_DEPTH), depth)
    assert np.array_equal(fb.read(L.FB_ACCUM), accum)
    fb.close()


@pytest.mark.parametrize("method,variant", [(L.METHOD_EARLYZ, 0), (L.METHOD_DEDUP, 1),
                                            (L.METHOD_EARLYZ_REDUCE, 2)])
def test_plain_literal(ctx, method, variant):
    n, w, h = 1_000_000, 1920, 1080
    v = synth.uniform_vertices_host(1, n, 100.0)
    cloud = ctx.plain_cloud(v)
    view = synth.look_at([150.0, 150.0, 150.0], [50.0, 50.0, 50.0], [0.0, 0.0, 1.0])
    proj = synth.perspective(60.0, w / h, 0.1, 1000.0)
    fb = ctx.framebuffer(w, h)
    fb.clear(0xFFFFFFFFFFFFFFFF)
    params = default_params(method, resolve=0, clear_after=0,
                            quirks=L.QUIRK_RESOLVE_TILES | LIT)
    ctx.render(cloud, make_view(view, proj, w, h), params, fb)
    got = fb.read(L.FB_WORDS)
    with O.arith(O.ARITH_LITERAL):
        want, _, _ = O.plain(view, proj, w, h, v, variant=variant)
    assert np.array_equal(got, want), first_diff(got, want)
    fb.close()
    cloud.close()


def test_loop_nodes_literal(ctx, tmp_path):
    from compute_rasterizer_gb300 import potree
    from helpers import camera_views, terrain_las
    n = 800_000
    _, rec, hdr = terrain_las(n, 400.0, 3)
    potree.write_octree(tmp_path, rec, n, hdr.scale[:], hdr.offset[:], hdr.min[:], hdr.max[:],
                        max_leaf=20000, chunk_levels=2)
    o = potree.open_octree(tmp_path)
    cloud = o.load(ctx)
    enc = o.encode()
    extent = np.array(hdr.max[:]) - np.array(hdr.min[:])
    proj = synth.perspective(60.0, 400 / 250, 0.1, 200000.0)
    node_quirks = O.NODE_LOOP | O.LEVEL4_80PX | O.ONE_WORLD
    for camname, view in camera_views(np.zeros(3), extent, enc[0]).items():
        cam = (view, proj, 400, 250)
        fb, params = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_NODES,
                             quirks=node_quirks | L.QUIRK_FLOAT_UNIFORMS | L.QUIRK_RESOLVE_TILES | LIT,
                             lod_skip_level=4)
        got = fb.read(L.FB_WORDS)
        with O.arith(O.ARITH_LITERAL):
            fr = O.make_frame(view, proj, 400, 250, np.zeros((1, 3)), culling=1, quirks=node_quirks,
                              payload=O.PAYLOAD_INDEX, lod_skip_level=4, float_uniforms=True)
            want = O.raster_batched(fr, enc[0], n, *enc[1:])
        assert np.array_equal(got, want), (camname, first_diff(got, want))
        fb.close()
    cloud.close()
    o.close()


@pytest.mark.parametrize("scale", [2.0 ** 70, 2.0 ** -80])
def test_literal_w_beyond_pair_range(ctx, small, scale):
    """The projection scaled by 2^70 or 2^-80: every clip w lies outside
    [2^-64, 2^64], where the literal pair body's division holds, and inside
    [2^-120, 2^120], so the literal raster takes the scalar body while the
    contract keeps its pairs.  Both equal their oracle modes."""
    cl, cloud = small
    m = L.METHOD_LOOP_LAS
    for camname in ("far", "mid", "near"):
        view, proj, w, h = cameras(cl)[camname]
        cam = (view, proj * scale, w, h)
        for quirks, arith in ((QUIRKS[m], O.ARITH_CONTRACT), (QUIRKS[m] | LIT, O.ARITH_LITERAL)):
            fb, _ = gpu_raw(ctx, cloud, cam, m, L.PAYLOAD_COLOR, quirks=quirks)
            got = fb.read(L.FB_WORDS)
            with O.arith(arith):
                fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[m], L.PAYLOAD_COLOR)
                want = O.raster_batched(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"],
                                        cl["rgba"])
            assert np.array_equal(got, want), (camname, scale, arith, first_diff(got, want))
            fb.close()
            hi = (want[: w * h] >> np.uint64(32)).astype(np.uint32)
            depth = hi[hi != 0xFF800000].view(np.float32)
            assert depth.size > 1000
            e = np.log2(depth)
            assert (e.min() > 64 or e.max() < -64) and e.min() > -120 and e.max() < 120


@pytest.mark.parametrize("seed", range(16))
def test_random_clouds_literal(ctx, seed):
    """The randomized clouds and cameras of test_gpu_fuzz.py (extents 1 m to
    10 km, eyes outside and inside the cloud, batches crossing the eye plane)
    with CR_QUIRK_LITERAL_ARITH: both batched loops and HQS."""
    from test_gpu_fuzz import random_case
    cl, cam = random_case(300 + seed)
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"],
                                  cl["box_min"])
    streams = (cl["lo"], cl["md"], cl["hi"], cl["rgba"])
    for method, payload in ((L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR),
                            (L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_INDEX)):
        fb, _ = gpu_raw(ctx, cloud, cam, method, payload, quirks=QUIRKS[method] | LIT)
        got = fb.read(L.FB_WORDS)
        with O.arith(O.ARITH_LITERAL):
            fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[method], payload)
            want = O.raster_batched(fr, cl["batches"], cl["n"], *streams)
        assert np.array_equal(got, want), (seed, method, payload, first_diff(got, want))
        fb.close()
    h = L.METHOD_LOOP_LAS_HQS
    fb, _ = gpu_raw(ctx, cloud, cam, h, quirks=QUIRKS[h] | LIT)
    with O.arith(O.ARITH_LITERAL):
        fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[h])
        depth, accum, _ = O.hqs(fr, cl["batches"], cl["n"], *streams)
    assert np.array_equal(fb.read(L.FB_DEPTH), depth), seed
    assert np.array_equal(fb.read(L.FB_ACCUM), accum), seed
    fb.close()
    cloud.close()


def test_multiview_and_server_refuse_literal(ctx, small):
    from compute_rasterizer_gb300.multiview import MultiView
    from compute_rasterizer_gb300._lib import CRError
    from compute_rasterizer_gb300.serve import Server
    cl, cloud = small
    params = default_params(L.METHOD_LOOP_LAS, quirks=QUIRKS[L.METHOD_LOOP_LAS] | LIT)
    with pytest.raises(CRError) as e:
        MultiView(ctx, cloud, [(64, 64)], params)
    assert e.value.status == L.UNSUPPORTED
    with pytest.raises(CRError) as e:
        Server(ctx, pool_bytes=1 << 26, quirks=QUIRKS[L.METHOD_LOOP_LAS] | LIT)
    assert e.value.status == L.UNSUPPORTED
