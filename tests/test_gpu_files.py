"""Clouds of many files, the loop_las_prefetch uvec4 addressing (H6) and the
2021 methods' tiled resolve, against the oracle bit for bit.

The reference binds one 256 B record per LAS file (compute_loop_las.h:100,
168-199) and every batch names its file (render.cs:22-49), so a tiled dataset
of hundreds of files renders in one frame.  Here the first 8 files' uniforms
travel in kernel parameters and every file's record is computed on the GPU
when there are more; these tests render a 300-file cloud (each file two batch
records, its own boxMin, first points on every value of firstPoint % 4)
through every path that takes a cloud: cr_render (loop_las both payloads,
loop_las_prefetch, HQS), a multi-view plan, the frame server, the
no-allocation entry point, and a cloud loaded from several LAS files."""
import ctypes as C

import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import default_params, make_view, synth
from compute_rasterizer_gb300.multiview import MultiView
from compute_rasterizer_gb300.serve import Server
from helpers import (QUIRKS, first_diff, gpu_raw, identity_cam, many_file_cameras, many_file_cloud,
                     oracle_frame, pixel_grid_cloud)
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NFILES = 300


@pytest.fixture(scope="module")
def tiled(ctx):
    cl = many_file_cloud(NFILES)
    assert len(cl["batches"]) == 2 * NFILES
    assert {s % 4 for s in np.cumsum([0] + cl["sizes"][:-1])} == {0, 1, 2, 3}
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"],
                                  cl["box_min"])
    cams = many_file_cameras(cl)
    yield cl, cloud, cams
    cloud.close()


def oracle_words(cl, cam, method, payload):
    fr = oracle_frame(cam, cl["box_min"], QUIRKS[method], payload)
    return O.raster_batched(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"],
                            threads=8)


def files_seen(cl, words):
    """Files whose points won a pixel (index payload)."""
    starts = np.cumsum([0] + cl["sizes"][:-1])
    idx = (words & np.uint64(0xFFFFFFFF)).astype(np.int64)
    depth = (words >> np.uint64(32)).astype(np.uint32).view(np.float32)
    idx = idx[(depth > 0) & (depth < 1e6)]
    return set(np.searchsorted(starts, idx, side="right") - 1)


@pytest.mark.parametrize("camname", ["far", "mid", "near"])
@pytest.mark.parametrize("method,payload", [(L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX),
                                            (L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR),
                                            (L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_INDEX)])
def test_many_files_raster(ctx, tiled, camname, method, payload):
    cl, cloud, cams = tiled
    cam = cams[camname]
    fb, params = gpu_raw(ctx, cloud, cam, method, payload)
    got = fb.read(L.FB_WORDS)
    want = oracle_words(cl, cam, method, payload)
    assert np.array_equal(got, want), first_diff(got, want)
    assert (got != L.DEFAULT_CLEAR).sum() > 500
    st = ctx.frame_stats(cloud, params)
    if camname == "far":
        if payload == L.PAYLOAD_INDEX:
            assert len(files_seen(cl, got)) > 100
    else:
        assert st.points_per_level[0] + st.points_per_level[1] > 0  # 20/30-bit batches
    ctx.resolve(cloud, params, fb)
    img = O.resolve_color(cam[2], cam[3], want) if payload else \
        O.resolve_index(cam[2], cam[3], want, cl["rgba"])
    assert np.array_equal(fb.read(L.FB_IMAGE), img)
    fb.close()


@pytest.mark.parametrize("camname", ["far", "mid"])
def test_many_files_hqs(ctx, tiled, camname):
    cl, cloud, cams = tiled
    cam = cams[camname]
    fb, params = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS_HQS)
    fr = oracle_frame(cam, cl["box_min"], QUIRKS[L.METHOD_LOOP_LAS_HQS])
    depth, accum, img = O.hqs(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
    assert np.array_equal(fb.read(L.FB_DEPTH), depth)
    assert np.array_equal(fb.read(L.FB_ACCUM), accum)
    ctx.resolve(cloud, params, fb)
    assert np.array_equal(fb.read(L.FB_IMAGE), img)
    assert (accum != 0).sum() > 500
    fb.close()


@pytest.mark.parametrize("method", [L.METHOD_LOOP_LAS, L.METHOD_LOOP_LAS_PREFETCH])
def test_many_files_multiview(ctx, tiled, method):
    cl, cloud, cams = tiled
    names = ["far", "mid", "near", "far"]
    sizes = [(cams[k][2], cams[k][3]) for k in names]
    sizes[3] = (200, 120)
    views = [cams[k] for k in names]
    views[3] = (cams["far"][0], synth.perspective(60.0, 200 / 120, 0.1, 200000.0), 200, 120)
    params = default_params(method, payload=L.PAYLOAD_INDEX, resolve=0, clear_after=0)
    import torch
    mv = MultiView(ctx, cloud, sizes, params)
    mv.set_views([make_view(*v) for v in views])
    want = [oracle_words(cl, v, method, L.PAYLOAD_INDEX) for v in views]
    s = torch.cuda.Stream()
    for frame in range(3):  # plain enqueue, then a graph captured and replayed
        mv.clear(stream=s.cuda_stream)
        mv.render(use_graph=frame > 0, stream=s.cuda_stream)
        ctx.sync(s.cuda_stream)
        for i in range(len(views)):
            got = mv.read(i, L.FB_WORDS, s.cuda_stream)
            assert np.array_equal(got, want[i]), (frame, i, first_diff(got, want[i]))
    mv.close()


def test_many_files_server(ctx, tiled):
    cl, cloud, cams = tiled
    views = [cams["far"], cams["mid"], cams["near"]]
    for plain in (False, True):
        srv = Server(ctx, pool_bytes=64 << 20, max_batch_views=8, max_inflight=2,
                     plain_launches=plain, payload=L.PAYLOAD_COLOR)
        cid = srv.add_cloud(cloud)
        images = [np.zeros(v[2] * v[3], np.uint32) for v in views]
        for i, v in enumerate(views):
            srv.submit(Server.request(cid, make_view(*v), images[i], user_tag=i))
        srv.drain(120000)
        done = srv.poll(max_n=8)
        assert len(done) == len(views) and all(c.status == L.OK for c in done)
        for i, v in enumerate(views):
            want = O.resolve_color(v[2], v[3], oracle_words(cl, v, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR))
            assert np.array_equal(images[i], want), (plain, i, first_diff(images[i], want))
        srv.close()


def test_many_files_las_ingest(ctx, tmp_path):
    """Twelve LAS files (a tiled terrain) loaded into one cloud equal the host
    layout builder's encoding of the same files, and render as the oracle."""
    from compute_rasterizer_gb300 import las
    from helpers import terrain_las
    from test_gpu_las import host_layout
    n_files, per = 12, 14001
    _, rec, hdr = terrain_las(n_files * per, 1500.0, 31)
    rec2 = rec.reshape(-1, L.LAS_FORMAT2_BYTES)
    scale, offset = np.array(hdr.scale[:]), np.array(hdr.offset[:])
    paths, files = [], []
    for i in range(n_files):
        chunk = np.ascontiguousarray(rec2[i * per:(i + 1) * per]).reshape(-1)
        xyz = chunk.reshape(per, -1)[:, :12].copy().view("<i4").reshape(-1, 3) * scale + offset
        path = las.write_las(tmp_path / f"tile_{i:02d}.las", chunk, per, scale, offset,
                             xyz.min(0), xyz.max(0))
        paths.append(path)
        files.append((chunk, las.read_info(path)))
    cloud, infos = las.load_files(ctx, paths)
    batches, lo, md, hi, rgba = host_layout(files)
    assert np.array_equal(cloud.read(0).view(np.uint8), batches.view(np.uint8))
    for which, w in zip((L.STREAM_LOW, L.STREAM_MED, L.STREAM_HIG, L.STREAM_RGBA), (lo, md, hi, rgba)):
        assert np.array_equal(cloud.read(which), w), which
    box = np.array([i.min[:] for i in infos])
    top = np.array([i.max[:] for i in infos]).max(0)
    yaw, pitch, radius, target = synth.zoom_to_cloud(box.min(0), top)
    cam = (synth.orbit_view(yaw, pitch, radius, target), synth.perspective(60.0, 1.5, 0.1, 2e5),
           300, 200)
    fb, _ = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS)
    want = O.raster_batched(oracle_frame(cam, box, QUIRKS[L.METHOD_LOOP_LAS]), batches,
                            n_files * per, lo, md, hi, rgba)
    assert np.array_equal(fb.read(L.FB_WORDS), want)
    assert (want != L.DEFAULT_CLEAR).sum() > 500
    fb.close()
    cloud.close()


def test_many_files_noalloc(ctx, tiled):
    """cr_render_batched_noalloc with 300 files (its records in the fixed array)."""
    lib = L.load()
    cl, cloud, cams = tiled
    d = cloud.device_pointers()
    box = np.ascontiguousarray(cl["box_min"], np.float64)
    for camname in ("far", "mid"):
        cam = cams[camname]
        want = oracle_words(cl, cam, L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_INDEX)
        out = ctx.framebuffer(cam[2], cam[3])
        out.clear()
        params = default_params(L.METHOD_LOOP_LAS_PREFETCH, resolve=0, clear_after=0)
        st = lib.cr_render_batched_noalloc(d["batches"], cloud.nb, cloud.n, d["low"], d["med"],
                                           d["hig"], d["rgba"], cloud.n + 64, box.ctypes.data,
                                           NFILES, C.byref(make_view(*cam)), C.byref(params),
                                           out.device_pointer(L.FB_WORDS), None)
        assert st == L.OK
        ctx.sync()
        got = out.read(L.FB_WORDS)
        assert np.array_equal(got, want), (camname, first_diff(got, want))
        out.close()


# ---- H6: loop_las_prefetch's uvec4 addressing --------------------------------

H6_FIRSTS = [1, 10242, 20483, 26484]  # firstPoint % 4 = 1, 2, 3, 0
H6_COUNTS = [10240, 10240, 6000, 1000]


@pytest.mark.parametrize("quirks", [L.QUIRKS_METHOD_DEFAULT, 0, L.QUIRK_UVEC4_BASE])
@pytest.mark.parametrize("block", [128, 256])
def test_uvec4_base_single_view(ctx, quirks, block):
    """Each point lands on its own pixel, so the index payload shows which
    points were visited: with the method's default the reference's thread-0
    drop and tail gap (las2/render.cs:319-341), with quirks 0 every point."""
    cl = pixel_grid_cloud(H6_FIRSTS, H6_COUNTS, 27490)
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"][:cl["n"]], cl["md"][:cl["n"]],
                                  cl["hi"][:cl["n"]], cl["rgba"][:cl["n"]], cl["box_min"])
    cam = identity_cam(1024, 32)
    fb, _ = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS_PREFETCH, quirks=quirks, culling=0,
                    block_threads=block)
    q = QUIRKS[L.METHOD_LOOP_LAS_PREFETCH] if quirks == L.QUIRKS_METHOD_DEFAULT else quirks
    fr = oracle_frame(cam, cl["box_min"], q, culling=0)
    want = O.raster_batched(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
    got = fb.read(L.FB_WORDS)
    assert np.array_equal(got, want), first_diff(got, want)
    # the default drops points: fewer pixels than the corrected behaviour
    dropped = int((want == L.DEFAULT_CLEAR).sum())
    if q & L.QUIRK_UVEC4_BASE:
        assert dropped > 60
    fb.close()
    cloud.close()


def test_uvec4_base_multiview(ctx):
    cl = pixel_grid_cloud(H6_FIRSTS, H6_COUNTS, 27490)
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"][:cl["n"]], cl["md"][:cl["n"]],
                                  cl["hi"][:cl["n"]], cl["rgba"][:cl["n"]], cl["box_min"])
    cam = identity_cam(1024, 32)
    for quirks in (L.QUIRKS_METHOD_DEFAULT, 0):
        params = default_params(L.METHOD_LOOP_LAS_PREFETCH, quirks=quirks, frustum_culling=0,
                                resolve=0, clear_after=0)
        mv = MultiView(ctx, cloud, [(1024, 32), (1024, 32)], params)
        mv.set_views([make_view(*cam), make_view(*cam)])
        mv.clear()
        mv.render()
        ctx.sync()
        q = QUIRKS[L.METHOD_LOOP_LAS_PREFETCH] if quirks == L.QUIRKS_METHOD_DEFAULT else quirks
        want = O.raster_batched(oracle_frame(cam, cl["box_min"], q, culling=0), cl["batches"],
                                cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
        for i in range(2):
            assert np.array_equal(mv.read(i, L.FB_WORDS), want), (quirks, i)
        mv.close()
    cloud.close()


# ---- the 2021 methods' tiled resolve ------------------------------------------

@pytest.mark.parametrize("method,variant", [(L.METHOD_EARLYZ, 0), (L.METHOD_DEDUP, 1),
                                            (L.METHOD_EARLYZ_REDUCE, 2)])
def test_plain_tiles_two_frames_1080p(ctx, method, variant):
    """Config 1 at 1920x1080 over two consecutive frames with the method's
    defaults: rows 1072-1079 are never resolved or re-cleared
    (compute_2021_earlyz.h:161-163), so their framebuffer words carry the
    first frame's points into the second and their image words stay 0."""
    from test_gpu_parity import config1_cam
    n, w, h = 4_194_304, 1920, 1080
    v1 = synth.uniform_vertices_host(1, n, 100.0)
    v2 = synth.uniform_vertices_host(2, n, 100.0)
    cam = config1_cam(w, h)
    fb = ctx.framebuffer(w, h)
    fb.clear(0xFFFFFFFFFFFFFFFF)
    want_fb, want_img = None, None
    for v in (v1, v2):
        cloud = ctx.plain_cloud(v)
        ctx.render(cloud, make_view(*cam), default_params(method), fb)
        ctx.sync()
        _, want_img, want_fb = O.plain(cam[0], cam[1], w, h, v, variant=variant, fb=want_fb,
                                       image=want_img)
        assert np.array_equal(fb.read(L.FB_WORDS), want_fb)
        assert np.array_equal(fb.read(L.FB_IMAGE), want_img)
        cloud.close()
    rows = want_img.reshape(h, w)[1072:]
    assert (rows == 0).all()
    tail = want_fb[:w * h].reshape(h, w)[1072:]
    assert (tail != np.uint64(0xFFFFFFFFFF3C321E)).any()
    # with quirks 0 every pixel is resolved and re-cleared
    fb.clear(0xFFFFFFFFFFFFFFFF)
    cloud = ctx.plain_cloud(v1)
    ctx.render(cloud, make_view(*cam), default_params(method, quirks=0), fb)
    ctx.sync()
    _, img0, fb0 = O.plain(cam[0], cam[1], w, h, v1, variant=variant, quirks=0)
    assert np.array_equal(fb.read(L.FB_WORDS), fb0)
    assert np.array_equal(fb.read(L.FB_IMAGE), img0)
    assert (img0.reshape(h, w)[1072:] != 0).any()
    fb.close()
    cloud.close()
