"""GPU parity: every framebuffer the CUDA path writes is compared bit for bit
with the oracle's (u64 depth|payload words incl. the guard tail, HQS u32
depth + u64 accumulators, resolved images), through the C ABI."""
import json
from pathlib import Path

import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import default_params, make_view, synth
from helpers import (QUIRKS, cameras, encoded, first_diff, gpu_raw, handmade_cloud, identity_cam,
                     oracle_frame)
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden.json"


@pytest.fixture(scope="module")
def small(ctx):
    cl = encoded(n=62674, extent=200.0, seed=7)
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"],
                                  cl["box_min"])
    return cl, cloud


def oracle_fb(cl, cam, method, payload):
    fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[method], payload)
    return O.raster_batched(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])


@pytest.mark.parametrize("camname", ["far", "near", "mid", "corner"])
@pytest.mark.parametrize("method,payload", [(L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX),
                                            (L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_INDEX),
                                            (L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR),
                                            (L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_COLOR)])
def test_batched_fb_and_image(ctx, small, camname, method, payload):
    cl, cloud = small
    cam = cameras(cl)[camname]
    fb, params = gpu_raw(ctx, cloud, cam, method, payload)
    got = fb.read(L.FB_WORDS)
    want = oracle_fb(cl, cam, method, payload)
    assert np.array_equal(got, want), first_diff(got, want)
    assert (got != L.DEFAULT_CLEAR).sum() > 50
    ctx.resolve(cloud, params, fb)
    img = fb.read(L.FB_IMAGE)
    w, h = cam[2], cam[3]
    ref = O.resolve_color(w, h, want) if payload else O.resolve_index(w, h, want, cl["rgba"])
    assert np.array_equal(img, ref), first_diff(img, ref)


@pytest.mark.parametrize("block", [128, 256, 512])
def test_block_sizes_agree(ctx, small, block):
    cl, cloud = small
    cam = cameras(cl)["near"]
    fb, _ = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR, block_threads=block,
                    ctas_per_sm=1)
    want = oracle_fb(cl, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR)
    assert np.array_equal(fb.read(L.FB_WORDS), want)


@pytest.mark.parametrize("camname", ["far", "near", "mid", "corner"])
def test_hqs(ctx, small, camname):
    cl, cloud = small
    cam = cameras(cl)[camname]
    fb, params = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS_HQS)
    fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[L.METHOD_LOOP_LAS_HQS])
    depth, accum, img = O.hqs(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
    gd = fb.read(L.FB_DEPTH)
    assert np.array_equal(gd, depth), first_diff(gd, depth)
    ga = fb.read(L.FB_ACCUM)
    assert np.array_equal(ga, accum), first_diff(ga, accum)
    ctx.resolve(cloud, params, fb)
    gi = fb.read(L.FB_IMAGE)
    assert np.array_equal(gi, img), first_diff(gi, img)


def config1_cam(w, h):
    view = synth.look_at([150.0, 150.0, 150.0], [50.0, 50.0, 50.0], [0.0, 0.0, 1.0])
    return view, synth.perspective(60.0, w / h, 0.1, 1000.0), w, h


@pytest.mark.parametrize("n,w,h", [(100_000, 320, 180), (4_194_304, 1920, 1080)])
def test_plain_path(ctx, n, w, h):
    v = synth.uniform_vertices_host(1, n, 100.0)
    cloud = ctx.plain_cloud(v)
    cam = config1_cam(w, h)
    fb = ctx.framebuffer(w, h)
    fb.clear(0xFFFFFFFFFFFFFFFF)
    params = default_params(L.METHOD_EARLYZ, resolve=0, clear_after=0)
    ctx.render(cloud, make_view(*cam), params, fb)
    got = fb.read(L.FB_WORDS)
    want, img, recleared = O.plain(cam[0], cam[1], w, h, v)
    assert np.array_equal(got, want), first_diff(got, want)
    params.resolve, params.clear_after = 1, 1
    ctx.resolve(cloud, params, fb)
    assert np.array_equal(fb.read(L.FB_IMAGE), img)
    assert np.array_equal(fb.read(L.FB_WORDS)[:w * h], recleared[:w * h])


def test_plain_device_generator_matches_host(ctx):
    n = 1_000_003
    cloud = synth.uniform_cloud_device(ctx, 5, n, 100.0)
    cam = config1_cam(640, 360)
    fb = ctx.framebuffer(640, 360)
    fb.clear(0xFFFFFFFFFFFFFFFF)
    ctx.render(cloud, make_view(*cam), default_params(L.METHOD_EARLYZ, resolve=0, clear_after=0), fb)
    want, _, _ = O.plain(cam[0], cam[1], 640, 360, synth.uniform_vertices_host(5, n, 100.0))
    assert np.array_equal(fb.read(L.FB_WORDS), want)


@pytest.mark.skipif(not GOLDEN.exists(), reason="no golden vectors")
def test_golden_digests(ctx):
    from golden import make_golden as G
    cases = json.loads(GOLDEN.read_text())["cases"]
    for case in cases:
        dg = case["digests"]
        if case["kind"] == "terrain":
            hdr, batches, lo, md, hi, rgba = G.terrain_inputs(case)
            assert G.dg(lo) == dg["low"] and G.dg(rgba) == dg["rgba"]
            cloud = ctx.cloud_from_arrays(batches, lo, md, hi, rgba, np.array(hdr.min[:]))
            for cname, c in case["cameras"].items():
                cam = (G.unhex(c["view"]), G.unhex(c["proj"]), c["width"], c["height"])
                for m in case["methods"]:
                    mid = {"loop_las": 0, "loop_las_prefetch": 1, "loop_las_hqs": 2}[m["method"]]
                    fb, params = gpu_raw(ctx, cloud, cam, mid, m["payload"])
                    if mid == 2:
                        assert G.dg(fb.read(L.FB_DEPTH)) == dg[f"{cname}/hqs/depth"]
                        assert G.dg(fb.read(L.FB_ACCUM)) == dg[f"{cname}/hqs/accum"]
                        ctx.resolve(cloud, params, fb)
                        assert G.dg(fb.read(L.FB_IMAGE)) == dg[f"{cname}/hqs/image"]
                        continue
                    key = f"{cname}/{m['method']}/{'color' if m['payload'] else 'index'}"
                    assert G.dg(fb.read(L.FB_WORDS)) == dg[key + "/fb"], key
                    ctx.resolve(cloud, params, fb)
                    assert G.dg(fb.read(L.FB_IMAGE)) == dg[key + "/image"], key
        else:
            v = synth.uniform_vertices_host(case["seed"], case["n"], case["size"])
            assert G.dg(v) == dg["vertices"]
            c = case["camera"]
            cloud = ctx.plain_cloud(v)
            fb = ctx.framebuffer(c["width"], c["height"])
            fb.clear(0xFFFFFFFFFFFFFFFF)
            p = default_params(L.METHOD_EARLYZ, resolve=0, clear_after=0)
            ctx.render(cloud, make_view(G.unhex(c["view"]), G.unhex(c["proj"]), c["width"],
                                        c["height"]), p, fb)
            assert G.dg(fb.read(L.FB_WORDS)) == dg["fb"], case["name"]
            p.resolve = 1
            ctx.resolve(cloud, p, fb)
            assert G.dg(fb.read(L.FB_IMAGE)) == dg["image"], case["name"]


def test_reciprocal_matches_frcp_rn_on_every_float(ctx):
    """The kernels' 1/w (hardware approximation + one Newton step, __frcp_rn
    outside [2^-126, 2^126)) equals CUDA's correctly rounded __frcp_rn for all
    2^32 bit patterns, so `xy / w` (render.cs:402) keeps the oracle's
    correctly rounded reciprocal."""
    import ctypes as C
    bad, first = C.c_uint64(), C.c_uint32()
    ctx.check(ctx.lib.cr_check_reciprocal(ctx.handle, C.byref(bad), C.byref(first)), "rcp check")
    assert bad.value == 0, hex(first.value)
    assert first.value == 0xFFFFFFFF


# ---- edge cases -------------------------------------------------------------

def run_handmade(ctx, hm, cam, method, payload=L.PAYLOAD_INDEX, quirks=None):
    cloud = ctx.cloud_from_arrays(hm["batches"], hm["lo"], hm["md"], hm["hi"], hm["rgba"],
                                  hm["box_min"])
    q = QUIRKS.get(method, 0) if quirks is None else quirks
    fb, _ = gpu_raw(ctx, cloud, cam, method, payload, quirks=q)
    fr = oracle_frame(cam, hm["box_min"][None], q, payload)
    want = O.raster_batched(fr, hm["batches"], hm["n"], hm["lo"], hm["md"], hm["hi"], hm["rgba"])
    return fb.read(L.FB_WORDS), want


def test_frustum_edge_writes_guard_row(ctx):
    s = 1.0 / 1024.0
    # x == 1 and y == 1 exactly (render.cs:404-409 keeps them): pixel W + H*W
    hm = handmade_cloud([(1023, 1023, 0), (1023, 500, 0), (0, 1023, 0)], [7, 8, 9],
                        box_min=(s, s, 0.0), box_max=(1.0 + s, 1.0 + s, 1.0))
    w, h = 64, 32
    got, want = run_handmade(ctx, hm, identity_cam(w, h), L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR)
    assert np.array_equal(got, want), first_diff(got, want)
    assert (int(got[w * h + w]) & 0xFFFFFFFF) == 7  # last guard entry


@pytest.mark.parametrize("axis", [1, 2])
@pytest.mark.parametrize("payload", [L.PAYLOAD_INDEX, L.PAYLOAD_COLOR])
def test_full_batch_with_tiny_extent(ctx, axis, payload):
    """A full 10-bit batch whose y or z extent is ~1e-33: its step scaled by
    2^-10 / 2^-20 underflows, so the batch leaves the paired decode for the
    general body; the framebuffer still matches the oracle."""
    rng = np.random.default_rng(11 + axis)
    pts = rng.integers(0, 1024, (10240, 3))
    colors = rng.integers(0, 1 << 24, 10240)
    lo, hi = [-1.0, -0.5, 0.0], [1.0, 0.5, 1.0]
    lo[axis], hi[axis] = 0.0, 1e-33
    hm = handmade_cloud(pts, colors, box_min=tuple(lo), box_max=tuple(hi))
    proj = np.eye(4)
    proj[2, 3], proj[3, 3] = 1.0, 2.0  # column-major: w = z + 2, so z reaches the depth
    cam = (np.eye(4).reshape(16), proj.reshape(16), 64, 32)
    got, want = run_handmade(ctx, hm, cam, L.METHOD_LOOP_LAS, payload)
    assert np.array_equal(got, want), first_diff(got, want)
    assert (got != L.DEFAULT_CLEAR).sum() > 20


@pytest.mark.parametrize("case", ["w_crosses_zero", "w_above_2^120"])
@pytest.mark.parametrize("method", [L.METHOD_LOOP_LAS, L.METHOD_LOOP_LAS_HQS])
def test_full_batch_outside_the_safe_w_range(ctx, case, method):
    """Full 10-bit batches whose clip w is not provably inside [2^-120, 2^120]
    (the cull's w-safe flag is clear) take the general body with the checked
    reciprocal; the result still matches the oracle."""
    rng = np.random.default_rng(21)
    pts = rng.integers(0, 1024, (10240, 3))
    colors = rng.integers(1, 1 << 24, 10240)
    if case == "w_crosses_zero":
        lo, hi = (-0.25, -0.25, -0.5), (0.25, 0.25, 0.5)
    else:
        lo, hi = (-1e36, -1e36, 2e36), (1e36, 1e36, 4e36)
    hm = handmade_cloud(pts, colors, box_min=lo, box_max=hi)
    proj = np.eye(4)
    proj[2, 3], proj[3, 3] = 1.0, 0.0  # column-major: w = z
    cam = (np.eye(4).reshape(16), proj.reshape(16), 64, 32)
    if method == L.METHOD_LOOP_LAS:
        got, want = run_handmade(ctx, hm, cam, method, L.PAYLOAD_COLOR)
        assert np.array_equal(got, want), first_diff(got, want)
        assert (got != L.DEFAULT_CLEAR).sum() > 20
        return
    cloud = ctx.cloud_from_arrays(hm["batches"], hm["lo"], hm["md"], hm["hi"], hm["rgba"],
                                  hm["box_min"])
    fb, _ = gpu_raw(ctx, cloud, cam, method)
    fr = oracle_frame(cam, hm["box_min"][None], QUIRKS[method])
    depth, accum, _ = O.hqs(fr, hm["batches"], hm["n"], hm["lo"], hm["md"], hm["hi"], hm["rgba"])
    assert np.array_equal(fb.read(L.FB_DEPTH), depth)
    assert np.array_equal(fb.read(L.FB_ACCUM), accum)


def test_full_batch_with_infinite_step(ctx):
    """A batch whose x extent overflows float (-2e38 .. 2e38): the decode step
    is infinite, so decoded x is inf or NaN; every clip coordinate then is
    inf or NaN and no point is in view, in the oracle and on the GPU alike."""
    rng = np.random.default_rng(5)
    pts = rng.integers(0, 1024, (10240, 3))
    hm = handmade_cloud(pts, rng.integers(1, 1 << 24, 10240), box_min=(-2e38, -0.5, 0.0),
                        box_max=(2e38, 0.5, 1.0))
    proj = np.eye(4)
    proj[0, 0], proj[1, 0] = 0.0, 1.0  # column-major: clip x = y
    proj[0, 3] = 1e-39  # w = 1e-39 * x + 1
    cam = (np.eye(4).reshape(16), proj.reshape(16), 64, 32)
    got, want = run_handmade(ctx, hm, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR)
    assert np.array_equal(got, want), first_diff(got, want)


@pytest.mark.parametrize("payload", [L.PAYLOAD_INDEX, L.PAYLOAD_COLOR])
def test_equal_depth_ties_take_min_payload(ctx, payload):
    pts = [(300, 300, 10)] * 40 + [(301, 300, 10)] * 3
    colors = list(range(1000, 960, -1)) + [5, 4, 6]
    hm = handmade_cloud(pts, colors)
    got, want = run_handmade(ctx, hm, identity_cam(), L.METHOD_LOOP_LAS, payload)
    assert np.array_equal(got, want)


def test_all_culled_frame(ctx, small):
    cl, cloud = small
    view = synth.look_at([-5000.0, -5000.0, 100.0], [-10000.0, -10000.0, 100.0], [0, 0, 1.0])
    cam = (view, synth.perspective(60.0, 4 / 3, 0.1, 200000.0), 320, 240)
    fb, params = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS)
    assert (fb.read(L.FB_WORDS) == L.DEFAULT_CLEAR).all()
    ctx.resolve(cloud, params, fb)
    assert (fb.read(L.FB_IMAGE) == L.BACKGROUND).all()


@pytest.mark.parametrize("pad", [1, 2, 3])
def test_unaligned_first_point_multi_file(ctx, pad):
    """Batches of a second file start at a non-multiple of 4 (LasLoaderSparse
    sparse offsets); the 128-bit loads must mask the neighbours."""
    a = encoded(n=10240 + pad, extent=60.0, seed=31)
    b = encoded(n=25000, extent=80.0, seed=32)
    n = a["n"] + b["n"]
    bb = b["batches"].copy()
    bb["first_point"] += a["n"]
    bb["file_index"] = 1
    batches = np.concatenate([a["batches"], bb])
    streams = [np.concatenate([a[k], b[k]]) for k in ("lo", "md", "hi", "rgba")]
    box = np.stack([a["box_min"], b["box_min"] + np.array([70.0, 0.0, 0.0])])
    cloud = ctx.cloud_from_arrays(batches, *streams, box)
    for camname in ("far", "near"):
        cam = cameras(b)[camname]
        for method in (L.METHOD_LOOP_LAS, L.METHOD_LOOP_LAS_PREFETCH):
            fb, _ = gpu_raw(ctx, cloud, cam, method, L.PAYLOAD_INDEX)
            fr = oracle_frame(cam, box, QUIRKS[method])
            want = O.raster_batched(fr, batches, n, *streams)
            got = fb.read(L.FB_WORDS)
            assert np.array_equal(got, want), (camname, method, first_diff(got, want))


@pytest.fixture(scope="module")
def eight_files(ctx):
    """Eight files of two full batches each, every file with its own box: full
    10-bit batches of every file index take the paired decode/projection body
    with that file's uniforms."""
    parts, batches, boxes = [], [], []
    for f in range(8):
        c = encoded(n=20480, extent=40.0, seed=40 + f)
        b = c["batches"].copy()
        b["first_point"] += f * 20480
        b["file_index"] = f
        parts.append(c)
        batches.append(b)
        boxes.append(c["box_min"] + np.array([50.0 * (f % 4), 50.0 * (f // 4), 3.0 * f]))
    batches = np.concatenate(batches)
    streams = [np.concatenate([c[k] for c in parts]) for k in ("lo", "md", "hi", "rgba")]
    box = np.stack(boxes)
    tops = np.stack([bx + (c["box_max"] - c["box_min"]) for bx, c in zip(boxes, parts)])
    cl = dict(n=8 * 20480, batches=batches, box_min=box.min(0), box_max=tops.max(0),
              streams=streams, boxes=box)
    return cl, ctx.cloud_from_arrays(batches, *streams, box)


@pytest.mark.parametrize("camname", ["far", "corner"])
@pytest.mark.parametrize("payload", [L.PAYLOAD_INDEX, L.PAYLOAD_COLOR])
def test_every_file_index_raster(ctx, eight_files, camname, payload):
    cl, cloud = eight_files
    cam = cameras(cl)[camname]
    fb, _ = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS, payload)
    fr = oracle_frame(cam, cl["boxes"], QUIRKS[L.METHOD_LOOP_LAS], payload)
    want = O.raster_batched(fr, cl["batches"], cl["n"], *cl["streams"])
    got = fb.read(L.FB_WORDS)
    assert np.array_equal(got, want), first_diff(got, want)
    if camname == "far" and payload == L.PAYLOAD_INDEX:
        idx = got[got != L.DEFAULT_CLEAR] & 0xFFFFFFFF
        assert len(np.unique(idx // 20480)) == 8  # every file wrote pixels


@pytest.mark.parametrize("camname", ["far", "corner"])
def test_every_file_index_hqs(ctx, eight_files, camname):
    cl, cloud = eight_files
    cam = cameras(cl)[camname]
    fb, params = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS_HQS)
    fr = oracle_frame(cam, cl["boxes"], QUIRKS[L.METHOD_LOOP_LAS_HQS])
    depth, accum, img = O.hqs(fr, cl["batches"], cl["n"], *cl["streams"])
    assert np.array_equal(fb.read(L.FB_DEPTH), depth)
    assert np.array_equal(fb.read(L.FB_ACCUM), accum)
    ctx.resolve(cloud, params, fb)
    assert np.array_equal(fb.read(L.FB_IMAGE), img)


def test_hqs_one_pixel_receives_a_million_points(ctx):
    nb = 98
    n = nb * 10240
    lo = np.full(n, 400 | (400 << 10) | (50 << 20), np.uint32)
    rng = np.random.default_rng(0)
    rgba = rng.integers(0, 1 << 24, n, dtype=np.uint32)
    b = np.zeros(nb, L.BATCH_DTYPE)
    b["min_x"], b["min_y"], b["min_z"] = -1.0, -1.0, 0.0
    b["max_x"], b["max_y"], b["max_z"] = 1.0, 1.0, 1.0
    b["num_points"] = 10240
    b["first_point"] = np.arange(nb) * 10240
    zeros = np.zeros(n, np.uint32)
    cloud = ctx.cloud_from_arrays(b, lo, zeros, zeros, rgba, np.zeros(3))
    cam = identity_cam(64, 32)
    fb, params = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS_HQS)
    fr = oracle_frame(cam, np.zeros((1, 3)), QUIRKS[L.METHOD_LOOP_LAS_HQS])
    depth, accum, img = O.hqs(fr, b, n, lo, zeros, zeros, rgba)
    ga = fb.read(L.FB_ACCUM)
    assert np.array_equal(ga, accum)
    assert (ga[1::2] >> 32).max() == n  # every point counted once (n, not n + 1: full batches)
    ctx.resolve(cloud, params, fb)
    assert np.array_equal(fb.read(L.FB_IMAGE), img)


def test_resolve_with_clear_restores_every_word(ctx, small):
    cl, cloud = small
    cam = cameras(cl)["corner"]
    fb = ctx.framebuffer(cam[2], cam[3])
    fb.clear()
    p = default_params(L.METHOD_LOOP_LAS)
    ctx.render(cloud, make_view(*cam), p, fb)
    ctx.sync()
    assert (fb.read(L.FB_WORDS) == L.DEFAULT_CLEAR).all()
    # the next frame starts clean: same image twice
    img1 = fb.read(L.FB_IMAGE)
    ctx.render(cloud, make_view(*cam), p, fb)
    assert np.array_equal(fb.read(L.FB_IMAGE), img1)


def test_device_flag_on_out_of_range_record(ctx):
    """A record pointing past the streams is skipped and reported (no fault)."""
    import torch
    n = 20480
    p = synth.synth_params(L.SYNTH_TERRAIN, 100.0, 3)
    rec = torch.empty(n * 26, dtype=torch.uint8, device="cuda")
    hdr = L.LasHeader()
    import ctypes as C
    lib = L.load()
    ctx.check(lib.cr_synth_points_device(ctx.handle, C.byref(p), n, rec.data_ptr(), C.byref(hdr),
                                         None), "gen")
    cloud = ctx.cloud(n, 2, 1)
    d = cloud.device_pointers()
    sc, of, mn = (np.ascontiguousarray(x[:], np.float64) for x in (hdr.scale, hdr.offset, hdr.min))
    ctx.check(lib.cr_encode_las_device(ctx.handle, rec.data_ptr(), n, 26, 2, sc.ctypes.data,
                                       of.ctypes.data, mn.ctypes.data, 1_000_000, 0, d["batches"],
                                       d["low"], d["med"], d["hig"], d["rgba"], None), "encode")
    cloud.set_files(mn)
    fb = ctx.framebuffer(64, 64)
    fb.clear()
    view = synth.orbit_view(0.5, -0.6, 150.0, mn + 50.0)
    ctx.render(cloud, make_view(view, synth.perspective(60, 1.0, 0.1, 1e5), 64, 64),
               default_params(L.METHOD_LOOP_LAS, resolve=0, clear_after=0), fb)
    with pytest.raises(Exception) as e:
        ctx.sync()
    assert getattr(e.value, "status", None) == L.DEVICE_FLAG
    assert (fb.read(L.FB_WORDS) == L.DEFAULT_CLEAR).all()
    ctx.sync()  # flag was cleared


def test_gpu_generator_sort_encoder_match_host(ctx):
    import ctypes as C

    import torch
    lib = L.load()
    n = 200_001
    p = synth.synth_params(L.SYNTH_TERRAIN_BOXES, 400.0, 17, num_boxes=4, points_per_box=5000)
    host, hh = synth.las_records_host(p, n, morton=False)
    rec = torch.empty(n * 26, dtype=torch.uint8, device="cuda")
    hd = L.LasHeader()
    ctx.check(lib.cr_synth_points_device(ctx.handle, C.byref(p), n, rec.data_ptr(), C.byref(hd),
                                         None), "gen")
    assert np.array_equal(rec.cpu().numpy(), host)
    assert list(hd.min) == list(hh.min) and list(hd.max) == list(hh.max)
    ctx.check(lib.cr_morton_sort_device(ctx.handle, rec.data_ptr(), n, 26, C.byref(hd), None), "sort")
    sorted_host, _ = synth.las_records_host(p, n, morton=True)
    assert np.array_equal(rec.cpu().numpy(), sorted_host)
    ref = synth.encode_las(sorted_host, n, hh)
    cloud = ctx.cloud(n, len(ref[0]), 1)
    d = cloud.device_pointers()
    sc, of, mn = (np.ascontiguousarray(x[:], np.float64) for x in (hd.scale, hd.offset, hd.min))
    ctx.check(lib.cr_encode_las_device(ctx.handle, rec.data_ptr(), n, 26, 2, sc.ctypes.data,
                                       of.ctypes.data, mn.ctypes.data, 0, 0, d["batches"], d["low"],
                                       d["med"], d["hig"], d["rgba"], None), "encode")
    ctx.sync()
    assert np.array_equal(cloud.read(0).view(np.uint8), ref[0].view(np.uint8)), "batches"
    for which, arr in zip((L.STREAM_LOW, L.STREAM_MED, L.STREAM_HIG, L.STREAM_RGBA), ref[1:]):
        assert np.array_equal(cloud.read(which), arr), which


def test_synth_cloud_device_pipeline(ctx):
    n = 300_000
    p = synth.synth_params(L.SYNTH_TERRAIN, 500.0, 23)
    cloud, hdr = synth.build_cloud_device(ctx, p, n)
    rec, hh = synth.las_records_host(p, n)
    cl = dict(n=n, batches=None)
    batches, lo, md, hi, rgba = synth.encode_las(rec, n, hh)
    assert list(hdr.min) == list(hh.min)
    cl.update(batches=batches, lo=lo, md=md, hi=hi, rgba=rgba, box_min=np.array(hh.min[:]),
              box_max=np.array(hh.max[:]))
    for camname in ("far", "near"):
        cam = cameras(cl)[camname]
        fb, _ = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR)
        want = oracle_fb(cl, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR)
        assert np.array_equal(fb.read(L.FB_WORDS), want), camname


@pytest.mark.parametrize("camname", ["far", "mid"])
@pytest.mark.parametrize("cut", [4, 3])
@pytest.mark.parametrize("method", [L.METHOD_LOOP_LAS, L.METHOD_LOOP_LAS_HQS])
def test_lod_skip_level(ctx, small, camname, cut, method):
    """compute_loop_nodes/render.cs:273-276: batches at precision level >= the
    cut are not rendered; the oracle applies the same cut."""
    cl, cloud = small
    cam = cameras(cl)[camname]
    fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[method], O.PAYLOAD_INDEX)
    fr.lod_skip_level = cut
    args = (cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
    fb, params = gpu_raw(ctx, cloud, cam, method, L.PAYLOAD_INDEX, lod_skip_level=cut)
    st = ctx.frame_stats(cloud, params)
    assert all(st.points_per_level[lv] == 0 for lv in range(cut, 5))
    if method == L.METHOD_LOOP_LAS_HQS:
        depth, accum, _ = O.hqs(fr, *args)
        assert np.array_equal(fb.read(L.FB_DEPTH), depth)
        assert np.array_equal(fb.read(L.FB_ACCUM), accum)
    else:
        want = O.raster_batched(fr, *args)
        got = fb.read(L.FB_WORDS)
        assert np.array_equal(got, want), first_diff(got, want)
        full = oracle_fb(cl, cam, method, L.PAYLOAD_INDEX)
        if camname == "far":
            assert not np.array_equal(want, full)  # the cut removed batches


@pytest.mark.parametrize("method,variant", [(L.METHOD_DEDUP, 1), (L.METHOD_EARLYZ_REDUCE, 2)])
@pytest.mark.parametrize("n,w,h", [(100_003, 320, 180), (4_194_304, 1920, 1080), (200_000, 64, 48)])
def test_plain_warp_variants(ctx, method, variant, n, w, h):
    """compute_2021_dedup / compute_2021_earlyz_reduce: the warp reductions
    over 32 consecutive points and the depth << 24 | color packing, bit for
    bit with the oracle (a partial last warp, the full config-1 scene, and a
    64x48 view where most of a warp lands on one pixel)."""
    v = synth.uniform_vertices_host(3, n, 100.0)
    cloud = ctx.plain_cloud(v)
    cam = config1_cam(w, h)
    fb = ctx.framebuffer(w, h)
    fb.clear(0xFFFFFFFFFFFFFFFF)
    ctx.render(cloud, make_view(*cam), default_params(method, resolve=0, clear_after=0), fb)
    got = fb.read(L.FB_WORDS)
    want, img, recleared = O.plain(cam[0], cam[1], w, h, v, variant=variant)
    assert np.array_equal(got, want), first_diff(got, want)
    early, _, _ = O.plain(cam[0], cam[1], w, h, v)
    assert not np.array_equal(want, early)  # the packing differs from early-z's
    params = default_params(method)
    ctx.resolve(cloud, params, fb)
    assert np.array_equal(fb.read(L.FB_IMAGE), img)
    assert np.array_equal(fb.read(L.FB_WORDS)[:w * h], recleared[:w * h])
    fb.close()
    cloud.close()


@pytest.mark.parametrize("loaded", [(2 * 10240 + 5, 4), (0, 0)])
@pytest.mark.parametrize("method", [L.METHOD_LOOP_LAS, L.METHOD_LOOP_LAS_PREFETCH,
                                    L.METHOD_LOOP_LAS_HQS])
def test_partially_loaded_cloud(ctx, small, method, loaded):
    """numPointsLoaded / numBatchesLoaded: with 4 records and 20,485 points
    loaded, loop_las dispatches 4 records and the methods that dispatch by
    points ceil(20485 / 10240) = 3; the oracle gets the same prefix."""
    cl, cloud = small
    points, batches = loaded
    cloud.set_loaded(points, batches)
    try:
        cam = cameras(cl)["far"]
        fb, params = gpu_raw(ctx, cloud, cam, method, L.PAYLOAD_INDEX)
        fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[method])
        args = (cl["batches"][:batches], points, cl["lo"], cl["md"], cl["hi"], cl["rgba"])
        if method == L.METHOD_LOOP_LAS_HQS:
            depth, accum, _ = O.hqs(fr, *args)
            assert np.array_equal(fb.read(L.FB_DEPTH), depth)
            assert np.array_equal(fb.read(L.FB_ACCUM), accum)
        else:
            want = O.raster_batched(fr, *args)
            got = fb.read(L.FB_WORDS)
            assert np.array_equal(got, want), first_diff(got, want)
            if points == 0:
                assert (got == L.DEFAULT_CLEAR).all()
        fb.close()
    finally:
        cloud.set_loaded(-1, -1)


def test_loaded_counts_reach_multiview_plans(ctx, small):
    """A plan (CUDA graph replay included) draws what is loaded at each frame."""
    import torch
    from compute_rasterizer_gb300.multiview import MultiView
    cl, cloud = small
    cams = [cameras(cl)[k] for k in ("far", "mid")]
    params = default_params(L.METHOD_LOOP_LAS, resolve=0, clear_after=0)
    mv = MultiView(ctx, cloud, [(c[2], c[3]) for c in cams], params)
    mv.set_views([make_view(*c) for c in cams])
    st = torch.cuda.Stream()
    try:
        for points, batches in ((-1, -1), (3 * 10240, 3), (-1, -1)):
            cloud.set_loaded(points, batches)
            mv.clear(stream=st.cuda_stream)
            mv.render(True, st.cuda_stream)
            ctx.sync(st.cuda_stream)
            for i, cam in enumerate(cams):
                fb, _ = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS)
                assert np.array_equal(mv.read(i, L.FB_WORDS), fb.read(L.FB_WORDS)), (points, i)
                fb.close()
    finally:
        cloud.set_loaded(-1, -1)
        mv.close()
