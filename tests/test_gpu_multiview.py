"""Multi-view plans: every view's framebuffer and image equal a cr_render of
that view alone, bit for bit, for every group width, block size and payload,
with and without CUDA-graph replay; the oracle agrees on sampled views."""
import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import default_params, make_view, synth
from compute_rasterizer_gb300.multiview import MultiView
from helpers import QUIRKS, camera_views, encoded, first_diff, gpu_raw, oracle_frame
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(ctx):
    cl = encoded(n=62674, extent=200.0, seed=7)
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"],
                                  cl["box_min"])
    base = camera_views(cl["box_min"], cl["box_max"], cl["batches"])
    rng = np.random.default_rng(5)
    target = (cl["box_min"] + cl["box_max"]) / 2
    views = list(base.values())
    for _ in range(7):
        views.append(synth.orbit_view(rng.uniform(-3, 3), rng.uniform(-1.3, -0.2),
                                      rng.uniform(20, 400), target + rng.uniform(-60, 60, 3)))
    sizes = [(320, 240), (64, 48), (200, 150), (96, 96), (333, 111), (128, 256), (40, 30),
             (256, 256), (150, 100), (77, 55), (300, 200)]
    cams = []
    for v, (w, h) in zip(views, sizes):
        cams.append((v, synth.perspective(60.0, w / h, 0.1, 200000.0), w, h))
    return cl, cloud, cams


def single_view(ctx, cloud, cam, method, payload):
    fb, params = gpu_raw(ctx, cloud, cam, method, payload)
    words = fb.read(L.FB_WORDS)
    ctx.resolve(cloud, params, fb)
    return words, fb.read(L.FB_IMAGE)


@pytest.mark.parametrize("group,block", [(1, 128), (3, 64), (8, 128), (8, 256), (5, 128)])
@pytest.mark.parametrize("method,payload", [(L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX),
                                            (L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_COLOR)])
def test_multiview_equals_single_views(ctx, scene, group, block, method, payload):
    cl, cloud, cams = scene
    params = default_params(method, payload=payload, views_per_group=group, block_threads=block,
                            resolve=0, clear_after=0)
    mv = MultiView(ctx, cloud, [(c[2], c[3]) for c in cams], params)
    mv.set_views([make_view(*c) for c in cams])
    mv.clear()
    mv.render()
    ctx.sync()
    words = [mv.read(i, L.FB_WORDS) for i in range(len(cams))]
    params.resolve = 1
    mv.set_params(params)
    mv.clear()
    mv.render()
    ctx.sync()
    for i, cam in enumerate(cams):
        want_w, want_img = single_view(ctx, cloud, cam, method, payload)
        assert np.array_equal(words[i], want_w), (i, first_diff(words[i], want_w))
        img = mv.read(i, L.FB_IMAGE)
        assert np.array_equal(img, want_img), (i, first_diff(img, want_img))
    mv.close()


def test_multiview_matches_oracle_on_sampled_views(ctx, scene):
    cl, cloud, cams = scene
    params = default_params(L.METHOD_LOOP_LAS, views_per_group=8, resolve=0, clear_after=0)
    mv = MultiView(ctx, cloud, [(c[2], c[3]) for c in cams], params)
    mv.set_views([make_view(*c) for c in cams])
    mv.clear()
    mv.render()
    ctx.sync()
    for i in (0, 1, 2, 5, 9):
        fr = oracle_frame(cams[i], cl["box_min"][None], QUIRKS[L.METHOD_LOOP_LAS])
        want = O.raster_batched(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
        got = mv.read(i, L.FB_WORDS)
        assert np.array_equal(got, want), (i, first_diff(got, want))
    mv.close()


def test_multiview_graph_replay_and_clear(ctx, scene):
    import torch
    cl, cloud, cams = scene
    params = default_params(L.METHOD_LOOP_LAS, payload=L.PAYLOAD_COLOR, views_per_group=4)
    mv = MultiView(ctx, cloud, [(c[2], c[3]) for c in cams], params)
    mv.set_views([make_view(*c) for c in cams])
    s = torch.cuda.Stream()
    mv.clear(stream=s.cuda_stream)
    for _ in range(3):  # capture on the first call, replay after
        mv.render(use_graph=True, stream=s.cuda_stream)
    ctx.sync(s.cuda_stream)
    for i, cam in enumerate(cams):
        _, want_img = single_view(ctx, cloud, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR)
        assert np.array_equal(mv.read(i, L.FB_IMAGE, s.cuda_stream), want_img), i
        # resolve re-cleared every word, guard tail included
        assert (mv.read(i, L.FB_WORDS, s.cuda_stream) == L.DEFAULT_CLEAR).all(), i
    # new cameras reach the captured graph through the staging copy
    mv.set_views([make_view(cams[(i + 1) % len(cams)][0], cams[i][1], cams[i][2], cams[i][3])
                  for i in range(len(cams))])
    mv.render(use_graph=True, stream=s.cuda_stream)
    ctx.sync(s.cuda_stream)
    for i in (0, 4):
        cam = (cams[(i + 1) % len(cams)][0], cams[i][1], cams[i][2], cams[i][3])
        _, want_img = single_view(ctx, cloud, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR)
        assert np.array_equal(mv.read(i, L.FB_IMAGE, s.cuda_stream), want_img), i
    mv.close()


def test_autotune_keeps_output_identical(ctx, scene):
    cl, cloud, cams = scene
    params = default_params(L.METHOD_LOOP_LAS, resolve=0, clear_after=0)
    mv = MultiView(ctx, cloud, [(c[2], c[3]) for c in cams], params)
    mv.set_views([make_view(*c) for c in cams])
    mv.clear()
    best, report = mv.autotune(frames=2)
    assert best.block_threads in (64, 128, 256) and best.views_per_group in (1, 2, 4, 8)
    assert len(report) == 12 and all(v > 0 for v in report.values())
    mv.clear()
    mv.render()
    ctx.sync()
    for i in (0, 3, 7):
        want, _ = single_view(ctx, cloud, cams[i], L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX)
        assert np.array_equal(mv.read(i, L.FB_WORDS), want), i
    mv.close()


def test_multiview_lod_cut_equals_single_views(ctx, scene):
    """The level-of-detail cut applies per view: every view equals cr_render
    of that view alone with the same cut."""
    cl, cloud, cams = scene
    params = default_params(L.METHOD_LOOP_LAS, payload=L.PAYLOAD_INDEX, views_per_group=8,
                            resolve=0, clear_after=0, lod_skip_level=3)
    mv = MultiView(ctx, cloud, [(c[2], c[3]) for c in cams], params)
    mv.set_views([make_view(*c) for c in cams])
    mv.clear()
    mv.render()
    ctx.sync()
    for i, cam in enumerate(cams):
        fb, _ = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX, lod_skip_level=3)
        want = fb.read(L.FB_WORDS)
        got = mv.read(i, L.FB_WORDS)
        assert np.array_equal(got, want), (i, first_diff(got, want))
        fb.close()
    mv.close()


def stereo_cams(cl, rng_seed=9):
    """Stereo pairs (translate(-+ipd/2) * V_head, equal sizes) of the far,
    near, mid and corner poses and of random orbits, with two decoys: a pair
    of unequal sizes and a pair with different fields of view."""
    from compute_rasterizer_gb300.workloads import eye_view
    heads = list(camera_views(cl["box_min"], cl["box_max"], cl["batches"]).values())
    rng = np.random.default_rng(rng_seed)
    target = (cl["box_min"] + cl["box_max"]) / 2
    for _ in range(3):
        heads.append(synth.orbit_view(rng.uniform(-3, 3), rng.uniform(-1.3, -0.2), rng.uniform(5, 300),
                                      target + rng.uniform(-60, 60, 3)))
    cams, paired = [], []
    for k, h in enumerate(heads):
        w, hh = [(320, 240), (160, 176), (200, 150), (96, 96), (240, 240), (128, 160), (300, 200)][k]
        proj = synth.perspective(90.0, w / hh, 0.1, 200000.0)
        for side in (-0.5, 0.5):
            cams.append((eye_view(h, -side * 0.064), proj, w, hh))
        paired += [True, False]
    # decoys: unequal sizes; unequal fields of view
    h = heads[0]
    cams.append((eye_view(h, 0.032), synth.perspective(90.0, 4 / 3, 0.1, 200000.0), 320, 240))
    cams.append((eye_view(h, -0.032), synth.perspective(90.0, 4 / 3, 0.1, 200000.0), 160, 120))
    cams.append((eye_view(h, 0.032), synth.perspective(90.0, 4 / 3, 0.1, 200000.0), 200, 150))
    cams.append((eye_view(h, -0.032), synth.perspective(70.0, 4 / 3, 0.1, 200000.0), 200, 150))
    paired += [False] * 4
    return cams, paired


def expected_pairs(paired, G):
    count = 0
    for g0 in range(0, len(paired), G):
        s = 0
        while s + 1 < G and g0 + s + 1 < len(paired):
            if paired[g0 + s]:
                count += 1
                s += 2
            else:
                s += 1
    return count


@pytest.mark.parametrize("group,block", [(8, 128), (2, 64), (3, 128), (5, 256)])
@pytest.mark.parametrize("payload", [L.PAYLOAD_INDEX, L.PAYLOAD_COLOR])
def test_stereo_pairs_share_rows_bit_exact(ctx, scene, group, block, payload):
    """Stereo eyes share y, w and 1/w: the plan finds the pairs (not the
    decoys, not across group borders) and every view still equals cr_render
    of that view alone, words and images, through graph replay too."""
    import torch
    cl, cloud, _ = scene
    cams, paired = stereo_cams(cl)
    params = default_params(L.METHOD_LOOP_LAS, payload=payload, views_per_group=group, block_threads=block)
    mv = MultiView(ctx, cloud, [(c[2], c[3]) for c in cams], params)
    mv.set_views([make_view(*c) for c in cams])
    assert mv.shared_pairs() == expected_pairs(paired, group) > 0
    s = torch.cuda.Stream()
    mv.clear(stream=s.cuda_stream)
    for _ in range(2):
        mv.render(use_graph=True, stream=s.cuda_stream)
    ctx.sync(s.cuda_stream)
    p0 = default_params(L.METHOD_LOOP_LAS, payload=payload, views_per_group=group, block_threads=block,
                        resolve=0, clear_after=0)
    mv2 = MultiView(ctx, cloud, [(c[2], c[3]) for c in cams], p0)
    mv2.set_views([make_view(*c) for c in cams])
    mv2.clear()
    mv2.render()
    ctx.sync()
    for i, cam in enumerate(cams):
        want_w, want_img = single_view(ctx, cloud, cam, L.METHOD_LOOP_LAS, payload)
        got = mv2.read(i, L.FB_WORDS)
        assert np.array_equal(got, want_w), (i, first_diff(got, want_w))
        assert np.array_equal(mv.read(i, L.FB_IMAGE, s.cuda_stream), want_img), i
    mv.close()
    mv2.close()


def test_stereo_pairs_many_files_and_oracle(ctx):
    """A 300-file cloud (file records computed on the GPU): shared pairs stay
    bit-exact, against single views and against the oracle."""
    from compute_rasterizer_gb300.workloads import eye_view
    from helpers import many_file_cameras, many_file_cloud
    cl = many_file_cloud()
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"], cl["box_min"])
    cams = []
    for cam in list(many_file_cameras(cl).values())[:3]:
        for side in (-0.5, 0.5):
            cams.append((eye_view(cam[0], -side * 0.064), cam[1], cam[2], cam[3]))
    params = default_params(L.METHOD_LOOP_LAS, views_per_group=8, resolve=0, clear_after=0)
    mv = MultiView(ctx, cloud, [(c[2], c[3]) for c in cams], params)
    mv.set_views([make_view(*c) for c in cams])
    assert mv.shared_pairs() == 3
    mv.clear()
    mv.render()
    ctx.sync()
    for i, cam in enumerate(cams):
        want, _ = single_view(ctx, cloud, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX)
        got = mv.read(i, L.FB_WORDS)
        assert np.array_equal(got, want), (i, first_diff(got, want))
        if i in (0, 3):
            fr = oracle_frame(cam, cl["box_min"], QUIRKS[L.METHOD_LOOP_LAS])
            ref = O.raster_batched(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
            assert np.array_equal(got, ref), (i, first_diff(got, ref))
    mv.close()
    cloud.close()
