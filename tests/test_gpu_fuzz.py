"""Seeded random parity: clouds of random size, extent (1 m to 10 km) and kind,
cameras from far outside to inside the cloud (batches crossing the eye plane,
20/30-bit levels, w-safe and not), random fields of view, near planes and
resolutions; every batched method against the oracle, bit for bit."""
import math

import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import synth
from helpers import QUIRKS, encoded, first_diff, gpu_raw, oracle_frame
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def random_case(seed):
    rng = np.random.default_rng(1000 + seed)
    n = int(rng.integers(20_000, 120_000))
    extent = float(10 ** rng.uniform(0.0, 4.0))
    if seed % 3 == 0:
        cl = encoded(n=n, extent=extent, seed=seed, kind=L.SYNTH_TERRAIN_BOXES, num_boxes=4,
                     points_per_box=3000)
    else:
        cl = encoded(n=n, extent=extent, seed=seed)
    bmin, bmax = cl["box_min"], cl["box_max"]
    size = bmax - bmin
    target = bmin + size * rng.uniform(0.0, 1.0, 3)
    radius = float(np.linalg.norm(size)) * 10 ** rng.uniform(-3.0, 0.5)
    view = synth.orbit_view(rng.uniform(-math.pi, math.pi), rng.uniform(-1.5, 0.3), radius, target)
    w, h = int(rng.integers(16, 400)), int(rng.integers(16, 300))
    proj = synth.perspective(rng.uniform(20.0, 120.0), w / h, 10 ** rng.uniform(-3.0, 0.0), 1e6)
    return cl, (view, proj, w, h)


@pytest.mark.parametrize("seed", range(40))
def test_random_clouds_and_cameras(ctx, seed):
    cl, cam = random_case(seed)
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"],
                                  cl["box_min"])
    streams = (cl["lo"], cl["md"], cl["hi"], cl["rgba"])
    for method, payload in ((L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX),
                            (L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR),
                            (L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_COLOR)):
        fb, _ = gpu_raw(ctx, cloud, cam, method, payload)
        fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[method], payload)
        want = O.raster_batched(fr, cl["batches"], cl["n"], *streams)
        got = fb.read(L.FB_WORDS)
        assert np.array_equal(got, want), (seed, method, payload, first_diff(got, want))
        fb.close()
    fb, _ = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS_HQS)
    fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[L.METHOD_LOOP_LAS_HQS])
    depth, accum, _ = O.hqs(fr, cl["batches"], cl["n"], *streams)
    assert np.array_equal(fb.read(L.FB_DEPTH), depth), seed
    assert np.array_equal(fb.read(L.FB_ACCUM), accum), seed
    fb.close()
    cloud.close()


@pytest.mark.parametrize("seed", range(8))
def test_random_multiview_plans(ctx, seed):
    from compute_rasterizer_gb300 import default_params, make_view
    from compute_rasterizer_gb300.multiview import MultiView
    cl, _ = random_case(100 + seed)
    rng = np.random.default_rng(2000 + seed)
    bmin, bmax = cl["box_min"], cl["box_max"]
    size = bmax - bmin
    cams = []
    for _ in range(int(rng.integers(2, 13))):
        target = bmin + size * rng.uniform(0.0, 1.0, 3)
        radius = float(np.linalg.norm(size)) * 10 ** rng.uniform(-2.5, 0.5)
        view = synth.orbit_view(rng.uniform(-math.pi, math.pi), rng.uniform(-1.5, 0.3), radius,
                                target)
        w, h = int(rng.integers(16, 200)), int(rng.integers(16, 200))
        cams.append((view, synth.perspective(rng.uniform(30.0, 110.0), w / h, 0.01, 1e6), w, h))
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"],
                                  cl["box_min"])
    payload = L.PAYLOAD_COLOR if seed % 2 else L.PAYLOAD_INDEX
    params = default_params(L.METHOD_LOOP_LAS, payload=payload,
                            views_per_group=int(rng.integers(1, 9)), resolve=0, clear_after=0)
    mv = MultiView(ctx, cloud, [(c[2], c[3]) for c in cams], params)
    mv.set_views([make_view(*c) for c in cams])
    mv.clear()
    mv.render()
    ctx.sync()
    for i, cam in enumerate(cams):
        fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[L.METHOD_LOOP_LAS], payload)
        want = O.raster_batched(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
        got = mv.read(i, L.FB_WORDS)
        assert np.array_equal(got, want), (seed, i, first_diff(got, want))
    mv.close()
    cloud.close()


@pytest.mark.parametrize("seed", range(6))
def test_random_plain_frames(ctx, seed):
    from compute_rasterizer_gb300 import default_params, make_view
    rng = np.random.default_rng(3000 + seed)
    n = int(rng.integers(10_000, 200_000))
    v = synth.uniform_vertices_host(seed, n, 100.0)
    cloud = ctx.plain_cloud(v)
    eye = rng.uniform(-50.0, 250.0, 3)
    view = synth.look_at(eye, rng.uniform(0.0, 100.0, 3), [0.0, 0.0, 1.0])
    w, h = int(rng.integers(16, 300)), int(rng.integers(16, 300))
    proj = synth.perspective(rng.uniform(30.0, 110.0), w / h, 0.1, 1000.0)
    for method, variant in ((L.METHOD_EARLYZ, 0), (L.METHOD_DEDUP, 1), (L.METHOD_EARLYZ_REDUCE, 2)):
        fb = ctx.framebuffer(w, h)
        fb.clear(0xFFFFFFFFFFFFFFFF)
        ctx.render(cloud, make_view(view, proj, w, h), default_params(method, resolve=0,
                                                                       clear_after=0), fb)
        want, _, _ = O.plain(view, proj, w, h, v, variant=variant)
        got = fb.read(L.FB_WORDS)
        assert np.array_equal(got, want), (seed, method, first_diff(got, want))
        fb.close()
    cloud.close()
