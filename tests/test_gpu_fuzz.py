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
