"""Frame server: every served image equals a render of that view alone, bit
for bit, whether the request shared a multi-view launch with others (batched
arm) or was rendered by itself (plain arm); admission refuses what cannot fit
and memory pressure limits batches without losing requests."""
import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import default_params, make_view, synth
from compute_rasterizer_gb300.serve import Server, latency_summary, request_bytes
from helpers import encoded, first_diff, gpu_raw

pytestmark = pytest.mark.gpu

SIZES = [(64, 48), (128, 96), (200, 150), (320, 240), (333, 111), (96, 96)]


@pytest.fixture(scope="module")
def scenes(ctx):
    specs = [(62674, 200.0, 7), (150001, 300.0, 8), (30001, 100.0, 9)]
    clouds, boxes = [], []
    for n, extent, seed in specs:
        cl = encoded(n=n, extent=extent, seed=seed)
        clouds.append(ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"],
                                            cl["rgba"], cl["box_min"]))
        boxes.append((cl["box_min"], cl["box_max"]))
    rng = np.random.default_rng(11)
    reqs = []
    for i in range(40):
        c = int(rng.choice(3, p=[0.5, 0.3, 0.2]))
        bmin, bmax = boxes[c]
        target = (bmin + bmax) / 2 + rng.uniform(-20, 20, 3)
        view = synth.orbit_view(rng.uniform(-3, 3), rng.uniform(-1.3, -0.2),
                                rng.uniform(30, 400), target)
        w, h = SIZES[int(rng.integers(len(SIZES)))]
        reqs.append((c, (view, synth.perspective(60.0, w / h, 0.1, 200000.0), w, h)))
    return clouds, reqs


_solo_cache = {}


def solo_image(ctx, cloud, cam, payload, key):
    if (key, payload) not in _solo_cache:
        fb, params = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS, payload)
        ctx.resolve(cloud, params, fb)
        _solo_cache[(key, payload)] = fb.read(L.FB_IMAGE)
        fb.close()
    return _solo_cache[(key, payload)]


def serve_all(srv, ids, reqs):
    images = [np.zeros(cam[2] * cam[3], np.uint32) for _, cam in reqs]
    for i, (c, cam) in enumerate(reqs):
        srv.submit(Server.request(ids[c], make_view(*cam), images[i], user_tag=i))
    srv.drain(120000)
    done = srv.poll(max_n=len(reqs) + 8)
    return images, done


@pytest.mark.parametrize("plain", [False, True])
@pytest.mark.parametrize("payload", [L.PAYLOAD_COLOR, L.PAYLOAD_INDEX])
def test_served_images_equal_solo_renders(ctx, scenes, plain, payload):
    clouds, reqs = scenes
    srv = Server(ctx, pool_bytes=64 << 20, max_batch_views=16, max_inflight=2,
                 plain_launches=plain, payload=payload)
    ids = [srv.add_cloud(c) for c in clouds]
    images, done = serve_all(srv, ids, reqs)
    assert len(done) == len(reqs)
    assert all(c.status == L.OK for c in done), [c.status for c in done]
    assert sorted(c.user_tag for c in done) == list(range(len(reqs)))
    views = [c.batch_views for c in done]
    if plain:
        assert max(views) == 1
    else:
        assert max(views) > 1  # the burst was batched
    for i, (c, cam) in enumerate(reqs):
        want = solo_image(ctx, clouds[c], cam, payload, i)
        assert np.array_equal(images[i], want), (i, plain, first_diff(images[i], want))
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["rejected"] == 0
    assert st["pool_used_bytes"] == 0
    srv.close()


def test_same_request_alone_and_in_a_mix(ctx, scenes):
    """One view served alone, then inside a burst of 39 others: same image."""
    clouds, reqs = scenes
    srv = Server(ctx, pool_bytes=64 << 20, max_batch_views=64)
    ids = [srv.add_cloud(c) for c in clouds]
    c0, cam0 = reqs[3]
    alone = np.zeros(cam0[2] * cam0[3], np.uint32)
    srv.submit(Server.request(ids[c0], make_view(*cam0), alone))
    srv.drain(60000)
    (first,) = srv.poll()
    assert first.status == L.OK and first.batch_views == 1
    images, done = serve_all(srv, ids, reqs)
    mixed = [c for c in done if c.user_tag == 3][0]
    assert mixed.batch_views > 1
    assert np.array_equal(alone, images[3])
    srv.close()


def test_admission_refuses_what_cannot_fit(ctx, scenes):
    clouds, _ = scenes
    pool = 1 << 20
    srv = Server(ctx, pool_bytes=pool)
    cid = srv.add_cloud(clouds[0])
    bmin = np.zeros(3)
    big = make_view(synth.orbit_view(0.5, -0.6, 300.0, bmin),
                    synth.perspective(60.0, 1.0, 0.1, 200000.0), 512, 512)
    assert request_bytes(512, 512) > pool
    st, _ = srv.try_submit(Server.request(cid, big))
    assert st == L.ADMISSION_REJECTED
    st, _ = srv.try_submit(Server.request(cid + 7, big))
    assert st == L.INVALID_ARG
    small = make_view(synth.orbit_view(0.5, -0.6, 300.0, bmin),
                      synth.perspective(60.0, 64 / 48, 0.1, 200000.0), 64, 48)
    srv.submit(Server.request(cid, small))
    srv.drain(60000)
    (c,) = srv.poll()
    assert c.status == L.OK
    s = srv.stats()
    assert s["rejected"] == 1 and s["completed"] == 1
    srv.close()


def test_queue_bound_rejects_and_accepted_requests_finish(ctx, scenes):
    clouds, reqs = scenes
    srv = Server(ctx, pool_bytes=64 << 20, max_queued=2, max_inflight=1)
    ids = [srv.add_cloud(c) for c in clouds]
    accepted, refused = [], 0
    images = {}
    for i, (c, cam) in enumerate(reqs):
        img = np.zeros(cam[2] * cam[3], np.uint32)
        st, _ = srv.try_submit(Server.request(ids[c], make_view(*cam), img, user_tag=i))
        if st == L.OK:
            accepted.append(i)
            images[i] = img
        else:
            assert st == L.ADMISSION_REJECTED
            refused += 1
    srv.drain(120000)
    done = srv.poll(max_n=64)
    assert sorted(c.user_tag for c in done) == accepted
    assert all(c.status == L.OK for c in done)
    s = srv.stats()
    assert s["rejected"] == refused and s["completed"] == len(accepted)
    for i in accepted:
        c, cam = reqs[i]
        assert np.array_equal(images[i], solo_image(ctx, clouds[c], cam, L.PAYLOAD_COLOR, i))
    srv.close()


def test_memory_pressure_limits_batches(ctx, scenes):
    clouds, reqs = scenes
    per = request_bytes(320, 240)
    srv = Server(ctx, pool_bytes=2 * per + 4096, max_batch_views=64)
    cid = srv.add_cloud(clouds[1])
    rng = np.random.default_rng(3)
    cams = []
    for _ in range(12):
        view = synth.orbit_view(rng.uniform(-3, 3), rng.uniform(-1.2, -0.3), rng.uniform(50, 400),
                                np.zeros(3))
        cams.append((view, synth.perspective(60.0, 320 / 240, 0.1, 200000.0), 320, 240))
    images, done = serve_all(srv, [cid], [(0, cam) for cam in cams])
    assert len(done) == 12 and all(c.status == L.OK for c in done)
    s = srv.stats()
    assert s["max_views_in_launch"] <= 2
    assert s["pool_peak_bytes"] <= s["pool_bytes"]
    for i, cam in enumerate(cams):
        assert np.array_equal(images[i], solo_image(ctx, clouds[1], cam, L.PAYLOAD_COLOR, 1000 + i))
    srv.close()


def test_replay_reports_ordered_times(ctx, scenes):
    clouds, reqs = scenes
    srv = Server(ctx, pool_bytes=64 << 20)
    ids = [srv.add_cloud(c) for c in clouds]
    requests = [Server.request(ids[c], make_view(*cam), user_tag=i) for i, (c, cam) in enumerate(reqs)]
    arrival = np.arange(len(reqs), dtype=np.float64) * 500.0  # 2000 req/s
    done = srv.replay(requests, arrival)
    assert (done["status"] == L.OK).all()
    assert (done["user_tag"] == np.arange(len(reqs))).all()
    assert (done["t_launch_us"] >= done["t_arrival_us"]).all()
    assert (done["t_done_us"] >= done["t_launch_us"]).all()
    d = np.diff(done["t_arrival_us"])
    assert np.allclose(d, 500.0)
    summ = latency_summary(done)
    assert summ["completed"] == len(reqs) and summ["p99_ms"] >= summ["p50_ms"] > 0
    srv.close()


def test_close_finishes_outstanding_requests(ctx, scenes):
    clouds, reqs = scenes
    srv = Server(ctx, pool_bytes=64 << 20, max_batch_views=8)
    ids = [srv.add_cloud(c) for c in clouds]
    images = []
    for i, (c, cam) in enumerate(reqs[:16]):
        img = np.zeros(cam[2] * cam[3], np.uint32)
        images.append(img)
        srv.submit(Server.request(ids[c], make_view(*cam), img, user_tag=i))
    srv.close()  # returns after every accepted request completed
    for i, (c, cam) in enumerate(reqs[:16]):
        assert np.array_equal(images[i], solo_image(ctx, clouds[c], cam, L.PAYLOAD_COLOR, i))


def test_injected_launch_failure_does_not_wedge_the_loop(ctx, scenes):
    """A launch whose (host-simulated) allocation fails completes its requests
    with OUT_OF_MEMORY; the other requests and every later launch are served."""
    clouds, reqs = scenes
    srv = Server(ctx, pool_bytes=64 << 20, max_batch_views=64, max_inflight=1)
    ids = [srv.add_cloud(c) for c in clouds]
    srv.inject(L.INJECT_LAUNCH_ALLOC, 1)
    images, done = serve_all(srv, ids, reqs)
    failed = [c for c in done if c.status != L.OK]
    assert len(done) == len(reqs) and failed
    assert all(c.status == L.OUT_OF_MEMORY for c in failed)
    assert len({c.t_launch_us for c in failed}) == 1  # one launch failed
    for c in done:
        if c.status == L.OK:
            i = c.user_tag
            want = solo_image(ctx, clouds[reqs[i][0]], reqs[i][1], L.PAYLOAD_COLOR, i)
            assert np.array_equal(images[i], want)
    images, done = serve_all(srv, ids, reqs)
    assert all(c.status == L.OK for c in done)
    s = srv.stats()
    assert s["failed"] == len(failed) and s["pool_used_bytes"] == 0
    srv.close()


def test_server_draws_the_loaded_part(ctx, scenes):
    """The server reads a cloud's loaded counts at every launch."""
    clouds, reqs = scenes
    srv = Server(ctx, pool_bytes=64 << 20)
    ids = [srv.add_cloud(c) for c in clouds]
    c0, cam0 = [r for r in reqs if r[0] == 1][0]
    cloud = clouds[c0]
    try:
        for points, batches in ((5 * 10240, 5), (-1, -1)):
            cloud.set_loaded(points, batches)
            img = np.zeros(cam0[2] * cam0[3], np.uint32)
            srv.submit(Server.request(ids[c0], make_view(*cam0), img))
            srv.drain(60000)
            (done,) = srv.poll()
            assert done.status == L.OK
            fb, params = gpu_raw(ctx, cloud, cam0, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR)
            ctx.resolve(cloud, params, fb)
            assert np.array_equal(img, fb.read(L.FB_IMAGE)), points
            fb.close()
    finally:
        cloud.set_loaded(-1, -1)
        srv.close()
