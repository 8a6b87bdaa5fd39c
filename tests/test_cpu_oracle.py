"""CPU tests: the oracle pinned to the reference's glm matrix code, the product's
host builders checked against the oracle, quirk semantics, and golden vectors."""
import ctypes as C
import json
import math
from pathlib import Path

import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import synth
from helpers import QUIRKS, cameras, encoded, handmade_cloud, identity_cam, oracle_frame
from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden.json"


def _p(a):
    return a.ctypes.data


def test_unorm_roundtrip_exact():
    c = np.arange(256, dtype=np.float32)
    r = (np.float32(255.0) * (c / np.float32(255.0))).astype(np.float32)
    assert np.array_equal(r.astype(np.uint32), np.arange(256))


@pytest.mark.skipif(not O.GLMREF.exists(), reason="reference glm probe not built (no reference tree)")
def test_matrices_match_reference_glm():
    g = O.glmref()
    o = O.lib()
    lib = L.load()
    rng = np.random.default_rng(3)
    for _ in range(300):
        yaw, pitch = rng.uniform(-3, 3), rng.uniform(-1.5, 1.5)
        radius = rng.uniform(10, 20000)
        tgt = np.ascontiguousarray(rng.uniform(-1e4, 1e4, 3))
        W, H = int(rng.integers(64, 4000)), int(rng.integers(64, 4000))
        wg = np.zeros(16)
        g.glmref_orbit_world(yaw, pitch, radius, _p(tgt), _p(wg))
        wo = np.zeros(16)
        o.or_orbit_world(yaw, pitch, radius, _p(tgt), _p(wo))
        assert np.array_equal(wg, wo)
        vg, pg = np.zeros(16), np.zeros(16)
        g.glmref_camera(60.0, W, H, 0.1, 200000.0, _p(wg), _p(vg), _p(pg))
        po = np.zeros(16)
        o.or_perspective(math.pi * 60.0 / 180.0, W / H, 0.1, 200000.0, _p(po))
        assert np.array_equal(po, pg)
        # product host code: perspective + orbit view
        pp = synth.perspective(60.0, W / H, 0.1, 200000.0)
        assert np.array_equal(pp, pg)
        vp = synth.orbit_view(yaw, pitch, radius, tgt)
        assert np.array_equal(vp.astype(np.float32), vg.astype(np.float32))
        # per-file float uniforms (compute_loop_las.h:166-200)
        bm = np.ascontiguousarray(rng.uniform(-1e5, 1e5, 3))
        tf, wf, vwf, pf = (np.zeros(16, np.float32) for _ in range(4))
        g.glmref_file_record(_p(vg), _p(pg), _p(bm), _p(tf), _p(wf), _p(vwf), _p(pf))
        ff = O.FileFrame()
        o.or_file_setup(_p(vg), _p(pg), _p(bm), C.byref(ff))
        assert np.array_equal(np.frombuffer(ff.transform, np.float32), tf)
        assert np.array_equal(np.frombuffer(ff.view_world, np.float32), vwf)
        a, b = np.zeros(16, np.float32), np.zeros(16, np.float32)
        g.glmref_plain_transform(_p(vg), _p(pg), _p(a))
        o.or_plain_transform(_p(vg), _p(pg), _p(b))
        assert np.array_equal(a, b)
        eye = np.ascontiguousarray(rng.uniform(-500, 500, 3))
        ce = np.ascontiguousarray(rng.uniform(-50, 50, 3))
        up = np.array([0.0, 0.0, 1.0])
        la, lb = np.zeros(16), np.zeros(16)
        g.glmref_look_at(_p(eye), _p(ce), _p(up), _p(la))
        o.or_look_at(_p(eye), _p(ce), _p(up), _p(lb))
        assert np.array_equal(la, lb)
        assert np.array_equal(synth.look_at(eye, ce, up), la)


@pytest.mark.parametrize("n", [1, 10239, 10240, 10241, 33333])
def test_host_encoder_matches_oracle(n):
    rec, hdr = synth.las_records_host(synth.synth_params(L.SYNTH_TERRAIN, 300.0, n), n)
    ours = synth.encode_las(rec, n, hdr, sparse_offset=5, file_index=0)
    ref = O.encode_las(rec, n, 26, 2, hdr.scale[:], hdr.offset[:], hdr.min[:], sparse_offset=5)
    for a, b in zip(ours, ref):
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    b = ours[0]
    assert b["num_points"].sum() == n
    assert (b["first_point"] == 5 + 10240 * np.arange(len(b))).all()
    # decode at 30 bit stays inside the float AABB's quantisation grid
    assert (ours[1] >> 30 == 0).all() and (ours[2] >> 30 == 0).all()


def test_encoder_zero_extent_axis_and_formats():
    n = 500
    rec = np.zeros((n, 34), dtype=np.uint8)
    xyz = np.stack([np.full(n, 1234), np.arange(n) * 3, np.arange(n) % 7], 1).astype("<i4")
    rec[:, 0:12] = xyz.view(np.uint8).reshape(n, 12)
    rgb = np.stack([np.arange(n) * 131 % 65536, np.arange(n) % 256, np.full(n, 300)], 1).astype("<u2")
    for fmt, off in ((3, 28), (2, 20)):
        r = rec.copy()
        r[:, off:off + 6] = rgb.view(np.uint8).reshape(n, 6)
        r = np.ascontiguousarray(r).reshape(-1)
        sc, of, bm = [0.01] * 3, [10.0, 20.0, 30.0], [11.0, 19.0, 29.0]
        lib = L.load()
        nb = int(lib.cr_num_batches(n))
        batches = np.zeros(nb, L.BATCH_DTYPE)
        st = [np.zeros(n, np.uint32) for _ in range(4)]
        arr = lambda v: np.ascontiguousarray(v, np.float64)
        sca, ofa, bma = arr(sc), arr(of), arr(bm)
        assert lib.cr_encode_las(_p(r), n, 34, fmt, _p(sca), _p(ofa), _p(bma), 0, 0, _p(batches),
                                 *(_p(s) for s in st)) == 0
        ref = O.encode_las(r, n, 34, fmt, sc, of, bm)
        assert np.array_equal(batches.view(np.uint8), ref[0].view(np.uint8))
        for a, b in zip(st, ref[1:]):
            assert np.array_equal(a, b)
        assert (st[0] & 1023 == 0).all()  # zero-extent x quantises to 0
        R = st[3] & 0xFF
        exp = rgb[:, 0].astype(np.int64)
        exp = np.where(exp < 256, exp, exp // 256)
        assert np.array_equal(R, exp)


def test_encode_standard_matches_oracle():
    n = 2000
    p = synth.synth_params(L.SYNTH_TERRAIN, 100.0, 5)
    rec, hdr = synth.las_records_host(p, n, morton=False)
    lib = L.load()
    v = np.zeros(n, L.VERTEX_DTYPE)
    sc, of, bm = (np.ascontiguousarray(x[:], np.float64) for x in (hdr.scale, hdr.offset, hdr.min))
    assert lib.cr_encode_standard(_p(rec), n, 26, 2, _p(sc), _p(of), _p(bm), _p(v)) == 0
    w = np.zeros(n, L.VERTEX_DTYPE)
    O.lib().or_encode_standard(_p(rec), n, 26, 2, _p(sc), _p(of), _p(bm), _p(w))
    assert np.array_equal(v.view(np.uint8), w.view(np.uint8))
    assert ((v["color"] >> 24) == 255).all()


def test_generator_deterministic_and_morton_sorted():
    p = synth.synth_params(L.SYNTH_TERRAIN_BOXES, 500.0, 11, num_boxes=3, points_per_box=1000)
    a, ha = synth.las_records_host(p, 20000, morton=False)
    b, hb = synth.las_records_host(p, 20000, morton=False)
    assert np.array_equal(a, b)
    s, hs = synth.las_records_host(p, 20000, morton=True)
    assert sorted(map(bytes, a.reshape(-1, 26))) == sorted(map(bytes, s.reshape(-1, 26)))
    xyz = np.frombuffer(s.reshape(-1, 26)[:, :12].tobytes(), "<i4").reshape(-1, 3)
    pts = xyz * 0.001
    mn = np.array(hs.min[:])
    cube = max(hs.max[k] - hs.min[k] for k in range(3))
    q = np.minimum(((pts - mn) / cube * 2097152.0).astype(np.uint32), 2097151)
    o = O.lib()
    codes = [o.or_morton3(int(x), int(y), int(z)) for x, y, z in q]
    assert all(codes[i] <= codes[i + 1] for i in range(len(codes) - 1))
    # header bounds are the quantised extremes
    assert hs.min[0] == xyz[:, 0].min() * 0.001 and hs.max[2] == xyz[:, 2].max() * 0.001


@pytest.mark.skipif(not O.SFREF.exists(), reason="Sort_Frugal probe not built (no reference tree)")
def test_morton_order_matches_reference_sorter():
    """The oracle's Morton code equals Sort_Frugal's mortonEncode_magicbits on
    full 32-bit inputs (both keep 21 bits), and the product's host sort leaves
    records in nondecreasing reference code over the reference's quantisation,
    apart from the far-face value 2^21 that the product clamps to 2^21 - 1."""
    sf, o = O.sfref(), O.lib()
    rng = np.random.default_rng(5)
    vals = np.concatenate([rng.integers(0, 2**32, (3000, 3), dtype=np.uint64),
                           rng.integers(0, 2**21, (3000, 3), dtype=np.uint64),
                           np.array([[0, 0, 0], [2**21 - 1] * 3, [2**21] * 3, [2**32 - 1] * 3],
                                    np.uint64)])
    for x, y, z in vals.tolist():
        assert o.or_morton3(x, y, z) == sf.sfref_morton(x, y, z)
    p = synth.synth_params(L.SYNTH_TERRAIN_BOXES, 300.0, 4, num_boxes=4, points_per_box=800)
    s, hs = synth.las_records_host(p, 30000, morton=True)
    xyz = np.frombuffer(s.reshape(-1, 26)[:, :12].tobytes(), "<i4").reshape(-1, 3)
    mn = np.array(hs.min[:])
    cube = max(hs.max[k] - hs.min[k] for k in range(3))
    pts = xyz * np.array(hs.scale[:]) + np.array(hs.offset[:])
    q = ((pts - mn) / cube * 2097152.0).astype(np.uint64)
    q = np.minimum(q, 2**21 - 1)
    codes = [sf.sfref_morton(int(x), int(y), int(z)) for x, y, z in q.tolist()]
    assert all(codes[i] <= codes[i + 1] for i in range(len(codes) - 1))


def test_quirk_semantics():
    cl = encoded(n=25000, extent=150.0, seed=3)
    cam = cameras(cl)["near"]
    base = oracle_frame(cam, cl["box_min"][None], 0)
    args = (cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
    fb0 = O.raster_batched(base, *args)
    fb1 = O.raster_batched(oracle_frame(cam, cl["box_min"][None], O.L0_X12), *args)
    b = cl["batches"]
    mins = np.ascontiguousarray(np.stack([b["min_x"], b["min_y"], b["min_z"]], 1), np.float32)
    maxs = np.ascontiguousarray(np.stack([b["max_x"], b["max_y"], b["max_z"]], 1), np.float32)
    lv = [O.lib().or_precision_level(C.byref(base), C.byref(base.files[0]), _p(mins[i:i + 1]),
                                     _p(maxs[i:i + 1])) for i in range(len(b))]
    assert 0 in lv, "near camera must produce a 30-bit batch"
    assert not np.array_equal(fb0, fb1), "H1 changes the 30-bit decode"
    # H2: the inclusive bound also processes local index numPoints; here that is
    # the zero padding word past N, which decodes to the batch's min corner
    hm = handmade_cloud([(512, 512, 100), (700, 300, 200), (100, 900, 300)], [1, 2, 3])
    cam = identity_cam(64, 32)
    hargs = (hm["batches"], hm["n"], hm["lo"], hm["md"], hm["hi"], hm["rgba"])
    fa = O.raster_batched(oracle_frame(cam, hm["box_min"][None], 0), *hargs)
    fb = O.raster_batched(oracle_frame(cam, hm["box_min"][None], O.INCLUSIVE_END), *hargs)
    diff = np.nonzero(fa != fb)[0]
    assert len(diff) == 1 and diff[0] == 0 and (int(fb[0]) & 0xFFFFFFFF) == 3
    assert sum(int(v) != 0xFF800000FF800000 for v in fa) == 3
    # H3: ceil(numPoints / 10240) records are dispatched, not every record
    assert O.lib().or_dispatch_batches(12, 10240 * 10 + 5, O.DISPATCH_BY_POINTS) == 11
    assert O.lib().or_dispatch_batches(12, 10240 * 10 + 5, 0) == 12


def test_oracle_threads_equal_scalar():
    cl = encoded(n=50000, extent=120.0, seed=9)
    for name, cam in cameras(cl).items():
        for payload in (O.PAYLOAD_INDEX, O.PAYLOAD_COLOR):
            fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[L.METHOD_LOOP_LAS], payload)
            args = (cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
            a = O.raster_batched(fr, *args)
            b = O.raster_batched(fr, *args, threads=4)
            assert np.array_equal(a, b), name


@pytest.mark.skipif(not GOLDEN.exists(), reason="golden vectors not generated")
def test_golden_vectors():
    from golden import make_golden as G
    g = json.loads(GOLDEN.read_text())
    for case in g["cases"]:
        if case.get("cpu_check", True) is False:
            continue
        got = G.run_case(case)
        assert got == case["digests"], case["name"]


def _warp_scene(seed=4, warps=48, W=64, H=32):
    """Points whose pixel and depth are known: w = z exactly, x and y placed
    so that x / w lands on pixel centres.  Few pixels, so warps collide;
    negative z culls a lane."""
    rng = np.random.default_rng(seed)
    n = 32 * warps - 5  # a partial last warp
    v = np.zeros(n, dtype=L.VERTEX_DTYPE)
    px = rng.integers(0, 2, n)
    py = rng.integers(0, 2, n)
    # depths that differ in their low mantissa byte, where the color's top
    # byte lands in the key; x / w stays deep inside the chosen pixel
    zs = np.array([1.0 + k * 2.0**-23 for k in range(6)] + [2.0, -2.0], dtype=np.float32)
    z = rng.choice(zs, n).astype(np.float64)
    v["x"] = ((px + 0.5) * 2.0 / W - 1.0) * np.abs(z)
    v["y"] = ((py + 0.5) * 2.0 / H - 1.0) * np.abs(z)
    v["z"] = z
    v["color"] = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    proj = np.zeros(16)
    proj[0] = proj[5] = proj[10] = 1.0
    proj[11] = 1.0  # w = z (column-major: row 3, column 2)
    return v, np.eye(4).reshape(16), proj, W, H, px + py * W


def _warp_reference(v, pix, variant, words):
    fb = np.full(words, 0xFFFFFFFFFFFFFFFF, dtype=np.uint64)
    depth = v["z"].astype(np.float32).view(np.uint32).astype(np.int64)
    ok = v["z"] > 0
    for w0 in range(0, len(v), 32):
        lanes = range(w0, min(w0 + 32, len(v)))
        act = [i for i in lanes if ok[i]]
        write = set()
        if variant == 0:
            write = set(act)
        elif variant == 1:
            for i in act:
                write.add(i) if depth[i] == min(depth[j] for j in act if pix[j] == pix[i]) else None
        else:
            same = len({pix[i] for i in act}) <= 1
            mind = min((depth[i] for i in act), default=None)
            for i in act:
                q = w0 + ((i - w0) ^ 1)
                q_ok = q < len(v) and ok[q]
                if (same and depth[i] == mind) or (not same and (not q_ok or pix[q] != pix[i]
                                                                 or depth[i] <= depth[q])):
                    write.add(i)
        for i in write:
            key = np.uint64((int(depth[i]) << 24) | int(v["color"][i]))
            fb[pix[i]] = min(fb[pix[i]], key)
    return fb


@pytest.mark.parametrize("variant", [1, 2])
def test_plain_warp_variants_oracle_semantics(variant):
    """The oracle's dedup / early-z & reduce warp rules against a plain Python
    restatement on a scene with exact pixels and depths."""
    v, view, proj, W, H, pix = _warp_scene()
    got, _, _ = O.plain(view, proj, W, H, v, variant=variant)
    want = _warp_reference(v, pix, variant, O.fb_words(W, H))
    assert np.array_equal(got, want)


@pytest.mark.parametrize("variant", [1, 2])
def test_plain_warp_variants_keep_the_closer_point(variant):
    """Lanes 0 and 1 on one pixel: lane 0 closer but with color alpha 0xFF,
    lane 1 one ulp farther with alpha 0, so lane 1's depth << 24 | color key
    is the smaller one; lane 2 on another pixel.  Both reductions drop lane 1
    before the atomic, so the pixel keeps lane 0's key."""
    v, view, proj, W, H, _ = _warp_scene()
    v = v[:3].copy()
    d0 = np.float32(1.0)
    d1 = np.nextafter(d0, np.float32(2.0))
    for i, (px, z, color) in enumerate([(5, d0, 0xFF102030), (5, d1, 0x00405060), (9, d0, 0x7F000001)]):
        v["z"][i] = z
        v["x"][i] = ((px + 0.5) * 2.0 / W - 1.0) * float(z)
        v["y"][i] = (0.5 * 2.0 / H - 1.0) * float(z)
        v["color"][i] = color
    got, _, _ = O.plain(view, proj, W, H, v, variant=variant)
    key0 = (int(d0.view(np.uint32)) << 24) | 0xFF102030
    key1 = (int(d1.view(np.uint32)) << 24) | 0x00405060
    assert key1 < key0
    assert int(got[5]) == key0
    every, _, _ = O.plain(view, proj, W, H, v, variant=0)
    assert int(every[5]) >> 32 == int(d0.view(np.uint32))  # early-z: depth << 32 keeps lane 0 too


def test_precision_level_and_frustum_known_answers():
    """render.cs:199-231 and :176-197 on a scene with a closed-form projected
    size: a 90-degree camera at the origin looking down -z, 1000x1000 pixels,
    cubes of side s centred at distance 10, whose centre-to-edge distance on
    screen is 500 * (s * sqrt(3)) / 10 = 86.6 s pixels."""
    view = np.eye(4).reshape(16)
    proj = synth.perspective(90.0, 1.0, 0.1, 1000.0)
    fr = O.make_frame(view, proj, 1000, 1000, np.zeros((1, 3)))
    o = O.lib()
    want = {1.0: 4, 2.0: 3, 4.0: 2, 50.0: 1, 200.0: 0}  # 87, 173, 346, 4330, 17321 px
    for s, level in want.items():
        wmin = np.array([-s / 2, -s / 2, -10.0 - s / 2], np.float32)
        wmax = np.array([s / 2, s / 2, -10.0 + s / 2], np.float32)
        assert o.or_precision_level(C.byref(fr), C.byref(fr.files[0]), wmin.ctypes.data,
                                    wmax.ctypes.data) == level, s
        assert o.or_intersects_frustum(C.cast(fr.files[0].planes, C.c_void_p), wmin.ctypes.data,
                                       wmax.ctypes.data) == 1
    behind_min = np.array([-1, -1, 5], np.float32)
    behind_max = np.array([1, 1, 7], np.float32)
    assert o.or_intersects_frustum(C.cast(fr.files[0].planes, C.c_void_p), behind_min.ctypes.data,
                                   behind_max.ctypes.data) == 0
    beside_min = np.array([40, -1, -11], np.float32)  # x/|z| = 3.6 > 1
    beside_max = np.array([42, 1, -12], np.float32)
    assert o.or_intersects_frustum(C.cast(fr.files[0].planes, C.c_void_p), beside_min.ctypes.data,
                                   beside_max.ctypes.data) == 0


@pytest.mark.parametrize("bits", [10, 20, 30])
def test_encoder_round_trip_bounds(bits):
    """Quantise -> split -> decode (LasLoaderSparse.cpp:146-198, render.cs:333-397):
    a decoded coordinate is within size / 2^bits of the original, plus the
    float rounding of the stored AABB (H8: quantised against the double box,
    decoded against its float copy)."""
    n = 30000
    rec, hdr = synth.las_records_host(synth.synth_params(L.SYNTH_TERRAIN, 300.0, 12), n)
    batches, lo, md, hi, _ = synth.encode_las(rec, n, hdr)
    r = rec.reshape(n, 26)
    X = r[:, 0:12].copy().view("<i4").astype(np.float64)
    orig = X * np.array(hdr.scale[:]) + np.array(hdr.offset[:]) - np.array(hdr.min[:])
    for b in batches:
        sl = slice(int(b["first_point"]), int(b["first_point"]) + int(b["num_points"]))
        bmin = np.array([b["min_x"], b["min_y"], b["min_z"]], np.float64)
        bmax = np.array([b["max_x"], b["max_y"], b["max_z"]], np.float64)
        size = bmax - bmin
        q = []
        for k in range(3):
            w4, w8, w12 = ((s[sl] >> (10 * k)) & 1023 for s in (lo, md, hi))
            if bits == 10:
                q.append(w4.astype(np.float64) / 1024.0)
            elif bits == 20:
                q.append(((w4.astype(np.int64) << 10) | w8) / 2.0**20)
            else:
                q.append(((w4.astype(np.int64) << 20) | (w8.astype(np.int64) << 10) | w12) / 2.0**30)
        dec = bmin + np.stack(q, axis=1) * size
        ulp = np.spacing(np.maximum(np.abs(bmin), np.abs(bmax)).astype(np.float32)).astype(np.float64)
        bound = size / 2.0**bits + 2 * ulp + 1e-12
        err = np.abs(dec - orig[sl])
        assert (err <= bound).all(), (bits, float((err - bound).max()))


def test_key_packing_orders_by_depth_then_payload():
    """render.cs:421-423: key = floatBitsToUint(w) << 32 | payload; for w > 0
    the unsigned key order is the (depth, payload) order."""
    rng = np.random.default_rng(2)
    w = rng.uniform(0.01, 1e5, 5000).astype(np.float32)
    w[::7] = w[1::7][: len(w[::7])]  # ties
    pay = rng.integers(0, 2**32, 5000, dtype=np.uint64)
    key = (w.view(np.uint32).astype(np.uint64) << np.uint64(32)) | pay
    assert np.array_equal(np.argsort(key, kind="stable"), np.lexsort((pay, w)))



def test_plain_byte_round_trip():
    """compute_2021_earlyz/resolve.cs:41-77 writes uvec4(255.0 * unpackUnorm4x8(ucol)):
    per byte trunc(255 * RN(c / 255)) in binary32.  That is c again for all 256
    bytes, so the GPU resolve copies the bytes; the oracle keeps the formula."""
    c = np.arange(256, dtype=np.float32)
    back = np.float32(255.0) * (c / np.float32(255.0))
    assert back.dtype == np.float32
    assert np.array_equal(np.trunc(back).astype(np.int64), np.arange(256))
    # the oracle's resolve (the formula) equals the byte copy word for word
    rng = np.random.default_rng(3)
    w, h = 64, 32
    fb = (rng.integers(1, 2**31, w * h + w + 1, dtype=np.uint64) << np.uint64(32)) | \
        rng.integers(0, 2**32, w * h + w + 1, dtype=np.uint64)
    fb[::5] &= np.uint64(0xFFFFFFFFFF000000)  # ucol == 0 -> (0, 0, 0, 255)
    ucol = (fb[: w * h] & np.uint64(0xFFFFFF)).astype(np.uint32)
    for zero_rule in (1, 0):
        img = np.empty(w * h, dtype=np.uint32)
        f = fb.copy()
        O.lib().or_resolve_plain(w, h, f.ctypes.data, img.ctypes.data, 0xFFFFFFFFFF3C321E, 0,
                                 zero_rule)
        # early-z: ucol == 0 -> (0,0,0,255); dedup (compute_2021_dedup/resolve.cs:15-21)
        # has no such rule and writes the zero bytes
        want = np.where(ucol == 0, np.uint32(0xFF000000), ucol) if zero_rule else ucol
        assert np.array_equal(img, want)
        assert (f == np.uint64(0xFFFFFFFFFF3C321E)).all()  # pixels and guard tail re-cleared


def test_plain_resolve_tiles():
    """compute_2021_earlyz.h:161-163 dispatches floor(W/16) x floor(H/16)
    groups of 16x16: with the tile quirk, pixels past the last full tile keep
    their image and framebuffer words (and the guard tail is untouched)."""
    rng = np.random.default_rng(5)
    w, h = 40, 35  # 2 x 2 full tiles: x < 32, y < 32 resolved
    fb = (rng.integers(1, 2**31, w * h + w + 1, dtype=np.uint64) << np.uint64(32)) | \
        rng.integers(1, 2**24, w * h + w + 1, dtype=np.uint64)
    img0 = rng.integers(0, 2**32, w * h, dtype=np.uint64).astype(np.uint32)
    img, f = img0.copy(), fb.copy()
    O.lib().or_resolve_plain(w, h, f.ctypes.data, img.ctypes.data, 7, O.RESOLVE_TILES, 1)
    x, y = np.meshgrid(np.arange(w), np.arange(h))
    inside = ((x < 32) & (y < 32)).reshape(-1)
    ucol = (fb[: w * h] & np.uint64(0xFFFFFF)).astype(np.uint32)
    assert np.array_equal(img[inside], ucol[inside])
    assert np.array_equal(img[~inside], img0[~inside])
    assert (f[: w * h][inside] == 7).all()
    assert np.array_equal(f[: w * h][~inside], fb[: w * h][~inside])
    assert np.array_equal(f[w * h:], fb[w * h:])


def test_uvec4_base_matches_las2_thread_loop():
    """H6 (compute_loop_las2/render.cs:319-341): the oracle's CR_QUIRK_UVEC4_BASE
    rule renders exactly the points the shader's 128 threads visit, for
    firstPoint % 4 = 0..3, full and partial batches, with and without the
    inclusive end (H2)."""
    from helpers import las2_visits, pixel_grid_cloud
    firsts = [1, 10242, 20483, 26484]  # firstPoint % 4 = 1, 2, 3, 0
    counts = [10240, 10240, 6000, 1000]
    total = 27490
    cl = pixel_grid_cloud(firsts, counts, total)
    ident = np.eye(4).reshape(16)
    for inclusive in (False, True):
        q = O.UVEC4_BASE | (O.INCLUSIVE_END if inclusive else 0)
        fr = O.make_frame(ident, ident, 1024, 32, cl["box_min"], culling=0, quirks=q)
        fb = O.raster_batched(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
        got = set(int(x) for x in (fb[:1024 * 32] & np.uint64(0xFFFFFFFF))) - {0xFF800000}
        want = {f + l for f, c in zip(firsts, counts) for l in las2_visits(f, c, inclusive)}
        assert got == want, (inclusive, sorted(want - got)[:8], sorted(got - want)[:8])
        # without the quirk every point of [first, first + count) is rendered
        fr0 = O.make_frame(ident, ident, 1024, 32, cl["box_min"], culling=0,
                           quirks=O.INCLUSIVE_END if inclusive else 0)
        fb0 = O.raster_batched(fr0, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
        assert (fb0 != fb).any()
