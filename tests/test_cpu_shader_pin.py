"""The oracle pinned to the reference's own GLSL shaders.

oracle/glsl_cpp.py translates the reference's compute shaders to C++ (the
statements as written, glm for the GLSL types and operators) and
oracle/shader_ref.cpp runs their dispatches on the CPU.  The oracle in its
literal arithmetic mode (IEEE operations in the source's order, glm's
association) must produce the same framebuffers bit for bit; the contract
mode, which the kernels follow, differs from it only in its FMA and
reciprocal choices, which GLSL leaves to the driver.  Skipped where the
reference checkout is absent (the probe is built from it)."""
import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from helpers import QUIRKS, cameras, encoded, many_file_cameras, many_file_cloud, oracle_frame
from oracle import oracle as O

pytestmark = pytest.mark.skipif(not O.SHADERREF.exists(),
                                reason="no reference checkout: shader probe not built")


def shader_files(fr, box_mins):
    """The shaders' File records (render.cs:44-49): transform, transformFrustum,
    world = translate(boxMin), padding; compute_loop_las.h:166-200."""
    files = np.zeros((len(box_mins), 64), np.float32)
    for i, bm in enumerate(np.asarray(box_mins, np.float64).reshape(-1, 3)):
        t = np.frombuffer(bytes(fr.files[i].transform), np.float32)
        files[i, :16] = t
        files[i, 16:32] = t
        world = np.eye(4)
        world[3, :3] = bm
        files[i, 32:48] = world.reshape(16).astype(np.float32)
    return files


def f32(m):
    return np.ascontiguousarray(np.asarray(m, np.float64).reshape(16).astype(np.float32))


def ref_loop_las(cam, cl, box_mins, fr):
    view, proj, w, h = cam
    fb = np.full(O.fb_words(w, h), L.DEFAULT_CLEAR, np.uint64)
    n = cl["n"]
    lo, md, hi = (O.pad_stream(a, n=n) for a in (cl["lo"], cl["md"], cl["hi"]))
    b = np.ascontiguousarray(cl["batches"])
    files = shader_files(fr, box_mins)
    fv, fp = f32(view), f32(proj)
    assert O.shaderref().ref_loop_las_render(b.ctypes.data, len(b), lo.ctypes.data, md.ctypes.data,
                                             hi.ctypes.data, files.ctypes.data, fv.ctypes.data,
                                             fp.ctypes.data, w, h, 1, n, fb.ctypes.data) == 0
    return fb


def oracle_loop_las(cam, cl, box_mins, mode):
    with O.arith(mode):
        fr = oracle_frame(cam, box_mins, O.L0_X12)
        fb = O.raster_batched(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], None,
                              clear=L.DEFAULT_CLEAR)
    return fr, fb


@pytest.mark.parametrize("camname", ["far", "near", "mid", "corner"])
def test_loop_las_literal_oracle_is_the_reference_shader(camname):
    """compute_loop_las/render.cs: 10/20/30-bit decode (H1's X_12 included),
    culling, precision level, early-z read and atomicMin, index payload."""
    cl = encoded()
    cam = cameras(cl)[camname]
    bm = cl["box_min"][None]
    fr, want = oracle_loop_las(cam, cl, bm, O.ARITH_LITERAL)
    got = ref_loop_las(cam, cl, bm, fr)
    assert (got != L.DEFAULT_CLEAR).sum() > 1000
    assert np.array_equal(got, want), int(np.argmax(got != want))
    # the contract (the kernels' arithmetic) differs only by its rounding choices
    _, contract = oracle_loop_las(cam, cl, bm, O.ARITH_CONTRACT)
    assert not np.array_equal(contract, want)


def test_loop_las_literal_oracle_is_the_reference_shader_many_files():
    """Per-file records through the shader's ssFiles[batch.fileIndex]."""
    cl = many_file_cloud(nfiles=24, base=10241, spread=900)
    for camname, cam in many_file_cameras(cl).items():
        fr, want = oracle_loop_las(cam, cl, cl["box_min"], O.ARITH_LITERAL)
        got = ref_loop_las(cam, cl, cl["box_min"], fr)
        assert np.array_equal(got, want), (camname, int(np.argmax(got != want)))


def ref_loop_las2(cam, cl, box_mins, fr):
    """compute_loop_las2/render.cs; its uvec4 prefetch reads up to 10,240 words
    past a batch's firstPoint / 4 whatever the batch holds, so the streams are
    padded (with zeros, as the device streams' tails) to cover them."""
    view, proj, w, h = cam
    fb = np.full(O.fb_words(w, h), L.DEFAULT_CLEAR, np.uint64)
    n = cl["n"]
    words = int(cl["batches"]["first_point"].max()) + 10240 + 64
    lo, md, hi = (O.pad_stream(a, pad=words - len(a)) for a in (cl["lo"], cl["md"], cl["hi"]))
    b = np.ascontiguousarray(cl["batches"])
    files = shader_files(fr, box_mins)
    fv, fp = f32(view), f32(proj)
    assert O.shaderref().ref_loop_las2_render(b.ctypes.data, len(b), lo.ctypes.data,
                                              md.ctypes.data, hi.ctypes.data, files.ctypes.data,
                                              fv.ctypes.data, fp.ctypes.data, w, h, 1, n,
                                              fb.ctypes.data) == 0
    return fb


def oracle_loop_las2(cam, cl, box_mins, mode):
    with O.arith(mode):
        fr = oracle_frame(cam, box_mins, QUIRKS[L.METHOD_LOOP_LAS_PREFETCH])
        fb = O.raster_batched(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], None,
                              clear=L.DEFAULT_CLEAR)
    return fr, fb


@pytest.mark.parametrize("camname", ["far", "near", "mid", "corner"])
def test_loop_las2_literal_oracle_is_the_reference_shader(camname):
    """compute_loop_las2/render.cs (loop_las_prefetch): the uvec4 prefetch loop,
    `localIndex > numPoints` (one point past a partial batch, H2), and
    ceil(numPoints / 10240) workgroups (H3)."""
    cl = encoded()
    cam = cameras(cl)[camname]
    bm = cl["box_min"][None]
    fr, want = oracle_loop_las2(cam, cl, bm, O.ARITH_LITERAL)
    got = ref_loop_las2(cam, cl, bm, fr)
    assert (got != L.DEFAULT_CLEAR).sum() > 1000
    assert np.array_equal(got, want), int(np.argmax(got != want))


def test_loop_las2_uvec4_base_matches_the_reference_shader():
    """Files whose first points fall on every firstPoint % 4: the shader's
    uvec4 base firstPoint / 4 + tid drops thread 0 and the batch's last
    firstPoint % 4 points (H6), which the oracle's CR_QUIRK_UVEC4_BASE rule
    reproduces."""
    cl = many_file_cloud(nfiles=24, base=10241, spread=900)
    assert {int(f) % 4 for f in cl["batches"]["first_point"]} == {0, 1, 2, 3}
    for camname, cam in many_file_cameras(cl).items():
        fr, want = oracle_loop_las2(cam, cl, cl["box_min"], O.ARITH_LITERAL)
        got = ref_loop_las2(cam, cl, cl["box_min"], fr)
        assert np.array_equal(got, want), (camname, int(np.argmax(got != want)))


@pytest.mark.parametrize("camname", ["far", "near", "mid", "corner"])
def test_hqs_literal_oracle_is_the_reference_shaders(camname):
    """compute_loop_las_hqs/depth.cs then color.cs: the u32 depth pass, the
    1.01 depth window and the two 64-bit (R | G << 32, B | count << 32)
    accumulators per pixel."""
    cl = encoded()
    view, proj, w, h = cam = cameras(cl)[camname]
    bm = cl["box_min"][None]
    with O.arith(O.ARITH_LITERAL):
        fr = oracle_frame(cam, bm, QUIRKS[L.METHOD_LOOP_LAS_HQS])
        depth, accum, _ = O.hqs(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
    n = cl["n"]
    lo, md, hi, rgba = (O.pad_stream(a, n=n) for a in (cl["lo"], cl["md"], cl["hi"], cl["rgba"]))
    got_d = np.full(O.fb_words(w, h), 0xFF800000, np.uint32)
    got_a = np.zeros(2 * O.fb_words(w, h), np.int64)
    b = np.ascontiguousarray(cl["batches"])
    files = shader_files(fr, bm)
    fv, fp = f32(view), f32(proj)
    assert O.shaderref().ref_hqs_render(b.ctypes.data, len(b), lo.ctypes.data, md.ctypes.data,
                                        hi.ctypes.data, rgba.ctypes.data, files.ctypes.data,
                                        fv.ctypes.data, fp.ctypes.data, w, h, 1, n,
                                        got_d.ctypes.data, got_a.ctypes.data) == 0
    assert (got_d != 0xFF800000).sum() > 1000
    assert np.array_equal(got_d, depth), int(np.argmax(got_d != depth))
    assert np.array_equal(got_a.view(np.uint64), accum), int(np.argmax(got_a.view(np.uint64) != accum))


def padded(words, width, height, fill, dtype=np.uint64, per_pixel=1):
    """A copy of a per-pixel buffer long enough for the resolves' partial
    16 x 16 tiles, which read words past W*H; the extra words hold `fill`."""
    h16, w16 = -(-height // 16) * 16, -(-width // 16) * 16
    need = per_pixel * (h16 * width + w16 + 16)
    out = np.full(max(need, len(words)), fill, dtype)
    out[:len(words)] = words
    return out


def test_loop_las_resolve_is_the_reference_shader():
    """compute_loop_las/resolve.cs (window 0) over ceil(W/16) x ceil(H/16)
    groups at a size that leaves partial tiles: the index payload's color
    gather, point index 0 and empty pixels to the background."""
    cl = encoded()
    cam = cameras(cl, width=331, height=250)["far"]
    _, fb = oracle_loop_las(cam, cl, cl["box_min"][None], O.ARITH_LITERAL)
    w, h = cam[2], cam[3]
    want = O.resolve_index(w, h, fb, cl["rgba"])
    got = np.zeros(w * h, np.uint32)
    rgba = O.pad_stream(cl["rgba"], n=cl["n"])
    fbp = padded(fb, w, h, 0xFFFFFFFFFFFFFFFF)
    assert O.shaderref().ref_loop_las_resolve(fbp.ctypes.data, rgba.ctypes.data, w, h,
                                              got.ctypes.data) == 0
    assert (want != 0x00443322).sum() > 1000
    assert np.array_equal(got, want), int(np.argmax(got != want))


def test_hqs_resolve_is_the_reference_shader():
    """compute_loop_las_hqs/resolve.cs: integer means of the accumulated
    colors, empty pixels to the background, partial tiles."""
    cl = encoded()
    cam = cameras(cl, width=331, height=250)["far"]
    with O.arith(O.ARITH_LITERAL):
        fr = oracle_frame(cam, cl["box_min"][None], QUIRKS[L.METHOD_LOOP_LAS_HQS])
        _, accum, want = O.hqs(fr, cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
    w, h = cam[2], cam[3]
    got = np.zeros(w * h, np.uint32)
    acc = padded(accum, w, h, 0, per_pixel=2)
    assert O.shaderref().ref_hqs_resolve(acc.ctypes.data, w, h, got.ctypes.data) == 0
    assert (want != 0x00443322).sum() > 1000
    assert np.array_equal(got, want), int(np.argmax(got != want))


@pytest.mark.parametrize("w,h", [(1920, 1080), (333, 250)])
def test_earlyz_render_and_resolve_are_the_reference_shaders(w, h):
    """compute_2021_earlyz/render.cs and resolve.cs (config 1's scene): the
    early-z depth compare and 64-bit atomicMin over 16-byte points, then the
    floor(W/16) x floor(H/16) resolve with its re-clear.  The render compares
    depths only, so two points of one pixel at the same depth keep the first
    in the shader's order and the smaller key in the oracle's (both outcomes
    of the reference's race on a GPU): such pixels must agree on the depth."""
    from compute_rasterizer_gb300 import synth
    n = 128 * 6000
    v = synth.uniform_vertices_host(3, n, 100.0)
    view = synth.look_at([150.0, 150.0, 150.0], [50.0, 50.0, 50.0], [0.0, 0.0, 1.0])
    proj = synth.perspective(60.0, w / h, 0.1, 1000.0)
    with O.arith(O.ARITH_LITERAL):
        want_fb, want_img, want_cleared = O.plain(view, proj, w, h, v)
    T = np.empty(16, np.float32)
    vd = np.ascontiguousarray(np.asarray(view, np.float64).reshape(16))
    pd = np.ascontiguousarray(np.asarray(proj, np.float64).reshape(16))
    O.lib().or_plain_transform(vd.ctypes.data, pd.ctypes.data, T.ctypes.data)
    fb = np.full(O.fb_words(w, h), 0xFFFFFFFFFFFFFFFF, np.uint64)
    g = O.shaderref()
    vv = np.ascontiguousarray(v)
    assert g.ref_earlyz_render(vv.ctypes.data, n, T.ctypes.data, w, h, fb.ctypes.data) == 0
    assert (fb != 0xFFFFFFFFFFFFFFFF).sum() > 10000
    differ = fb != want_fb
    assert np.array_equal(fb[differ] >> np.uint64(32), want_fb[differ] >> np.uint64(32))
    assert differ.sum() <= 16, int(differ.sum())
    fb[differ] = want_fb[differ]  # the same race outcome on both sides for the resolve
    img = np.zeros(w * h * 4, np.uint8)
    assert g.ref_earlyz_resolve(fb.ctypes.data, w, h, img.ctypes.data) == 0
    assert np.array_equal(img.view(np.uint32), want_img), int(np.argmax(img.view(np.uint32) != want_img))
    assert np.array_equal(fb, want_cleared)


@pytest.fixture(scope="module")
def octree_nodes(tmp_path_factory):
    """A Potree 2.0 octree of an 800,000-point terrain, encoded one batch per
    node (the root over 64,512 points, so the 500-step loop cap cuts it)."""
    from compute_rasterizer_gb300 import potree, synth
    from helpers import camera_views, terrain_las
    d = tmp_path_factory.mktemp("pin_octree")
    n = 800_000
    _, rec, hdr = terrain_las(n, 400.0, 3)
    nodes = potree.write_octree(d, rec, n, hdr.scale[:], hdr.offset[:], hdr.min[:], hdr.max[:],
                                max_leaf=20000, chunk_levels=2)
    assert max(nd["num_points"] for nd in nodes) > 64512
    o = potree.open_octree(d)
    enc = o.encode()
    o.close()
    extent = np.array(hdr.max[:]) - np.array(hdr.min[:])
    views = camera_views(np.zeros(3), extent, enc[0])
    proj = synth.perspective(60.0, 400 / 250, 0.1, 200000.0)
    return enc, n, {k: (v, proj, 400, 250) for k, v in views.items()}


@pytest.mark.parametrize("camname", ["far", "mid", "near", "corner"])
def test_loop_nodes_literal_oracle_is_the_reference_shader(octree_nodes, camname):
    """compute_loop_nodes/render.cs: one workgroup per node, min(ceil(n/128),
    500) + 4 steps of one uvec4 per invocation, the 80 px level cut and the
    one world matrix, float uniforms."""
    enc, n, cams = octree_nodes
    view, proj, w, h = cam = cams[camname]
    with O.arith(O.ARITH_LITERAL):
        fr = O.make_frame(view, proj, w, h, np.zeros((1, 3)), culling=1,
                          quirks=O.NODE_LOOP | O.LEVEL4_80PX | O.ONE_WORLD, payload=O.PAYLOAD_INDEX,
                          lod_skip_level=4, float_uniforms=True)
        want = O.raster_batched(fr, enc[0], n, *enc[1:4], None, clear=L.DEFAULT_CLEAR)
    batches = np.ascontiguousarray(enc[0])
    words = int(batches["first_point"].max()) + 4 * 128 * 130 + 64
    lo, md, hi = (O.pad_stream(a, pad=words - len(a)) for a in enc[1:4])
    T = np.ascontiguousarray(np.frombuffer(bytes(fr.files[0].transform), np.float32))
    fb = np.full(O.fb_words(w, h), L.DEFAULT_CLEAR, np.uint64)
    assert O.shaderref().ref_loop_nodes_render(batches.ctypes.data, len(batches), lo.ctypes.data,
                                               md.ctypes.data, hi.ctypes.data, f32(view).ctypes.data,
                                               f32(proj).ctypes.data, T.ctypes.data, w, h, 1, n,
                                               fb.ctypes.data) == 0
    assert (fb != L.DEFAULT_CLEAR).sum() > 100
    assert np.array_equal(fb, want), int(np.argmax(fb != want))


@pytest.mark.parametrize("method,variant", [("dedup", 1), ("reduce", 2)])
@pytest.mark.parametrize("n,w,h", [(128 * 3000, 320, 180), (128 * 1500, 64, 48)])
def test_warp_variants_are_the_reference_shaders(method, variant, n, w, h):
    """compute_2021_dedup/render.cs (subgroupPartitionNV + PartitionedMin)
    and compute_2021_earlyz_reduce/render.cs (subgroupAllEqual, subgroupMin,
    subgroupClusteredXor / Min over lane pairs, taken only by the lanes the
    short-circuit reaches) with 32-invocation subgroups in lockstep, against
    the oracle's warp rules: the random scene and a 64x48 view where most
    of a subgroup lands on one pixel."""
    from compute_rasterizer_gb300 import synth
    v = synth.uniform_vertices_host(3, n, 100.0)
    view = synth.look_at([150.0, 150.0, 150.0], [50.0, 50.0, 50.0], [0.0, 0.0, 1.0])
    proj = synth.perspective(60.0, w / h, 0.1, 1000.0)
    with O.arith(O.ARITH_LITERAL):
        want, _, _ = O.plain(view, proj, w, h, v, variant=variant)
    T = np.empty(16, np.float32)
    vd = np.ascontiguousarray(np.asarray(view, np.float64).reshape(16))
    pd = np.ascontiguousarray(np.asarray(proj, np.float64).reshape(16))
    O.lib().or_plain_transform(vd.ctypes.data, pd.ctypes.data, T.ctypes.data)
    fb = np.full(O.fb_words(w, h), 0xFFFFFFFFFFFFFFFF, np.uint64)
    vv = np.ascontiguousarray(v)
    fn = O.shaderref().ref_dedup_render if variant == 1 else O.shaderref().ref_reduce_render
    assert fn(vv.ctypes.data, n, T.ctypes.data, w, h, fb.ctypes.data) == 0
    assert (fb != 0xFFFFFFFFFFFFFFFF).sum() > 100
    assert np.array_equal(fb, want), int(np.argmax(fb != want))


def ray_vertices(w, h, rays, seed, pairs):
    """Points on view rays of pixel centres (view = identity): every subgroup
    of 32 consecutive points on one ray (pairs=False) or each lane pair on
    its own ray (pairs=True), depths 2 + k * 2^-20 a few ulps apart along a
    ray (k the lane, or 0 and 3 within a pair), so that
    depth << 24 | color lets a farther point's color byte win: which lanes a
    subgroup lets through decides the framebuffer."""
    from compute_rasterizer_gb300 import synth
    proj = np.asarray(synth.perspective(60.0, w / h, 0.1, 1000.0), np.float64).reshape(16)
    rng = np.random.default_rng(seed)
    n = 32 * rays
    lane = np.arange(n) % 32
    ray = np.arange(n) // (2 if pairs else 32)
    px, py = rng.integers(0, w, ray.max() + 1)[ray], rng.integers(0, h, ray.max() + 1)[ray]
    sx, sy = (2.0 * (px + 0.5) / w - 1.0), (2.0 * (py + 0.5) / h - 1.0)
    depth = 2.0 + ((lane & 1) * 3 if pairs else lane) * 2.0 ** -20
    v = np.zeros(n, dtype=L.VERTEX_DTYPE)
    v["x"], v["y"], v["z"] = sx * depth / proj[0], sy * depth / proj[5], -depth
    v["color"] = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    return v, np.eye(4), proj


@pytest.mark.parametrize("variant", [1, 2])
@pytest.mark.parametrize("pairs", [False, True])
def test_warp_variants_on_crowded_subgroups(variant, pairs):
    """Subgroups whose lanes share pixels at nearly equal depths: the
    partitions (dedup), the all-equal fast path and the lane-pair clusters
    (early-z & reduce) decide which keys reach the framebuffer, and the
    result differs from every point submitting."""
    w, h = 64, 48
    v, view, proj = ray_vertices(w, h, 600, 5 + variant, pairs)
    n = len(v)
    with O.arith(O.ARITH_LITERAL):
        want, _, _ = O.plain(view, proj, w, h, v, variant=variant)
    T = np.empty(16, np.float32)
    vd, pd = np.ascontiguousarray(view.reshape(16)), np.ascontiguousarray(proj)
    O.lib().or_plain_transform(vd.ctypes.data, pd.ctypes.data, T.ctypes.data)
    fb = np.full(O.fb_words(w, h), 0xFFFFFFFFFFFFFFFF, np.uint64)
    vv = np.ascontiguousarray(v)
    fn = O.shaderref().ref_dedup_render if variant == 1 else O.shaderref().ref_reduce_render
    assert fn(vv.ctypes.data, n, T.ctypes.data, w, h, fb.ctypes.data) == 0
    assert np.array_equal(fb, want), int(np.argmax(fb != want))
    # every point submitting its key: the same points one per subgroup (the
    # other 31 invocations behind the camera, culled) -- the subgroup rules
    # are what makes the two framebuffers differ
    spread = np.zeros(32 * n, dtype=L.VERTEX_DTYPE)
    spread["z"] = 1.0
    spread[::32] = v
    with O.arith(O.ARITH_LITERAL):
        everyone, _, _ = O.plain(view, proj, w, h, spread, variant=variant)
    assert (want != 0xFFFFFFFFFFFFFFFF).sum() > 300
    assert np.array_equal(want != 0xFFFFFFFFFFFFFFFF, everyone != 0xFFFFFFFFFFFFFFFF)
    assert (want != everyone).sum() > 50
