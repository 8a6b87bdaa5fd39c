"""loop_nodes ("render Potree nodes") on a Potree 2.0 dataset, against the
oracle bit for bit: every octree node a batch of up to 64,512 points
(compute_loop_nodes/render.cs:296-300; the root here holds 250,000 and is cut
there), node-level culling and precision at 80 px, the level-4 cut (:273),
float uniforms (compute_loop_nodes.h:128-139) and the tiled resolve
(compute_loop_nodes.h:199-201)."""
import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import potree, synth
from helpers import camera_views, first_diff, gpu_raw, terrain_las
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NODE_QUIRKS = O.NODE_LOOP | O.LEVEL4_80PX | O.ONE_WORLD


@pytest.fixture(scope="module")
def octree(ctx, tmp_path_factory):
    d = tmp_path_factory.mktemp("octree")
    n = 2_000_000
    _, rec, hdr = terrain_las(n, 800.0, 3)
    nodes = potree.write_octree(d, rec, n, hdr.scale[:], hdr.offset[:], hdr.min[:], hdr.max[:],
                                max_leaf=20000, chunk_levels=2)
    o = potree.open_octree(d)
    cloud = o.load(ctx)
    enc = o.encode()
    assert max(nd["num_points"] for nd in nodes) > 64512
    assert sum(nd["num_points"] > 10240 for nd in nodes) > 10
    extent = np.array(hdr.max[:]) - np.array(hdr.min[:])
    views = camera_views(np.zeros(3), extent, enc[0])
    proj = synth.perspective(60.0, 400 / 250, 0.1, 200000.0)
    cams = {k: (v, proj, 400, 250) for k, v in views.items()}
    yield o, cloud, enc, n, cams
    cloud.close()
    o.close()


def oracle_words(enc, n, cam, lod=4, culling=1):
    view, proj, w, h = cam
    fr = O.make_frame(view, proj, w, h, np.zeros((1, 3)), culling=culling, quirks=NODE_QUIRKS,
                      payload=O.PAYLOAD_INDEX, lod_skip_level=lod, float_uniforms=True)
    return O.raster_batched(fr, enc[0], n, *enc[1:])


def test_loaded_cloud_equals_host_encoding(ctx, octree):
    o, cloud, enc, n, cams = octree
    assert np.array_equal(cloud.read(0).view(np.uint8), enc[0].view(np.uint8))
    for which, w in zip((L.STREAM_LOW, L.STREAM_MED, L.STREAM_HIG, L.STREAM_RGBA), enc[1:]):
        assert np.array_equal(cloud.read(which), w), which


@pytest.mark.parametrize("camname", ["far", "mid", "near", "corner"])
def test_loop_nodes_matches_oracle(ctx, octree, camname):
    o, cloud, enc, n, cams = octree
    cam = cams[camname]
    fb, params = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_NODES)
    assert params.lod_skip_level == 4
    got = fb.read(L.FB_WORDS)
    want = oracle_words(enc, n, cam)
    assert np.array_equal(got, want), first_diff(got, want)
    assert (got != L.DEFAULT_CLEAR).sum() > 100
    ctx.resolve(cloud, params, fb)
    img = O.resolve_index_tiles(cam[2], cam[3], want, enc[4])
    assert np.array_equal(fb.read(L.FB_IMAGE), img)
    # rows 240-249 (past the last full 16-pixel tile) keep the zeros of a new image
    assert (fb.read(L.FB_IMAGE).reshape(250, 400)[240:] == 0).all()
    fb.close()


def test_loop_nodes_lod_cut_and_node_cap(ctx, octree):
    """Without the level cut more nodes draw; the root's points past the
    64,512 the loop reaches never do."""
    o, cloud, enc, n, cams = octree
    cam = cams["far"]
    fb, _ = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_NODES, lod_skip_level=0)
    all_levels = oracle_words(enc, n, cam, lod=0)
    assert np.array_equal(fb.read(L.FB_WORDS), all_levels)
    assert (all_levels != oracle_words(enc, n, cam)).any()
    drawn = all_levels != L.DEFAULT_CLEAR
    ids = (all_levels & np.uint64(0xFFFFFFFF))[drawn].astype(np.int64)
    root = enc[0][0]
    assert root["num_points"] > 64512
    lo, hi = int(root["first_point"]) + 64512, int(root["first_point"]) + int(root["num_points"])
    assert not ((ids >= lo) & (ids < hi)).any()
    fb.close()
