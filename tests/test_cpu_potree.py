"""Potree 2.0 ingest (include/cr_potree.h) on the host: the hierarchy reader
against the node list the writer produced, and the node encoder against a
numpy restatement of PotreeData.h:361-452."""
import json

import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import potree
from helpers import terrain_las


@pytest.fixture(scope="module")
def dataset(tmp_path_factory):
    d = tmp_path_factory.mktemp("potree")
    _, rec, hdr = terrain_las(300_000, 400.0, 5)
    nodes = potree.write_octree(d, rec, 300_000, hdr.scale[:], hdr.offset[:], hdr.min[:], hdr.max[:],
                                max_leaf=4000, chunk_levels=2)
    return d, nodes, hdr


def test_hierarchy_matches_writer(dataset):
    d, nodes, hdr = dataset
    o = potree.open_octree(d)
    assert o.info.num_points == 300_000 and o.info.num_nodes == len(nodes)
    assert o.info.bytes_per_point == 21 and o.info.rgb_offset == 15
    assert o.info.max_level == max(n["level"] for n in nodes) >= 3  # several hierarchy chunks
    assert all(n["num_points"] > 0 for n in nodes)
    got = o.nodes()
    for a, b in zip(got, nodes):
        for k in ("level", "num_points", "byte_offset", "byte_size", "child_mask", "min", "max"):
            assert a[k] == b[k], (k, a, b)
    meta = json.loads((d / "metadata.json").read_text())
    assert meta["hierarchy"]["firstChunkSize"] < (d / "hierarchy.bin").stat().st_size


def encode_reference(d, nodes, quirks=-1):
    """PotreeData.h:361-452 in numpy: x = X * scale + offset - boxMin (double);
    X30 = uint32(((x - nodeMin) / nodeSize) * 2^30) & MASK_30BIT; 4b/8b words
    from bits 29..20 / 19..10, the 12b word from bits 19..10 again; RGB16 -> 8."""
    meta = json.loads((d / "metadata.json").read_text())
    scale, offset = np.array(meta["scale"]), np.array(meta["offset"])
    bmin = np.array(meta["boundingBox"]["min"])
    raw = np.fromfile(d / "octree.bin", np.uint8).reshape(-1, 21)
    n = meta["points"]
    lo, md, hi, rgba = (np.zeros(n, np.uint32) for _ in range(4))
    wrap = quirks == -1 or quirks & L.POTREE_QUIRK_WRAP30
    x12_8 = quirks == -1 or quirks & L.POTREE_QUIRK_12B_FROM_8B
    for nd in nodes:
        first, cnt = nd["byte_offset"] // 21, nd["num_points"]
        r = raw[first:first + cnt]
        x = r[:, :12].copy().view("<i4").reshape(-1, 3).astype(np.float64) * scale + offset - bmin
        mn, mx = np.array(nd["min"]), np.array(nd["max"])
        t = ((x - mn) / (mx - mn)) * 1073741824.0
        if wrap:
            q = (t.astype(np.int64) & 0x3FFFFFFF).astype(np.uint32)
        else:
            q = np.clip(t, 0, 1073741823).astype(np.uint32)

        def word(s):
            return ((q[:, 0] >> s) & 1023) | (((q[:, 1] >> s) & 1023) << 10) | (((q[:, 2] >> s) & 1023) << 20)
        lo[first:first + cnt] = word(20)
        md[first:first + cnt] = word(10)
        hi[first:first + cnt] = word(10) if x12_8 else word(0)
        c = r[:, 15:21].copy().view("<u2").reshape(-1, 3).astype(np.uint32)
        c = np.where(c > 255, c // 256, c)
        rgba[first:first + cnt] = c[:, 0] | (c[:, 1] << 8) | (c[:, 2] << 16)
    return lo, md, hi, rgba


@pytest.mark.parametrize("quirks", [L.POTREE_QUIRKS_DEFAULT, 0])
def test_encoder_matches_restatement(dataset, quirks):
    d, nodes, _ = dataset
    o = potree.open_octree(d)
    batches, *streams = o.encode(quirks)
    want = encode_reference(d, nodes, quirks)
    for g, w in zip(streams, want):
        assert np.array_equal(g, w)
    assert np.array_equal(batches["first_point"], [n["byte_offset"] // 21 for n in nodes])
    assert np.array_equal(batches["num_points"], [n["num_points"] for n in nodes])
    assert np.array_equal(batches["file_index"], [n["level"] for n in nodes])  # the node level
    assert np.array_equal(batches["max_x"], np.float32([n["max"][0] for n in nodes]))
    if quirks == L.POTREE_QUIRKS_DEFAULT:
        assert np.array_equal(streams[2], streams[1])  # the 12b word repeats the 8b one


def test_open_errors(tmp_path, dataset):
    d, _, _ = dataset
    with pytest.raises(L.CRError) as e:
        potree.open_octree(tmp_path / "missing")
    assert e.value.status == L.NOT_FOUND
    bad = tmp_path / "bad"
    bad.mkdir()
    (bad / "hierarchy.bin").write_bytes((d / "hierarchy.bin").read_bytes())
    (bad / "metadata.json").write_text("{\"points\": 10, \"scale\": [1, 1]}")
    with pytest.raises(L.CRError) as e:
        potree.open_octree(bad)
    assert e.value.status == L.INVALID_ARG
    meta = json.loads((d / "metadata.json").read_text())
    meta["hierarchy"]["firstChunkSize"] = 21  # not a whole entry
    (bad / "metadata.json").write_text(json.dumps(meta))
    with pytest.raises(L.CRError):
        potree.open_octree(bad)


def test_node_loop_rule_in_oracle():
    """compute_loop_nodes/render.cs:296-300 restated literally (threads of
    uvec4 from firstPoint / 4, `continue` past numPoints) against the
    oracle's per-batch point count."""
    import ctypes as C

    from oracle import oracle as O

    def visits(first, n):
        loop = min(-(-n // 128), 500) + 4
        out = 0
        for t in range(128):
            base = first // 4 + t
            for i in range(loop // 4):
                for j in range(4):
                    local = (4 * (base + i * 128) + j - first) & 0xFFFFFFFF
                    if local < n:
                        out += 1
        return out
    fn = O.lib().or_points_in_batch
    fn.argtypes, fn.restype = [C.c_void_p, C.c_int32], C.c_int64
    for first, n in ((0, 0), (5, 1), (3, 10240), (8, 20000), (2, 64000), (1, 64512), (0, 70000),
                     (7, 250000)):
        b = np.zeros(1, L.BATCH_DTYPE)
        b["first_point"], b["num_points"] = first, n
        assert fn(b.ctypes.data, O.NODE_LOOP) == visits(first, n), (first, n)
