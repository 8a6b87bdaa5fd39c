"""LAS ingest on the GPU: two files (LAS 1.2 and a multi-task LAS 1.4) and
the reference's own example file load into clouds whose batch records and
word streams equal the host encoder's, file by file at the files' sparse
offsets, and render as a cloud built from those host arrays does."""
import json
from pathlib import Path

import numpy as np
import pytest

import compute_rasterizer_gb300 as cr
from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import las, synth
from helpers import first_diff

pytestmark = pytest.mark.gpu

FIX = json.loads((Path(__file__).parent / "golden" / "las_5points_14.json").read_text())


def host_layout(files):
    """Host encoder per file at its sparse offset -> concatenated layout."""
    parts, point = [], 0
    for fi, (rec, info) in enumerate(files):
        n = int(info.num_points)
        out = synth.encode_las(rec, n, info, bytes_per_point=info.bytes_per_point,
                               point_format=info.point_format, sparse_offset=point, file_index=fi,
                               box_min=np.array(info.min[:]))
        parts.append(out)
        point += n
    return [np.concatenate([p[k] for p in parts]) for k in range(5)]


def test_two_files_equal_host_encoder(ctx, tmp_path):
    specs = [(50_001, 150.0, 21, (1, 2)), (1_100_000, 400.0, 22, (1, 4))]
    paths, files = [], []
    for i, (n, extent, seed, version) in enumerate(specs):
        rec, hdr = synth.las_records_host(synth.synth_params(L.SYNTH_TERRAIN, extent, seed), n)
        p = las.write_las(tmp_path / f"f{i}.las", rec, n, hdr.scale, hdr.offset, hdr.min, hdr.max,
                          version=version)
        paths.append(p)
        files.append((rec, las.read_info(p)))
    cloud, infos = las.load_files(ctx, paths)
    ctx.sync()
    want = host_layout(files)
    got_b = cloud.read(0)
    assert np.array_equal(got_b.view(np.uint8), want[0].view(np.uint8))
    for which, w in zip((L.STREAM_LOW, L.STREAM_MED, L.STREAM_HIG, L.STREAM_RGBA), want[1:]):
        g = cloud.read(which)
        assert np.array_equal(g, w), (which, first_diff(g, w))
    assert (got_b["file_index"][:5] == 0).all() and (got_b["file_index"][-3:] == 1).all()

    # the ingested cloud renders as the host-built one
    ref = ctx.cloud_from_arrays(*want, np.array([i.min[:] for i in infos]))
    bmin = np.minimum(np.array(infos[0].min[:]), np.array(infos[1].min[:]))
    view = synth.orbit_view(0.6, -0.7, 300.0, bmin + 100.0)
    proj = synth.perspective(60.0, 320 / 240, 0.1, 200000.0)
    imgs = []
    for c in (cloud, ref):
        fb = ctx.framebuffer(320, 240)
        fb.clear()
        ctx.render(c, cr.make_view(view, proj, 320, 240), cr.default_params(L.METHOD_LOOP_LAS), fb)
        ctx.sync()
        imgs.append(fb.read(L.FB_IMAGE))
        fb.close()
    assert np.array_equal(imgs[0], imgs[1])
    assert (imgs[0] != L.BACKGROUND).sum() > 100


def test_reference_example_file(ctx, tmp_path):
    p = tmp_path / "5points_14.las"
    p.write_bytes(bytes.fromhex(FIX["bytes_hex"]))
    cloud, (info,) = las.load_files(ctx, [p])
    ctx.sync()
    rec = las.read_records(p, info)
    want = host_layout([(rec, info)])
    assert np.array_equal(cloud.read(0).view(np.uint8), want[0].view(np.uint8))
    for which, w in zip((L.STREAM_LOW, L.STREAM_MED, L.STREAM_HIG, L.STREAM_RGBA), want[1:]):
        assert np.array_equal(cloud.read(which), w)
