"""LAZ ingest on the GPU (include/cr_laz.h): the committed LAZ files whose
point data LASzip wrote (point formats 0-3 and the LAS 1.4 formats 6-8) load
into clouds whose batch records and word streams equal the oracle's loadLas
encoding of the same records (colour 0 for point formats without RGB, as
loadLaz reads LASzip's zeroed rgb), render as the
oracle renders them, load beside LAS files in one cloud, and a multi-window
file written by the product's writer equals the LAS path of its records."""
import json
from pathlib import Path

import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import las, synth
from helpers import (LAZ_OFFSET, LAZ_SCALE, QUIRKS, camera_views, first_diff, gpu_raw, laz_box, laz_records,
                     oracle_frame)
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = json.loads((GOLDEN / "laz.json").read_text())["cases"]
STREAMS = (L.STREAM_LOW, L.STREAM_MED, L.STREAM_HIG, L.STREAM_RGBA)


def oracle_layout(rec, n, bpp, fmt, bmin, point=0, file_index=0):
    """The oracle's loadLas per load task of 1,024,000 points; colour 0
    without an RGB item."""
    parts = []
    for t0 in range(0, n, L.MAX_POINTS_PER_LOAD):
        cnt = min(L.MAX_POINTS_PER_LOAD, n - t0)
        out = O.encode_las(rec[t0 * bpp:(t0 + cnt) * bpp], cnt, bpp, fmt, LAZ_SCALE, LAZ_OFFSET, bmin,
                           sparse_offset=point + t0, file_index=file_index)
        parts.append(out)
    lay = [np.concatenate([p[k] for p in parts]) for k in range(5)]
    if fmt in (0, 1, 6):
        lay[4][:] = 0
    return lay


def assert_cloud(cloud, want, b0=0, p0=0):
    got = cloud.read(0)
    nb, n = len(want[0]), len(want[1])
    assert np.array_equal(got[b0:b0 + nb].view(np.uint8), want[0].view(np.uint8))
    for which, w in zip(STREAMS, want[1:]):
        g = cloud.read(which)[p0:p0 + n]
        assert np.array_equal(g, w), (which, first_diff(g, w))


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_fixture_loads_as_oracle_encodes(ctx, case):
    path = GOLDEN / "laz" / f"{case['name']}.laz"
    cloud, (info,) = las.load_files(ctx, [path], threads=3)
    ctx.sync()
    fmt, n = case["point_format"], case["points"]
    rec, bpp = laz_records(fmt, n, case["seed"], case["extra"])
    bmin = np.array(info.min[:])
    want = oracle_layout(rec, n, bpp, fmt, bmin)
    assert_cloud(cloud, want)
    # and renders as the oracle renders its layout (loop_las, index payload)
    bmax = np.array(info.max[:])
    view = camera_views(bmin, bmax, want[0])["far"]
    cam = (view, synth.perspective(60.0, 320 / 240, 0.1, 200000.0), 320, 240)
    fb, _ = gpu_raw(ctx, cloud, cam, L.METHOD_LOOP_LAS)
    ref = O.raster_batched(oracle_frame(cam, bmin, QUIRKS[L.METHOD_LOOP_LAS]), want[0], n, *want[1:])
    got = fb.read(L.FB_U64)
    assert np.array_equal(got, ref), first_diff(got, ref)
    assert (got[: 320 * 240] != L.DEFAULT_CLEAR).sum() > 50
    fb.close()


def test_laz_beside_las_files(ctx, tmp_path):
    """A .las, a .LAZ and a .laz in one cloud: file indices, sparse offsets and
    boxMins as the LAS-only loader lays them out."""
    specs = [(2, 30_000, 7, "a.las"), (3, 25_000, 8, "b.LAZ"), (2, 12_345, 9, "c.laz")]
    paths, files = [], []
    for fmt, n, seed, name in specs:
        rec, bpp = laz_records(fmt, n, seed)
        bmin, bmax = laz_box(rec, n, bpp)
        writer = las.write_laz if name.lower().endswith("laz") else las.write_las
        paths.append(writer(tmp_path / name, rec, n, LAZ_SCALE, LAZ_OFFSET, bmin, bmax, point_format=fmt,
                            bytes_per_point=bpp))
        files.append((rec, n, bpp, fmt, np.array(bmin)))
    cloud, infos = las.load_files(ctx, paths)
    ctx.sync()
    point, batch = 0, 0
    for fi, (rec, n, bpp, fmt, bmin) in enumerate(files):
        want = oracle_layout(rec, n, bpp, fmt, bmin, point=point, file_index=fi)
        assert_cloud(cloud, want, b0=batch, p0=point)
        point += n
        batch += len(want[0])


def test_multi_window_file_equals_las_path(ctx, tmp_path):
    """3.1M points in load tasks of 1,024,000, decoded in windows of whole
    tasks through the pipelined upload (chunks of 50,000 and of 700,000
    points, some across window borders) and in one window on all threads:
    every load equals the LAS path of the same records."""
    n, fmt = 3_100_000, 2
    p = synth.synth_params(L.SYNTH_TERRAIN, 800.0, 12)
    rec, hdr = synth.las_records_host(p, n)
    lz = las.write_laz(tmp_path / "big.laz", rec, n, hdr.scale, hdr.offset, hdr.min, hdr.max, chunk_size=50000)
    ls = las.write_las(tmp_path / "big.las", rec, n, hdr.scale, hdr.offset, hdr.min, hdr.max)
    ref, _ = las.load_files(ctx, [ls])
    ctx.sync()
    want = [ref.read(0)] + [ref.read(s) for s in STREAMS]
    lz2 = las.write_laz(tmp_path / "big_var.laz", rec, n, hdr.scale, hdr.offset, hdr.min, hdr.max,
                        chunk_size=L.LAZ_VARIABLE_CHUNKS, var_chunk=700_000)
    # one-task windows on one thread and on two (pipelined, chunks across
    # window borders), 3-task windows of 700,000-point chunks on one thread,
    # one window on all threads
    for path, threads in ((lz, 1), (lz, 2), (lz2, 1), (lz, 0)):
        cloud, _ = las.load_files(ctx, [path], threads=threads)
        ctx.sync()
        assert np.array_equal(cloud.read(0).view(np.uint8), want[0].view(np.uint8)), (path, threads)
        for which, w in zip(STREAMS, want[1:]):
            assert np.array_equal(cloud.read(which), w), (path, threads, which)
        cloud.close()
