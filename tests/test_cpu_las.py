"""LAS header parsing against the reference's own LAS 1.4 example file (its
bytes and independently decoded fields in tests/golden/las_5points_14.json),
and against files written by write_las; load-task batch counts."""
import json
from pathlib import Path

import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import las, synth
from compute_rasterizer_gb300._lib import CRError

FIX = json.loads((Path(__file__).parent / "golden" / "las_5points_14.json").read_text())


def check_fields(info, f):
    for k in ("version_major", "version_minor", "num_points", "offset_to_points", "point_format",
              "bytes_per_point"):
        assert getattr(info, k) == f[k], k
    for k in ("scale", "offset", "min", "max"):
        assert list(getattr(info, k)) == f[k], k


def test_reference_example_header():
    data = bytes.fromhex(FIX["bytes_hex"])
    assert len(data) == 1086
    check_fields(las.parse_header(data), FIX["fields"])


def test_rejects_what_is_not_a_las_header():
    data = bytearray.fromhex(FIX["bytes_hex"])
    with pytest.raises(CRError):
        las.parse_header(bytes(data[:226]))
    with pytest.raises(CRError):
        las.parse_header(bytes(data[:300]))  # 1.4 needs the 375-byte block
    bad = bytearray(data)
    bad[0:4] = b"LASG"
    with pytest.raises(CRError):
        las.parse_header(bytes(bad))
    short = bytearray(data)
    short[105:107] = (11).to_bytes(2, "little")
    with pytest.raises(CRError):
        las.parse_header(bytes(short))


@pytest.mark.parametrize("version", [(1, 2), (1, 4)])
def test_written_file_round_trips(tmp_path, version):
    n = 12345
    rec, hdr = synth.las_records_host(synth.synth_params(L.SYNTH_TERRAIN, 200.0, 9), n)
    p = las.write_las(tmp_path / "t.las", rec, n, hdr.scale, hdr.offset, hdr.min, hdr.max,
                      version=version)
    info = las.read_info(p)
    assert (info.version_major, info.version_minor) == version
    assert info.num_points == n and info.point_format == 2 and info.bytes_per_point == 26
    assert info.offset_to_points == (375 if version == (1, 4) else 227)
    for k in ("scale", "offset", "min", "max"):
        assert list(getattr(info, k)) == list(getattr(hdr, k)), k
    assert np.array_equal(las.read_records(p, info), rec)


def test_load_task_batch_counts():
    f = L.load().cr_las_num_batches
    assert [f(n) for n in (0, 1, 10240, 10241, 1024000, 1024001, 2048000, 2058240)] == \
        [0, 1, 1, 2, 100, 101, 200, 201]
