"""Host side of the frame server: the request generator of the serving
workload, pool accounting, the ctypes mirror of include/cr_serve.h."""
import ctypes as C

import numpy as np

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import workloads
from compute_rasterizer_gb300.serve import COMPLETION_DTYPE, latency_summary, request_bytes


def test_struct_layouts_match_the_header():
    # cr_request: cloud, pad, cr_view (2 x 16 doubles + 2 ints), pointer, tag
    assert C.sizeof(L.View) == 264
    assert C.sizeof(L.Request) == 8 + 264 + 8 + 8
    assert C.sizeof(L.Completion) == 8 + 8 + 4 + 4 + 3 * 8
    assert C.sizeof(L.ServerConfig) == 8 + 10 * 4 + 6 * 4
    assert COMPLETION_DTYPE.itemsize == C.sizeof(L.Completion)


def test_request_bytes_rounds_each_buffer():
    assert request_bytes(64, 48) == 25344 + 12288  # (3072 + 65) * 8 = 25096 -> 25344
    assert request_bytes(1920, 1080) % 256 == 0
    assert request_bytes(3840, 2160) < L.SERVE_MAX_POOL_BYTES


def test_serving_requests_are_seeded_poisson_zipf(built):
    boxes = [(np.zeros(3), np.array([100.0 * (i + 1), 100.0 * (i + 1), 20.0])) for i in range(8)]
    a1, c1 = workloads.serving_requests(boxes, 4000, rate=1000.0, seed=5)
    a2, c2 = workloads.serving_requests(boxes, 4000, rate=1000.0, seed=5)
    assert np.array_equal(a1, a2) and [c[0] for c in c1] == [c[0] for c in c2]
    assert a1[0] == 0.0 and (np.diff(a1) >= 0).all()
    # mean gap 1 ms within 5 %
    assert abs(np.diff(a1).mean() - 1000.0) < 50.0
    counts = np.bincount([c[0] for c in c1], minlength=8) / 4000
    w = workloads.zipf_weights(8, 1.1)
    assert np.abs(counts - w).max() < 0.03
    sizes = {(c[3], c[4]) for c in c1}
    assert sizes == set(workloads.SERVING_RESOLUTIONS)


def test_latency_summary_counts_rejections():
    d = np.zeros(4, dtype=COMPLETION_DTYPE)
    d["status"] = [L.OK, L.OK, L.ADMISSION_REJECTED, L.OK]
    d["t_arrival_us"] = [0, 100, 200, 300]
    d["t_done_us"] = [1000, 1100, 0, 2300]
    d["batch_views"] = [2, 2, 0, 1]
    s = latency_summary(d)
    assert s["completed"] == 3 and s["rejected"] == 1 and s["failed"] == 0
    assert s["p50_ms"] == 1.0
    assert abs(s["served_req_per_s"] - 3 / 2.3e-3) < 1e-6
