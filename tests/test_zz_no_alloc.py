"""cr_render_batched_noalloc against cr_render.

Some callers cannot allocate device memory while they render: an engine that
owns the GPU memory budget, a plugin running inside another application's
frame loop, or code recorded into a CUDA graph, where cudaMalloc and cudaFree
synchronise the device or are not allowed.  cr_render_batched_noalloc serves
them: its work list lives in a fixed device array inside the library instead
of a buffer it would allocate.  This test renders the same frames through it
and through cr_render and requires identical framebuffers (the tolerance of
every parity test here: bit for bit), on two calls in a row, because the
array keeps the previous call's contents and each call must clear what has to
start at zero.  It sits in a file that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import default_params, make_view
from helpers import cameras, encoded, first_diff, gpu_raw

pytestmark = pytest.mark.gpu

MAX_BATCHES = 131064  # CR_NOALLOC_MAX_BATCHES


def test_noalloc_matches_cr_render_two_calls_in_a_row(ctx):
    lib = L.load()
    cl = encoded(n=62674, extent=200.0, seed=7)
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"],
                                  cl["box_min"])
    d = cloud.device_pointers()
    box = np.ascontiguousarray(cl["box_min"], np.float64)
    cases = [("far", L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR),
             ("near", L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX),
             ("mid", L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_INDEX),
             ("corner", L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_COLOR)]
    for camname, method, payload in cases:
        cam = cameras(cl)[camname]
        ref_fb, _ = gpu_raw(ctx, cloud, cam, method, payload)
        ref = ref_fb.read(L.FB_WORDS)
        view = make_view(*cam)
        params = default_params(method, payload=payload, resolve=0, clear_after=0)
        out = ctx.framebuffer(cam[2], cam[3])
        for call in range(2):
            out.clear()
            st = lib.cr_render_batched_noalloc(
                d["batches"], cloud.nb, cloud.n, d["low"], d["med"], d["hig"], d["rgba"],
                cloud.n + 64, box.ctypes.data, 1, C.byref(view), C.byref(params),
                out.device_pointer(L.FB_WORDS), None)
            assert st == L.OK, (camname, call, st)
            ctx.sync()
            got = out.read(L.FB_WORDS)
            assert np.array_equal(got, ref), (camname, call, first_diff(got, ref))
        assert (ref != L.DEFAULT_CLEAR).sum() > 50


def test_noalloc_rejects_sizes_past_its_limit(ctx):
    lib = L.load()
    view = make_view(np.eye(4), np.eye(4), 64, 32)
    params = default_params(L.METHOD_LOOP_LAS, resolve=0, clear_after=0)
    box = np.zeros(3)
    dummy = 256  # never dereferenced: the call is refused before any launch
    st = lib.cr_render_batched_noalloc(dummy, MAX_BATCHES + 1, 1, dummy, dummy, dummy, dummy, 128,
                                       box.ctypes.data, 1, C.byref(view), C.byref(params), dummy,
                                       None)
    assert st == L.INVALID_ARG
    hqs = default_params(L.METHOD_LOOP_LAS_HQS, resolve=0, clear_after=0)
    st = lib.cr_render_batched_noalloc(dummy, 1, 1, dummy, dummy, dummy, dummy, 128,
                                       box.ctypes.data, 1, C.byref(view), C.byref(hqs), dummy, None)
    assert st == L.INVALID_ARG
