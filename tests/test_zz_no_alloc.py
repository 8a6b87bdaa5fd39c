"""cr_render_batched_noalloc against cr_render and the oracle.

Some callers cannot allocate device memory while they render: an engine that
owns the GPU memory budget and hands the renderer only buffers it already
placed, or a plugin running inside another application's frame loop, where a
cudaMalloc or cudaFree would synchronise or disturb the host's own device
work.  cr_render_batched_noalloc serves them: its work list (and the file
records of clouds with more than 8 files) lives in a fixed device array inside
the library instead of buffers it would allocate.  These tests render the same
frames through it and through cr_render and require identical framebuffers
(the tolerance of every parity test here: bit for bit), on two calls in a row,
because the array keeps the previous call's contents and each call must clear
what has to start at zero.  The array's address belongs to a CUDA context, so
one test renders in a second context made with the driver API (as a host
application may do, src/main.cpp:54-58 of the reference) after checking on the
host that the address the call uses is that context's own.  The file sits
where pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import default_params, make_view
from helpers import QUIRKS, cameras, encoded, first_diff, gpu_raw, oracle_frame
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MAX_BATCHES = L.NOALLOC_MAX_BATCHES


def call(lib, d, cloud_nb, cloud_n, box, nfiles, view, params, fb_ptr, stream=None, batches=None):
    return lib.cr_render_batched_noalloc(
        batches if batches is not None else d["batches"], cloud_nb, cloud_n, d["low"], d["med"],
        d["hig"], d["rgba"], cloud_n + 64, box.ctypes.data, nfiles, C.byref(view),
        C.byref(params), fb_ptr, stream)


@pytest.fixture(scope="module")
def small(ctx):
    cl = encoded(n=62674, extent=200.0, seed=7)
    cloud = ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"],
                                  cl["box_min"])
    yield cl, cloud
    cloud.close()


def test_noalloc_matches_cr_render_two_calls_in_a_row(ctx, small):
    lib = L.load()
    cl, cloud = small
    d = cloud.device_pointers()
    box = np.ascontiguousarray(cl["box_min"], np.float64)
    assert ctx.lib.cr_ctx_check(None, None) == L.OK  # no flag left by earlier work
    cases = [("far", L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR),
             ("near", L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX),
             ("mid", L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_INDEX),
             ("corner", L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_COLOR)]
    for camname, method, payload in cases:
        cam = cameras(cl)[camname]
        ref_fb, _ = gpu_raw(ctx, cloud, cam, method, payload)
        ref = ref_fb.read(L.FB_WORDS)
        want = O.raster_batched(oracle_frame(cam, cl["box_min"][None], QUIRKS[method], payload),
                                cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
        assert np.array_equal(ref, want), camname
        view = make_view(*cam)
        params = default_params(method, payload=payload, resolve=0, clear_after=0)
        out = ctx.framebuffer(cam[2], cam[3])
        for rep in range(2):
            out.clear()
            st = call(lib, d, cloud.nb, cloud.n, box, 1, view, params, out.device_pointer(L.FB_WORDS))
            assert st == L.OK, (camname, rep, st)
            ctx.sync()
            got = out.read(L.FB_WORDS)
            assert np.array_equal(got, ref), (camname, rep, first_diff(got, ref))
        assert (ref != L.DEFAULT_CLEAR).sum() > 50
        out.close()
        ref_fb.close()
    assert ctx.lib.cr_ctx_check(None, None) == L.OK


def test_noalloc_literal_arithmetic(ctx, small):
    """CR_QUIRK_LITERAL_ARITH through the no-allocation entry: the literal
    oracle's words, as cr_render gives them."""
    lib = L.load()
    cl, cloud = small
    d = cloud.device_pointers()
    box = np.ascontiguousarray(cl["box_min"], np.float64)
    for camname, method in (("far", L.METHOD_LOOP_LAS), ("near", L.METHOD_LOOP_LAS_PREFETCH)):
        cam = cameras(cl)[camname]
        quirks = QUIRKS[method] | L.QUIRK_LITERAL_ARITH
        with O.arith(O.ARITH_LITERAL):
            want = O.raster_batched(oracle_frame(cam, cl["box_min"][None], QUIRKS[method]),
                                    cl["batches"], cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
        params = default_params(method, resolve=0, clear_after=0, quirks=quirks)
        out = ctx.framebuffer(cam[2], cam[3])
        out.clear()
        assert call(lib, d, cloud.nb, cloud.n, box, 1, make_view(*cam), params,
                    out.device_pointer(L.FB_WORDS)) == L.OK
        ctx.sync()
        got = out.read(L.FB_WORDS)
        assert np.array_equal(got, want), (camname, first_diff(got, want))
        out.close()
    assert ctx.lib.cr_ctx_check(None, None) == L.OK


def test_noalloc_rejects_sizes_past_its_limit(ctx):
    lib = L.load()
    view = make_view(np.eye(4), np.eye(4), 64, 32)
    params = default_params(L.METHOD_LOOP_LAS, resolve=0, clear_after=0)
    box = np.zeros(3 * (L.NOALLOC_MAX_FILES + 1))
    dummy = 256  # never dereferenced: every call below is refused before any launch
    d = dict(batches=dummy, low=dummy, med=dummy, hig=dummy, rgba=dummy)

    def st(nb=1, n=1, nfiles=1, p=params):
        return call(lib, d, nb, n, box, nfiles, view, p, dummy)

    assert st(nb=MAX_BATCHES + 1) == L.INVALID_ARG
    assert st(nfiles=L.NOALLOC_MAX_FILES + 1) == L.INVALID_ARG
    assert st(nfiles=0) == L.INVALID_ARG
    assert st(p=default_params(L.METHOD_LOOP_LAS_HQS, resolve=0, clear_after=0)) == L.INVALID_ARG
    # it rasterizes only: a resolve or re-clear request is refused, not ignored
    assert st(p=default_params(L.METHOD_LOOP_LAS, resolve=1, clear_after=0)) == L.INVALID_ARG
    assert st(p=default_params(L.METHOD_LOOP_LAS, resolve=0, clear_after=1)) == L.INVALID_ARG
    addr, size = C.c_void_p(), C.c_int64()
    assert lib.cr_noalloc_scratch(C.byref(addr), C.byref(size)) == L.OK
    assert size.value == L.NOALLOC_SCRATCH_BYTES and addr.value


def test_noalloc_reports_a_skipped_record(ctx, small):
    """A batch record past the streams is skipped without a fault; the fixed
    array's error flag says so through cr_ctx_check(NULL, stream), which
    clears it."""
    import torch
    lib = L.load()
    cl, cloud = small
    d = cloud.device_pointers()
    bad = cl["batches"].copy()
    bad[2]["first_point"] = cl["n"]  # first_point + num_points beyond stream_words
    dev = torch.from_numpy(bad.view(np.uint8).copy()).cuda()
    cam = cameras(cl)["far"]
    params = default_params(L.METHOD_LOOP_LAS, resolve=0, clear_after=0)
    out = ctx.framebuffer(cam[2], cam[3])
    out.clear()
    box = np.ascontiguousarray(cl["box_min"], np.float64)
    torch.cuda.synchronize()
    st = call(lib, d, cloud.nb, cloud.n, box, 1, make_view(*cam), params,
              out.device_pointer(L.FB_WORDS), batches=dev.data_ptr())
    assert st == L.OK
    assert ctx.lib.cr_ctx_check(None, None) == L.DEVICE_FLAG
    assert ctx.lib.cr_ctx_check(None, None) == L.OK
    keep = np.delete(cl["batches"], 2)
    want = O.raster_batched(oracle_frame(cam, cl["box_min"][None], QUIRKS[L.METHOD_LOOP_LAS]),
                            keep, cl["n"], cl["lo"], cl["md"], cl["hi"], cl["rgba"])
    assert np.array_equal(out.read(L.FB_WORDS), want)
    out.close()


class _Driver:
    """The few driver-API calls a host application makes to own a context."""

    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        for name in ("cuInit", "cuDeviceGet", "cuCtxCreate_v2", "cuCtxDestroy_v2",
                     "cuCtxPopCurrent_v2", "cuCtxPushCurrent_v2", "cuCtxGetCurrent",
                     "cuCtxSynchronize", "cuMemAlloc_v2", "cuMemFree_v2", "cuMemcpyHtoD_v2",
                     "cuMemcpyDtoH_v2", "cuMemsetD32_v2", "cuPointerGetAttribute"):
            getattr(self.cu, name).restype = C.c_int

    def ok(self, r, what):
        assert r == 0, f"{what}: CUresult {r}"

    def alloc_copy(self, host: np.ndarray) -> int:
        p = C.c_uint64()
        self.ok(self.cu.cuMemAlloc_v2(C.byref(p), C.c_size_t(max(host.nbytes, 16))), "cuMemAlloc")
        self.ok(self.cu.cuMemcpyHtoD_v2(p, C.c_void_p(host.ctypes.data), C.c_size_t(host.nbytes)),
                "cuMemcpyHtoD")
        return p.value


def test_noalloc_in_a_second_driver_context(ctx, small):
    lib = L.load()
    cl, cloud = small
    cam = cameras(cl)["far"]
    method, payload = L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR
    ref_fb, _ = gpu_raw(ctx, cloud, cam, method, payload)
    ref = ref_fb.read(L.FB_WORDS)
    ref_fb.close()
    addr_a = C.c_void_p()
    size = C.c_int64()
    assert lib.cr_noalloc_scratch(C.byref(addr_a), C.byref(size)) == L.OK

    drv = _Driver()
    cu = drv.cu
    dev = C.c_int()
    drv.ok(cu.cuInit(0), "cuInit")
    drv.ok(cu.cuDeviceGet(C.byref(dev), 0), "cuDeviceGet")
    ctx_b = C.c_void_p()
    drv.ok(cu.cuCtxCreate_v2(C.byref(ctx_b), 0, dev), "cuCtxCreate")  # current on this thread
    bufs = []
    try:
        cur = C.c_void_p()
        drv.ok(cu.cuCtxGetCurrent(C.byref(cur)), "cuCtxGetCurrent")
        assert cur.value == ctx_b.value
        # host side, before any launch in this context: the address the call
        # will use belongs to this context, not to the primary one
        addr_b = C.c_void_p()
        assert lib.cr_noalloc_scratch(C.byref(addr_b), C.byref(size)) == L.OK
        owner = C.c_void_p()
        drv.ok(cu.cuPointerGetAttribute(C.byref(owner), 1, C.c_uint64(addr_b.value)),
               "CU_POINTER_ATTRIBUTE_CONTEXT")
        assert owner.value == ctx_b.value
        assert addr_b.value != addr_a.value

        n = cl["n"]
        streams = {k: O.pad_stream(cl[k], n=n) for k in ("lo", "md", "hi", "rgba")}
        d = {"batches": drv.alloc_copy(np.ascontiguousarray(cl["batches"])),
             "low": drv.alloc_copy(streams["lo"]), "med": drv.alloc_copy(streams["md"]),
             "hig": drv.alloc_copy(streams["hi"]), "rgba": drv.alloc_copy(streams["rgba"])}
        bufs += list(d.values())
        words = cam[2] * cam[3] + cam[2] + 1
        fb = C.c_uint64()
        drv.ok(cu.cuMemAlloc_v2(C.byref(fb), C.c_size_t(words * 8)), "cuMemAlloc fb")
        bufs.append(fb.value)
        box = np.ascontiguousarray(cl["box_min"], np.float64)
        params = default_params(method, payload=payload, resolve=0, clear_after=0)
        for rep in range(2):
            # 0xFF800000FF800000 in every word: the clear cr_fb_clear writes
            drv.ok(cu.cuMemsetD32_v2(fb, C.c_uint(0xFF800000), C.c_size_t(2 * words)), "cuMemsetD32")
            st = lib.cr_render_batched_noalloc(d["batches"], cloud.nb, n, d["low"], d["med"],
                                               d["hig"], d["rgba"], n + 64, box.ctypes.data, 1,
                                               C.byref(make_view(*cam)), C.byref(params),
                                               fb.value, None)
            assert st == L.OK, st
            drv.ok(cu.cuCtxSynchronize(), "cuCtxSynchronize")
            got = np.empty(words, np.uint64)
            drv.ok(cu.cuMemcpyDtoH_v2(C.c_void_p(got.ctypes.data), fb, C.c_size_t(words * 8)),
                   "cuMemcpyDtoH")
            assert np.array_equal(got, ref), (rep, first_diff(got, ref))
        assert lib.cr_ctx_check(None, None) == L.OK
    finally:
        for p in bufs:
            cu.cuMemFree_v2(C.c_uint64(p))
        popped = C.c_void_p()
        cu.cuCtxPopCurrent_v2(C.byref(popped))
        cu.cuCtxDestroy_v2(ctx_b)
    # back in the primary context: its own address, and a frame still renders
    again = C.c_void_p()
    assert lib.cr_noalloc_scratch(C.byref(again), C.byref(size)) == L.OK
    assert again.value == addr_a.value
    d = cloud.device_pointers()
    out = ctx.framebuffer(cam[2], cam[3])
    out.clear()
    assert call(lib, d, cloud.nb, cloud.n, np.ascontiguousarray(cl["box_min"], np.float64), 1,
                make_view(*cam), default_params(method, payload=payload, resolve=0, clear_after=0),
                out.device_pointer(L.FB_WORDS)) == L.OK
    ctx.sync()
    assert np.array_equal(out.read(L.FB_WORDS), ref)
    out.close()
