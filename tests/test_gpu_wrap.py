"""Clouds over caller-owned arrays (cr_cloud_wrap): streams kept in pinned host
memory (and, where the device reads pageable memory, in plain host arrays)
render every method exactly as the same cloud uploaded to device memory."""
import numpy as np
import pytest
import torch

from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import default_params, make_view
from compute_rasterizer_gb300._lib import CRError
from compute_rasterizer_gb300.multiview import MultiView
from helpers import QUIRKS, cameras, encoded, first_diff, gpu_raw

pytestmark = pytest.mark.gpu


def padded(a, words):
    out = np.zeros(words, np.uint32)
    out[:len(a)] = a
    return out


def pinned(a):
    t = torch.from_numpy(np.ascontiguousarray(a).view(np.uint8)).pin_memory()
    assert t.is_pinned()
    return t


@pytest.fixture(scope="module")
def clouds(ctx):
    cl = encoded(n=62674, extent=200.0, seed=7)
    dev = ctx.cloud_from_arrays(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"], cl["box_min"])
    words = cl["n"] + 64
    streams = [padded(cl[k], words) for k in ("lo", "md", "hi", "rgba")]
    host = ctx.cloud_wrap(cl["n"], len(cl["batches"]), pinned(cl["batches"]),
                          *(pinned(s) for s in streams), box_min=cl["box_min"], stream_words=words)
    return cl, dev, host


@pytest.mark.parametrize("camname", ["far", "near", "mid"])
@pytest.mark.parametrize("method,payload", [(L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR),
                                            (L.METHOD_LOOP_LAS, L.PAYLOAD_INDEX),
                                            (L.METHOD_LOOP_LAS_PREFETCH, L.PAYLOAD_COLOR),
                                            (L.METHOD_LOOP_LAS_HQS, L.PAYLOAD_INDEX)])
def test_pinned_host_cloud_renders_as_device_cloud(ctx, clouds, camname, method, payload):
    cl, dev, host = clouds
    cam = cameras(cl)[camname]
    out = []
    for c in (dev, host):
        fb, params = gpu_raw(ctx, c, cam, method, payload)
        what = L.FB_DEPTH if method == L.METHOD_LOOP_LAS_HQS else L.FB_WORDS
        words = fb.read(what)
        extra = fb.read(L.FB_ACCUM) if method == L.METHOD_LOOP_LAS_HQS else None
        ctx.resolve(c, params, fb)
        out.append((words, extra, fb.read(L.FB_IMAGE)))
        fb.close()
    (a, ax, ai), (b, bx, bi) = out
    assert np.array_equal(a, b), first_diff(a, b)
    if ax is not None:
        assert np.array_equal(ax, bx)
    assert np.array_equal(ai, bi)
    assert (ai != L.BACKGROUND).sum() > 50


def test_multiview_over_host_cloud(ctx, clouds):
    cl, dev, host = clouds
    cams = list(cameras(cl).values())
    params = default_params(L.METHOD_LOOP_LAS, payload=L.PAYLOAD_COLOR, resolve=0, clear_after=0)
    got = []
    for c in (dev, host):
        mv = MultiView(ctx, c, [(cam[2], cam[3]) for cam in cams], params)
        mv.set_views([make_view(*cam) for cam in cams])
        mv.clear()
        mv.render()
        ctx.sync()
        got.append([mv.read(i, L.FB_WORDS) for i in range(len(cams))])
        mv.close()
    for a, b in zip(*got):
        assert np.array_equal(a, b)


def test_host_cloud_reads_back_and_refuses_upload(ctx, clouds):
    cl, dev, host = clouds
    assert np.array_equal(host.read(L.STREAM_LOW), cl["lo"])
    assert np.array_equal(host.read(0).view(np.uint8), np.ascontiguousarray(cl["batches"]).view(np.uint8))
    with pytest.raises(CRError) as e:
        host.upload(cl["batches"], cl["lo"], cl["md"], cl["hi"], cl["rgba"], cl["box_min"])
    assert e.value.status == L.INVALID_ARG


def test_wrap_rejects_short_streams(ctx, clouds):
    cl = clouds[0]
    lo = pinned(padded(cl["lo"], cl["n"] + 64))
    with pytest.raises(CRError) as e:
        ctx.cloud_wrap(cl["n"], len(cl["batches"]), pinned(cl["batches"]), lo, stream_words=cl["n"] + 10)
    assert e.value.status == L.INVALID_ARG


def test_pageable_host_arrays(ctx, clouds):
    """Plain host arrays: accepted only where the device reads pageable memory
    (then they render as the device cloud), refused otherwise."""
    cl, dev, _ = clouds
    words = cl["n"] + 64
    streams = [padded(cl[k], words) for k in ("lo", "md", "hi", "rgba")]
    batches = np.ascontiguousarray(cl["batches"])
    try:
        c = ctx.cloud_wrap(cl["n"], len(batches), batches, *streams, box_min=cl["box_min"],
                           stream_words=words)
    except CRError as e:
        assert e.status == L.INVALID_ARG
        return
    cam = cameras(cl)["near"]
    fa, _ = gpu_raw(ctx, dev, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR)
    fb, _ = gpu_raw(ctx, c, cam, L.METHOD_LOOP_LAS, L.PAYLOAD_COLOR)
    assert np.array_equal(fa.read(L.FB_WORDS), fb.read(L.FB_WORDS))
    fa.close()
    fb.close()
    c.close()
