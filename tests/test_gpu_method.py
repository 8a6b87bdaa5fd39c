"""A reference-style frame loop in C++ through include/cr_method.hpp renders
the same images as the Python host layer."""
import subprocess

import numpy as np
import pytest

import compute_rasterizer_gb300 as cr
from compute_rasterizer_gb300 import _lib as L
from compute_rasterizer_gb300 import synth
from helpers import build_method_demo, first_diff

pytestmark = pytest.mark.gpu

N, SEED, EXTENT, W, H = 300_000, 3, 300.0, 320, 240


@pytest.mark.parametrize("method", ["loop_las", "loop_las_prefetch", "loop_las_hqs"])
def test_cpp_method_adapter_equals_python_render(ctx, tmp_path, method):
    exe = build_method_demo(tmp_path)
    cloud, hdr = synth.build_cloud_device(ctx, synth.synth_params(L.SYNTH_TERRAIN, EXTENT, SEED), N)
    bmin, bmax = np.array(hdr.min[:]), np.array(hdr.max[:])
    yaw, pitch, radius, target = synth.zoom_to_cloud(bmin, bmax)
    view = synth.orbit_view(yaw + 0.3, pitch, radius * 0.6, target)
    proj = synth.perspective(60.0, W / H, 0.1, 200000.0)
    cam = tmp_path / "cam.f64"
    np.concatenate([view, proj]).astype(np.float64).tofile(cam)
    out = tmp_path / "img.u32"
    res = subprocess.run([str(exe), "render", str(cam), str(out), method, str(N), str(SEED),
                          str(EXTENT), str(W), str(H)], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, (res.returncode, res.stderr)
    got = np.fromfile(out, dtype=np.uint32)

    mid = {"loop_las": L.METHOD_LOOP_LAS, "loop_las_prefetch": L.METHOD_LOOP_LAS_PREFETCH,
           "loop_las_hqs": L.METHOD_LOOP_LAS_HQS}[method]
    kind = L.FB_HQS if mid == L.METHOD_LOOP_LAS_HQS else L.FB_U64
    fb = ctx.framebuffer(W, H, kind)
    fb.clear(0xFF800000 if kind == L.FB_HQS else L.DEFAULT_CLEAR)
    ctx.render(cloud, cr.make_view(view, proj, W, H), cr.default_params(mid), fb)
    ctx.sync()
    want = fb.read(L.FB_IMAGE)
    assert got.shape == want.shape
    assert np.array_equal(got, want), first_diff(got, want)
    assert (want != L.BACKGROUND).sum() > 1000
    fb.close()
    cloud.close()
