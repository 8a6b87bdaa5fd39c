"""Synthetic clouds, cameras and the host layout builder, over the C ABI.

Cameras follow the reference's host code: Camera::update (Camera.h:34-39,
perspective from a vertical fov in degrees) and OrbitControls::update
(OrbitControls.h:116-135); the "zoom to point cloud" pose is the one
src/main.cpp:251-270 sets when a file is dropped.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib as L
from ._lib import CRError, ptr


def perspective(fovy_deg: float, aspect: float, znear: float, zfar: float) -> np.ndarray:
    out = np.zeros(16, dtype=np.float64)
    L.load().cr_perspective(fovy_deg, aspect, znear, zfar, ptr(out))
    return out


def look_at(eye, center, up) -> np.ndarray:
    out = np.zeros(16, dtype=np.float64)
    e, c, u = (np.ascontiguousarray(x, dtype=np.float64) for x in (eye, center, up))
    L.load().cr_look_at(ptr(e), ptr(c), ptr(u), ptr(out))
    return out


def orbit_view(yaw: float, pitch: float, radius: float, target) -> np.ndarray:
    out = np.zeros(16, dtype=np.float64)
    t = np.ascontiguousarray(target, dtype=np.float64)
    L.load().cr_orbit_view(yaw, pitch, radius, ptr(t), ptr(out))
    return out


def zoom_to_cloud(box_min, box_max):
    """(yaw, pitch, radius, target) of src/main.cpp:251-270."""
    bmin, bmax = np.asarray(box_min, np.float64), np.asarray(box_max, np.float64)
    size = bmax - bmin
    target = (bmax + bmin) / 2.0
    radius = math.sqrt(float(size[0] * size[0] + size[1] * size[1] + size[2] * size[2])) / 1.5
    return 0.53, -0.68, radius, target


def camera(width: int, height: int, view: np.ndarray, fovy: float = 60.0, znear: float = 0.1,
           zfar: float = 200000.0):
    """(view, proj, width, height) with Camera.h's defaults (fovy 60, near 0.1, far 200000)."""
    proj = perspective(fovy, width / height, znear, zfar)
    return view, proj, width, height


def synth_params(kind: int = L.SYNTH_TERRAIN, extent: float = 1000.0, seed: int = 1,
                 **kw) -> L.SynthParams:
    p = L.SynthParams()
    L.load().cr_synth_params_default(int(kind), float(extent), int(seed), C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def las_records_host(params: L.SynthParams, n: int, morton: bool = True):
    """LAS format-2 records (n x 26 bytes) and header, generated on the host."""
    lib = L.load()
    rec = np.empty(n * L.LAS_FORMAT2_BYTES, dtype=np.uint8)
    hdr = L.LasHeader()
    st = lib.cr_synth_points_host(C.byref(params), n, ptr(rec), C.byref(hdr))
    if st != L.OK:
        raise CRError(st, "cr_synth_points_host")
    if morton:
        st = lib.cr_morton_sort_host(ptr(rec), n, L.LAS_FORMAT2_BYTES, C.byref(hdr))
        if st != L.OK:
            raise CRError(st, "cr_morton_sort_host")
    return rec, hdr


def header_min(hdr: L.LasHeader) -> np.ndarray:
    return np.array(hdr.min[:], dtype=np.float64)


def header_max(hdr: L.LasHeader) -> np.ndarray:
    return np.array(hdr.max[:], dtype=np.float64)


def encode_las(records: np.ndarray, n: int, hdr: L.LasHeader, bytes_per_point: int = 26,
               point_format: int = 2, sparse_offset: int = 0, file_index: int = 0,
               box_min=None):
    """Host layout builder (LasLoaderSparse.cpp:37-212) -> (batches, low, med, hig, rgba)."""
    lib = L.load()
    nb = int(lib.cr_num_batches(n))
    batches = np.zeros(nb, dtype=L.BATCH_DTYPE)
    streams = [np.zeros(n, dtype=np.uint32) for _ in range(4)]
    scale = np.array(hdr.scale[:], np.float64)
    offset = np.array(hdr.offset[:], np.float64)
    bmin = np.asarray(header_min(hdr) if box_min is None else box_min, np.float64)
    st = lib.cr_encode_las(ptr(records), n, bytes_per_point, point_format, ptr(scale), ptr(offset),
                           ptr(bmin), sparse_offset, file_index, ptr(batches),
                           *(ptr(s) for s in streams))
    if st != L.OK:
        raise CRError(st, "cr_encode_las")
    return (batches, *streams)


def uniform_vertices_host(seed: int, n: int, size: float = 100.0) -> np.ndarray:
    v = np.empty(n, dtype=L.VERTEX_DTYPE)
    st = L.load().cr_synth_uniform_host(seed, n, size, ptr(v))
    if st != L.OK:
        raise CRError(st, "cr_synth_uniform_host")
    return v


def build_cloud_device(ctx, params: L.SynthParams, n: int, stream=None):
    """Generate, Morton-sort and encode `n` points on the GPU -> (Cloud, header)."""
    lib = L.load()
    cloud = ctx.cloud(n, int(lib.cr_num_batches(n)), 1)
    hdr = L.LasHeader()
    ctx.check(lib.cr_synth_cloud_device(ctx.handle, C.byref(params), n, cloud.handle,
                                        C.byref(hdr), stream), "cr_synth_cloud_device")
    return cloud, hdr


def build_cloud_device_timed(ctx, params: L.SynthParams, n: int, stream=None):
    """build_cloud_device stage by stage (generate, Morton sort, encode), each
    timed with CUDA events on `stream` -> (Cloud, header, {stage: ms})."""
    import torch
    lib = L.load()
    cloud = ctx.cloud(n, int(lib.cr_num_batches(n)), 1)
    hdr = L.LasHeader()
    rec = torch.empty(n * L.LAS_FORMAT2_BYTES, dtype=torch.uint8, device="cuda")
    st = torch.cuda.ExternalStream(stream) if stream else torch.cuda.current_stream()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    torch.cuda.synchronize()
    ev[0].record(st)
    ctx.check(lib.cr_synth_points_device(ctx.handle, C.byref(params), n, rec.data_ptr(),
                                         C.byref(hdr), stream), "generate")
    ev[1].record(st)
    ctx.check(lib.cr_morton_sort_device(ctx.handle, rec.data_ptr(), n, L.LAS_FORMAT2_BYTES,
                                        C.byref(hdr), stream), "Morton sort")
    ev[2].record(st)
    d = cloud.device_pointers()
    sc, of, mn = (np.ascontiguousarray(x[:], np.float64) for x in (hdr.scale, hdr.offset, hdr.min))
    ctx.check(lib.cr_encode_las_device(ctx.handle, rec.data_ptr(), n, L.LAS_FORMAT2_BYTES, 2,
                                       ptr(sc), ptr(of), ptr(mn), 0, 0, d["batches"], d["low"],
                                       d["med"], d["hig"], d["rgba"], stream), "encode")
    ev[3].record(st)
    ctx.sync(stream)
    cloud.set_files(mn)
    del rec
    torch.cuda.empty_cache()
    ms = {k: round(ev[i].elapsed_time(ev[i + 1]), 2)
          for i, k in enumerate(("generate", "morton_sort", "encode"))}
    ms["total"] = round(sum(ms.values()), 2)
    return cloud, hdr, ms


def uniform_cloud_device(ctx, seed: int, n: int, size: float = 100.0, stream=None):
    cloud = ctx.plain_cloud_empty(n)
    ctx.check(L.load().cr_synth_uniform_device(ctx.handle, seed, n, size, cloud.vertices_pointer(),
                                               stream), "cr_synth_uniform_device")
    ctx.sync(stream)
    return cloud
