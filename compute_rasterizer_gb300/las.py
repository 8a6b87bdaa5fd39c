"""LAS files in and out, over include/cr_las.h.

`load_files` is the drop-in for the reference's LasLoaderSparse::add +
loader threads + process (LasLoaderSparse.cpp:477-713): files are numbered
in the order given, their points laid out back to back, every file's load
tasks encoded on the GPU, and each file's boxMin set for its world matrix.
`write_las` writes LAS 1.2 / 1.4 files (no VLRs) from point records, for
exporting synthetic clouds and for the tests.
"""
from __future__ import annotations

import ctypes as C
import struct
from pathlib import Path

import numpy as np

from . import _lib as L
from ._lib import CRError


def parse_header(data: bytes) -> L.LasInfo:
    info = L.LasInfo()
    buf = np.frombuffer(data, dtype=np.uint8)
    st = L.load().cr_las_parse_header(buf.ctypes.data, len(buf), C.byref(info))
    if st != L.OK:
        raise CRError(st, "not a LAS header")
    return info


def read_info(path) -> L.LasInfo:
    with open(path, "rb") as f:
        return parse_header(f.read(L.LAS_14_HEADER))


def read_records(path, info: L.LasInfo) -> np.ndarray:
    n, bpp = int(info.num_points), int(info.bytes_per_point)
    rec = np.fromfile(path, dtype=np.uint8, count=n * bpp, offset=int(info.offset_to_points))
    if rec.size != n * bpp:
        raise CRError(L.INVALID_ARG, f"{path}: {rec.size} point bytes, header says {n * bpp}")
    return rec


def load_files(ctx, paths, stream=None):
    """All files into one cloud on the GPU -> (Cloud, [LasInfo])."""
    lib = L.load()
    infos = [read_info(p) for p in paths]
    n = sum(int(i.num_points) for i in infos)
    nb = sum(int(lib.cr_las_num_batches(int(i.num_points))) for i in infos)
    cloud = ctx.cloud(n, nb, len(paths))
    point, batch = 0, 0
    for fi, (path, info) in enumerate(zip(paths, infos)):
        rec = read_records(path, info)
        ctx.check(lib.cr_cloud_load_las(ctx.handle, cloud.handle, rec.ctypes.data, int(info.num_points),
                                        C.byref(info), point, batch, fi, stream), f"load {path}")
        point += int(info.num_points)
        batch += int(lib.cr_las_num_batches(int(info.num_points)))
    cloud.set_files(np.array([i.min[:] for i in infos], dtype=np.float64))
    return cloud, infos


def write_las(path, records: np.ndarray, n: int, scale, offset, box_min, box_max,
              point_format: int = 2, bytes_per_point: int = L.LAS_FORMAT2_BYTES,
              version=(1, 2)):
    """A LAS file with the public header block and `n` records, no VLRs."""
    major, minor = version
    hsize = L.LAS_14_HEADER if (major, minor) >= (1, 4) else L.LAS_MIN_HEADER
    h = bytearray(hsize)
    h[0:4] = b"LASF"
    h[24], h[25] = major, minor
    h[26:58] = b"compute_rasterizer_gb300".ljust(32, b"\0")
    struct.pack_into("<H", h, 94, hsize)
    struct.pack_into("<I", h, 96, hsize)
    struct.pack_into("<I", h, 100, 0)
    h[104] = point_format
    struct.pack_into("<H", h, 105, bytes_per_point)
    struct.pack_into("<I", h, 107, n if n < 2**32 and point_format < 6 else 0)
    struct.pack_into("<3d", h, 131, *scale)
    struct.pack_into("<3d", h, 155, *offset)
    struct.pack_into("<6d", h, 179, box_max[0], box_min[0], box_max[1], box_min[1],
                     box_max[2], box_min[2])
    if hsize == L.LAS_14_HEADER:
        struct.pack_into("<Q", h, 247, n)
    rec = np.ascontiguousarray(records, dtype=np.uint8)[: n * bytes_per_point]
    with open(path, "wb") as f:
        f.write(bytes(h))
        f.write(rec.tobytes())
    return Path(path)
