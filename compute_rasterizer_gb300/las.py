"""LAS and LAZ files in and out, over include/cr_las.h and include/cr_laz.h.

`load_files` is the drop-in for the reference's LasLoaderSparse::add +
loader threads + process (LasLoaderSparse.cpp:477-713): files are numbered
in the order given, their points laid out back to back, every file's load
tasks encoded on the GPU, and each file's boxMin set for its world matrix.
Paths ending in "laz" (any case, as the reference's iEndsWith) are decoded
by the native LASzip reader on host threads (loadLaz, :214-429); the rest
are read as LAS (loadLas).  `write_las` / `write_laz` write LAS 1.2 / 1.4
files from point records, for exporting synthetic clouds and for the tests.
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


def is_laz(path) -> bool:
    return str(path).lower().endswith("laz")


class LazFile:
    """A LAZ file read into memory with its LASzip VLR and chunk table parsed."""

    def __init__(self, path_or_bytes):
        self.lib = L.load()
        if isinstance(path_or_bytes, (bytes, bytearray, np.ndarray)):
            self.data = np.frombuffer(bytes(path_or_bytes), dtype=np.uint8)
        else:
            self.data = np.fromfile(path_or_bytes, dtype=np.uint8)
        self.info = L.LazInfo()
        h = C.c_void_p()
        st = self.lib.cr_laz_open(self.data.ctypes.data, self.data.size, C.byref(h), C.byref(self.info))
        if st != L.OK:
            raise CRError(st, "cr_laz_open: " + self.lib.cr_status_string(st).decode())
        self.handle = h

    @property
    def num_points(self) -> int:
        return int(self.info.las.num_points)

    def decode(self, first: int = 0, n: int | None = None, threads: int = 0) -> np.ndarray:
        """Points [first, first + n) as LAS records (uint8, n * bytes_per_point)."""
        n = self.num_points - first if n is None else n
        out = np.zeros(n * int(self.info.las.bytes_per_point), np.uint8)
        st = self.lib.cr_laz_decode(self.handle, first, n, out.ctypes.data, threads)
        if st != L.OK:
            raise CRError(st, "cr_laz_decode: " + self.lib.cr_status_string(st).decode())
        return out

    def close(self):
        if getattr(self, "handle", None):
            self.lib.cr_laz_close(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def load_files(ctx, paths, stream=None, threads: int = 0):
    """All files into one cloud on the GPU -> (Cloud, [LasInfo])."""
    lib = L.load()
    lazs = {i: LazFile(p) for i, p in enumerate(paths) if is_laz(p)}
    infos = [lazs[i].info.las if i in lazs else read_info(p) for i, p in enumerate(paths)]
    n = sum(int(i.num_points) for i in infos)
    nb = sum(int(lib.cr_las_num_batches(int(i.num_points))) for i in infos)
    cloud = ctx.cloud(n, nb, len(paths))
    point, batch = 0, 0
    for fi, (path, info) in enumerate(zip(paths, infos)):
        if fi in lazs:
            ctx.check(lib.cr_cloud_load_laz(ctx.handle, cloud.handle, lazs[fi].handle, point, batch, fi,
                                            threads, stream), f"load {path}")
            lazs[fi].close()
        else:
            rec = read_records(path, info)
            ctx.check(lib.cr_cloud_load_las(ctx.handle, cloud.handle, rec.ctypes.data, int(info.num_points),
                                            C.byref(info), point, batch, fi, stream), f"load {path}")
        point += int(info.num_points)
        batch += int(lib.cr_las_num_batches(int(info.num_points)))
    cloud.set_files(np.array([i.min[:] for i in infos], dtype=np.float64))
    return cloud, infos


def _header(n, scale, offset, box_min, box_max, point_format, bytes_per_point, version, vlrs=()):
    """The public header block and VLRs (user id, record id, payload)."""
    major, minor = version
    hsize = L.LAS_14_HEADER if (major, minor) >= (1, 4) else L.LAS_MIN_HEADER
    h = bytearray(hsize)
    h[0:4] = b"LASF"
    h[24], h[25] = major, minor
    h[26:58] = b"compute_rasterizer_gb300".ljust(32, b"\0")
    body = bytearray()
    for user, rid, payload in vlrs:
        body += struct.pack("<H16sHH32s", 0, user.encode().ljust(16, b"\0"), rid, len(payload),
                            b"compute_rasterizer_gb300".ljust(32, b"\0"))
        body += bytes(payload)
    struct.pack_into("<H", h, 94, hsize)
    struct.pack_into("<I", h, 96, hsize + len(body))
    struct.pack_into("<I", h, 100, len(vlrs))
    h[104] = point_format
    struct.pack_into("<H", h, 105, bytes_per_point)
    struct.pack_into("<I", h, 107, n if n < 2**32 and (point_format & 63) < 6 else 0)
    struct.pack_into("<3d", h, 131, *scale)
    struct.pack_into("<3d", h, 155, *offset)
    struct.pack_into("<6d", h, 179, box_max[0], box_min[0], box_max[1], box_min[1],
                     box_max[2], box_min[2])
    if hsize == L.LAS_14_HEADER:
        struct.pack_into("<Q", h, 247, n)
    return bytes(h) + bytes(body)


def write_las(path, records: np.ndarray, n: int, scale, offset, box_min, box_max,
              point_format: int = 2, bytes_per_point: int = L.LAS_FORMAT2_BYTES,
              version=(1, 2)):
    """A LAS file with the public header block and `n` records, no VLRs."""
    head = _header(n, scale, offset, box_min, box_max, point_format, bytes_per_point, version)
    rec = np.ascontiguousarray(records, dtype=np.uint8)[: n * bytes_per_point]
    with open(path, "wb") as f:
        f.write(head)
        f.write(rec.tobytes())
    return Path(path)


def laz_bytes(records: np.ndarray, n: int, scale, offset, box_min, box_max, point_format: int = 2,
              bytes_per_point: int = L.LAS_FORMAT2_BYTES, version=(1, 2),
              chunk_size: int = L.LAZ_DEFAULT_CHUNK, var_chunk: int = 0, threads: int = 0) -> bytes:
    """A LAZ file (LAS header with the point format's compression bit, the
    LASzip VLR, the compressed points) as bytes."""
    lib = L.load()
    vlr = np.zeros(34 + 6 * L.LAZ_MAX_ITEMS, np.uint8)
    vlen = C.c_int64()
    st = lib.cr_laz_vlr(point_format, bytes_per_point, chunk_size, vlr.ctypes.data, vlr.size, C.byref(vlen))
    if st != L.OK:
        raise CRError(st, "cr_laz_vlr")
    head = _header(n, scale, offset, box_min, box_max, point_format | 128, bytes_per_point, version,
                   [("laszip encoder", 22204, vlr[: vlen.value].tobytes())])
    rec = np.ascontiguousarray(records, dtype=np.uint8)[: n * bytes_per_point]
    cap = int(lib.cr_laz_compress_bound(n, bytes_per_point, chunk_size if chunk_size > 0 else var_chunk))
    out = np.zeros(cap, np.uint8)
    size = C.c_int64()
    st = lib.cr_laz_compress(rec.ctypes.data, n, point_format, bytes_per_point, chunk_size, var_chunk,
                             len(head), out.ctypes.data, cap, C.byref(size), threads)
    if st != L.OK:
        raise CRError(st, "cr_laz_compress")
    return head + out[: size.value].tobytes()


def write_laz(path, records: np.ndarray, n: int, scale, offset, box_min, box_max, **kw):
    """write_las's LAZ counterpart (keywords as laz_bytes)."""
    Path(path).write_bytes(laz_bytes(records, n, scale, offset, box_min, box_max, **kw))
    return Path(path)
