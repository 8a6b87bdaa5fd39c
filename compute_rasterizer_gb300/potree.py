"""Potree 2.0 octrees, over include/cr_potree.h.

`open_octree` / `Octree.load` are the drop-in for the reference's PotreeData
(modules/compute/PotreeData.h): metadata.json and hierarchy.bin are read
natively, octree.bin is encoded into the batched layout, one batch record per
node, and the cloud renders with CR_METHOD_LOOP_NODES.

`write_octree` writes a Potree 2.0 dataset (DEFAULT encoding, uncompressed
attributes) from LAS point records: an octree whose inner nodes keep a hashed
1/k sample of their points and pass the rest down, leaves of at most
`max_leaf` points, the hierarchy split into chunks of `chunk_levels` levels
with proxy entries, node boxes halved exactly as the reader derives them.  It
exports synthetic clouds and gives the tests datasets with a known node list.
"""
from __future__ import annotations

import ctypes as C
import json
import struct
from pathlib import Path

import numpy as np

from . import _lib as L
from ._lib import CRError, ptr


class Octree:
    """An opened Potree dataset (metadata and hierarchy parsed)."""

    def __init__(self, path):
        self.lib = L.load()
        self.path = Path(path)
        self.info = L.PotreeInfo()
        self.handle = None
        h = C.c_void_p()
        st = self.lib.cr_potree_open(str(self.path).encode(), C.byref(h), C.byref(self.info))
        if st != L.OK:
            raise CRError(st, f"cr_potree_open({path})")
        self.handle = h

    def nodes(self) -> list[dict]:
        n = int(self.info.num_nodes)
        arr = (L.PotreeNode * max(n, 1))()
        st = self.lib.cr_potree_nodes(self.handle, C.cast(arr, C.c_void_p), n)
        if st != L.OK:
            raise CRError(st, "cr_potree_nodes")
        return [dict(level=a.level, type=a.type, child_mask=a.child_mask, num_points=a.num_points,
                     byte_offset=a.byte_offset, byte_size=a.byte_size, min=tuple(a.min),
                     max=tuple(a.max)) for a in arr[:n]]

    def encode(self, quirks: int = L.POTREE_QUIRKS_DEFAULT):
        """octree.bin -> (batches, low, med, hig, rgba) on the host."""
        data = np.fromfile(self.path / "octree.bin", dtype=np.uint8)
        n, nb = int(self.info.num_points), int(self.info.num_nodes)
        batches = np.zeros(nb, L.BATCH_DTYPE)
        streams = [np.zeros(n, np.uint32) for _ in range(4)]
        st = self.lib.cr_potree_encode(self.handle, ptr(data), data.size, int(quirks), ptr(batches),
                                       *(ptr(s) for s in streams))
        if st != L.OK:
            raise CRError(st, "cr_potree_encode")
        return (batches, *streams)

    def load(self, ctx, quirks: int = L.POTREE_QUIRKS_DEFAULT, stream=None):
        """The encoded octree as a device cloud (one file at the origin)."""
        from .raster import Cloud
        h = C.c_void_p()
        ctx.check(self.lib.cr_potree_load(ctx.handle, self.handle, int(quirks), C.byref(h), stream),
                  "cr_potree_load")
        return Cloud(ctx, h, int(self.info.num_points), int(self.info.num_nodes), 1)

    def close(self):
        if self.handle:
            self.lib.cr_potree_close(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def open_octree(path) -> Octree:
    return Octree(path)


def _halve(mn, mx):
    """The split and the two children's bounds per axis, in float32 as
    createChildAABB computes them (PotreeData.h:112-140)."""
    fmn, fmx = np.float32(mn), np.float32(mx)
    half = ((fmx - fmn).astype(np.float32) / np.float32(2.0)).astype(np.float32)
    upper_min = (fmn + half).astype(np.float32)
    lower_max = (fmx - half).astype(np.float32)
    return fmn, fmx, upper_min, lower_max


def _child_box(mn, mx, index):
    fmn, fmx, upper_min, lower_max = _halve(mn, mx)
    cmn, cmx = fmn.copy(), fmx.copy()
    for k, bit in enumerate((4, 2, 1)):  # x, y, z
        if index & bit:
            cmn[k] = upper_min[k]
        else:
            cmx[k] = lower_max[k]
    return cmn.astype(np.float64), cmx.astype(np.float64)


def write_octree(path, records: np.ndarray, n: int, scale, offset, box_min, box_max,
                 bytes_per_point: int = L.LAS_FORMAT2_BYTES, max_leaf: int = 3000,
                 keep_every: int = 8, chunk_levels: int = 2, max_depth: int = 16):
    """Writes metadata.json, hierarchy.bin and octree.bin for LAS format-2
    records (X, Y, Z int32 at 0, 4, 8; R, G, B uint16 at 20).  Attributes:
    position (12 B), intensity (2 B), classification (1 B), rgb (6 B).
    Returns the node list in octree.bin order (preorder) for checks."""
    path = Path(path)
    path.mkdir(parents=True, exist_ok=True)
    rec = np.asarray(records, np.uint8).reshape(n, bytes_per_point)
    xyz = rec[:, :12].copy().view("<i4").reshape(n, 3)
    rgb = rec[:, 20:26].copy().view("<u2").reshape(n, 3)
    scale, offset = np.asarray(scale, np.float64), np.asarray(offset, np.float64)
    bmin, bmax = np.asarray(box_min, np.float64), np.asarray(box_max, np.float64)
    rel = xyz.astype(np.float64) * scale + offset - bmin

    nodes = []  # preorder: dict(level, min, max, idx, children)

    def build(idx, mn, mx, level):
        node = dict(level=level, min=mn, max=mx, children=[None] * 8)
        nodes.append(node)
        if len(idx) <= max_leaf or level >= max_depth:
            node["idx"] = idx
            return node
        h = ((idx.astype(np.uint64) * np.uint64(0x9E3779B1) + np.uint64(level * 0x85EBCA77 + 1))
             & np.uint64(0xFFFFFFFF)) >> np.uint64(16)
        sel = (h % np.uint64(keep_every)) == 0
        keep, rest = idx[sel], idx[~sel]
        node["idx"] = keep
        split = _halve(mn, mx)[2].astype(np.float64)
        r = rel[rest]
        octant = ((r[:, 0] >= split[0]) * 4 + (r[:, 1] >= split[1]) * 2 + (r[:, 2] >= split[2])).astype(int)
        for ci in range(8):
            sub = rest[octant == ci]
            if len(sub) == 0:
                continue
            cmn, cmx = _child_box(mn, mx, ci)
            node["children"][ci] = build(sub, cmn, cmx, level + 1)
        return node

    root = build(np.arange(n), np.zeros(3), bmax - bmin, 0)

    # octree.bin in preorder: position, intensity, classification, rgb
    bpp = 21
    off = 0
    parts = []
    for nd in nodes:
        idx = nd["idx"]
        nd["byte_offset"], nd["num_points"] = off, len(idx)
        out = np.zeros((len(idx), bpp), np.uint8)
        out[:, 0:12] = np.ascontiguousarray(xyz[idx], "<i4").view(np.uint8).reshape(-1, 12)
        out[:, 12:14] = np.ascontiguousarray((idx * 7) & 0xFFFF, "<u2").view(np.uint8).reshape(-1, 2)
        out[:, 14] = (idx % 5).astype(np.uint8)
        out[:, 15:21] = np.ascontiguousarray(rgb[idx], "<u2").view(np.uint8).reshape(-1, 6)
        parts.append(out.reshape(-1))
        nd["byte_size"] = out.size
        off += out.size
    (path / "octree.bin").write_bytes(np.concatenate(parts).tobytes() if parts else b"")

    # hierarchy.bin: chunks of `chunk_levels` levels, breadth first, proxies at the borders
    def is_proxy(nd, top):
        return nd is not top and nd["level"] - top["level"] >= chunk_levels

    def chunk_nodes(top):
        order, queue = [], [top]
        while queue:
            nd = queue.pop(0)
            order.append(nd)
            if is_proxy(nd, top):
                continue  # its subtree is its own chunk
            queue += [c for c in nd["children"] if c is not None]
        return order

    chunk_list, pending = [], [root]
    while pending:
        top = pending.pop(0)
        members = chunk_nodes(top)
        chunk_list.append((top, members))
        pending += [m for m in members if is_proxy(m, top)]
    pos = 0
    for top, members in chunk_list:
        top["chunk_offset"], top["chunk_size"] = pos, 22 * len(members)
        pos += 22 * len(members)
    blob = bytearray()
    for top, members in chunk_list:
        for nd in members:
            mask = sum(1 << ci for ci, c in enumerate(nd["children"]) if c is not None)
            if is_proxy(nd, top):
                blob += struct.pack("<BBIqq", 2, mask, nd["num_points"], nd["chunk_offset"],
                                    nd["chunk_size"])
            else:
                blob += struct.pack("<BBIqq", 0 if mask else 1, mask, nd["num_points"],
                                    nd["byte_offset"], nd["byte_size"])
    (path / "hierarchy.bin").write_bytes(bytes(blob))

    meta = {
        "version": "2.0", "name": "synthetic", "description": "", "points": int(n),
        "projection": "", "hierarchy": {"firstChunkSize": chunk_list[0][0]["chunk_size"],
                                        "stepSize": chunk_levels,
                                        "depth": max(d["level"] for d in nodes)},
        "offset": [float(x) for x in offset], "scale": [float(x) for x in scale],
        "spacing": float(np.max(bmax - bmin) / 128.0),
        "boundingBox": {"min": [float(x) for x in bmin], "max": [float(x) for x in bmax]},
        "encoding": "DEFAULT",
        "attributes": [
            {"name": "position", "description": "", "size": 12, "numElements": 3, "elementSize": 4,
             "type": "int32", "min": [float(x) for x in bmin], "max": [float(x) for x in bmax]},
            {"name": "intensity", "description": "", "size": 2, "numElements": 1, "elementSize": 2,
             "type": "uint16", "min": [0], "max": [65535]},
            {"name": "classification", "description": "", "size": 1, "numElements": 1,
             "elementSize": 1, "type": "uint8", "min": [0], "max": [4]},
            {"name": "rgb", "description": "", "size": 6, "numElements": 3, "elementSize": 2,
             "type": "uint16", "min": [0, 0, 0], "max": [65535, 65535, 65535]},
        ],
    }
    (path / "metadata.json").write_text(json.dumps(meta, indent=1))
    return [dict(level=d["level"], num_points=d["num_points"], byte_offset=d["byte_offset"],
                 byte_size=d["byte_size"], min=tuple(d["min"]), max=tuple(d["max"]),
                 child_mask=sum(1 << ci for ci, c in enumerate(d["children"]) if c is not None))
            for d in nodes]
