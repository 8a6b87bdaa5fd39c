"""Python handle over the multi-view plan (cr_mv_* in include/cr_raster.h)."""
from __future__ import annotations

import ctypes as C
import json

import numpy as np

from . import _lib as L
from ._lib import CRError, ptr


class MultiView:
    """Many views of one cloud rendered by one persistent launch per frame."""

    def __init__(self, ctx, cloud, sizes, params: L.RenderParams):
        self.ctx, self.lib = ctx, ctx.lib
        self.sizes = [(int(w), int(h)) for w, h in sizes]
        w = np.array([s[0] for s in self.sizes], np.int32)
        h = np.array([s[1] for s in self.sizes], np.int32)
        hd = C.c_void_p()
        st = self.lib.cr_mv_create(ctx.handle, cloud.handle, len(self.sizes), ptr(w), ptr(h),
                                   C.byref(params), C.byref(hd))
        if st != L.OK:
            raise CRError(st, "cr_mv_create: " + self.lib.cr_status_string(st).decode())
        self.handle = hd

    def _check(self, st, what):
        if st != L.OK:
            msg = self.lib.cr_mv_last_error(self.handle).decode()
            raise CRError(st, f"{what}: {self.lib.cr_status_string(st).decode()}: {msg}")

    def set_params(self, params: L.RenderParams):
        self._check(self.lib.cr_mv_set_params(self.handle, C.byref(params)), "set params")

    def get_params(self) -> L.RenderParams:
        p = L.RenderParams()
        self._check(self.lib.cr_mv_get_params(self.handle, C.byref(p)), "get params")
        return p

    def set_views(self, views):
        arr = (L.View * len(views))(*views)
        self._check(self.lib.cr_mv_set_views(self.handle, arr), "set views")

    def shared_pairs(self) -> int:
        """View pairs whose y / w projection rows the frame computes once."""
        n = C.c_int32()
        self._check(self.lib.cr_mv_shared_pairs(self.handle, C.byref(n)), "shared pairs")
        return n.value

    def render(self, use_graph: bool = False, stream=None):
        self._check(self.lib.cr_mv_render(self.handle, int(use_graph), stream), "render")

    def clear(self, value: int = L.DEFAULT_CLEAR, stream=None):
        self._check(self.lib.cr_mv_clear(self.handle, C.c_uint64(value), stream), "clear")

    def read(self, view: int, what: int, stream=None) -> np.ndarray:
        w, h = self.sizes[view]
        if what == L.FB_WORDS:
            out = np.empty(w * h + w + 1, np.uint64)
        else:
            out = np.empty(w * h, np.uint32)
        self._check(self.lib.cr_mv_read(self.handle, int(view), int(what), ptr(out), out.nbytes,
                                        stream), "read")
        self.ctx.sync(stream)
        return out

    def autotune(self, frames: int = 5, stream=None):
        best = L.RenderParams()
        buf = C.create_string_buffer(4096)
        self._check(self.lib.cr_mv_autotune(self.handle, int(frames), stream, C.byref(best), buf,
                                            4096), "autotune")
        return best, json.loads(buf.value.decode() or "{}")

    def close(self):
        if self.handle:
            self.lib.cr_mv_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
