"""Python handles over the C ABI: Context, Cloud, Framebuffer.

Every call goes through libcr_raster.so; errors raise CRError with the
library's message.  Device work runs on the CUDA stream passed as `stream`
(an int cudaStream_t, e.g. torch.cuda.current_stream().cuda_stream) or the
legacy default stream when it is None.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import CRError, ptr


def _dbl16(m) -> C.Array:
    a = np.ascontiguousarray(np.asarray(m, dtype=np.float64).reshape(16))
    return (C.c_double * 16)(*a.tolist())


def make_view(view, proj, width: int, height: int) -> L.View:
    """cr_view from column-major 4x4 matrices (flat 16 or 4x4 as stored by glm)."""
    v = L.View()
    v.view = _dbl16(view)
    v.proj = _dbl16(proj)
    v.width = int(width)
    v.height = int(height)
    return v


def default_params(method: int, **kw) -> L.RenderParams:
    lib = L.load()
    p = L.RenderParams()
    lib.cr_render_params_default(int(method), C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


class Context:
    """One cr_ctx on one device."""

    def __init__(self, device: int = 0):
        self.lib = L.load()
        h = C.c_void_p()
        st = self.lib.cr_ctx_create(int(device), C.byref(h))
        if st != L.OK:
            raise CRError(st, f"cr_ctx_create({device}) failed: "
                          + self.lib.cr_status_string(st).decode())
        self.handle = h
        self.num_sms = self.lib.cr_ctx_num_sms(h)

    def close(self):
        if self.handle:
            self.lib.cr_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, status: int, what: str = ""):
        if status != L.OK:
            msg = self.lib.cr_last_error(self.handle).decode()
            raise CRError(status, f"{what}: {self.lib.cr_status_string(status).decode()}: {msg}")

    def sync(self, stream=None):
        """Wait for `stream` and raise on a device error flag."""
        self.check(self.lib.cr_ctx_check(self.handle, stream), "device check")

    # ---- clouds -------------------------------------------------------------
    def cloud(self, num_points: int, num_batches: int, num_files: int = 1,
              mask: int = L.STREAM_ALL) -> "Cloud":
        h = C.c_void_p()
        self.check(self.lib.cr_cloud_create(self.handle, int(num_points), int(num_batches),
                                            int(num_files), int(mask), C.byref(h)), "cloud create")
        return Cloud(self, h, num_points, num_batches, num_files)

    def cloud_from_arrays(self, batches, low, med, hig, rgba, box_min, stream=None) -> "Cloud":
        batches = np.ascontiguousarray(batches, dtype=L.BATCH_DTYPE)
        box_min = np.ascontiguousarray(box_min, dtype=np.float64).reshape(-1)
        nfiles = box_min.size // 3
        c = self.cloud(len(low), len(batches), nfiles)
        c.upload(batches, low, med, hig, rgba, box_min, stream)
        return c

    def cloud_wrap(self, num_points: int, num_batches: int, batches, low, med=None, hig=None,
                   rgba=None, box_min=None, stream_words: int | None = None,
                   num_files: int = 1) -> "Cloud":
        """A cloud over caller-owned arrays (cr_cloud_wrap): numpy arrays, or
        objects with data_ptr() (device or pinned host tensors), each stream
        holding stream_words >= num_points + 64 words with zeros past the
        points.  The arrays are referenced, not copied, for the cloud's life."""
        arrays = [batches, low, med, hig, rgba]
        addr = [None if a is None else (a.data_ptr() if hasattr(a, "data_ptr") else ptr(a))
                for a in arrays]
        words = stream_words if stream_words is not None else int(num_points) + 64
        h = C.c_void_p()
        self.check(self.lib.cr_cloud_wrap(self.handle, int(num_points), int(num_batches),
                                          int(num_files), *addr, int(words), C.byref(h)),
                   "cloud wrap")
        c = Cloud(self, h, num_points, num_batches, num_files)
        c._arrays = arrays
        if box_min is not None:
            c.set_files(box_min)
        return c

    def plain_cloud(self, vertices, stream=None) -> "Cloud":
        v = np.ascontiguousarray(vertices, dtype=L.VERTEX_DTYPE)
        h = C.c_void_p()
        self.check(self.lib.cr_cloud_create_plain(self.handle, len(v), C.byref(h)), "plain cloud")
        c = Cloud(self, h, len(v), 0, 1, plain=True)
        self.check(self.lib.cr_cloud_upload_plain(self.handle, h, ptr(v), stream), "plain upload")
        self.sync(stream)
        return c

    def plain_cloud_empty(self, n: int) -> "Cloud":
        h = C.c_void_p()
        self.check(self.lib.cr_cloud_create_plain(self.handle, int(n), C.byref(h)), "plain cloud")
        return Cloud(self, h, int(n), 0, 1, plain=True)

    # ---- framebuffers -------------------------------------------------------
    def framebuffer(self, width: int, height: int, kind: int = L.FB_U64) -> "Framebuffer":
        h = C.c_void_p()
        self.check(self.lib.cr_fb_create(self.handle, int(width), int(height), int(kind),
                                         C.byref(h)), "fb create")
        return Framebuffer(self, h, int(width), int(height), int(kind))

    # ---- rendering ------------------------------------------------------------
    def render(self, cloud: "Cloud", view: L.View, params: L.RenderParams, fb: "Framebuffer",
               stream=None):
        self.check(self.lib.cr_render(self.handle, cloud.handle, C.byref(view), C.byref(params),
                                      fb.handle, stream), "cr_render")

    def timing_enable(self, max_frames: int):
        self.check(self.lib.cr_timing_enable(self.handle, int(max_frames)), "timing enable")

    def timing_read(self, stage: int, max_frames: int = 4096) -> np.ndarray:
        buf = (C.c_float * max_frames)()
        n = self.lib.cr_timing_read(self.handle, int(stage), buf, max_frames)
        if n < 0:
            raise CRError(L.CUDA_ERROR, "cr_timing_read failed")
        return np.frombuffer(buf, np.float32)[:n].copy()

    def frame_stats(self, cloud, params: L.RenderParams) -> L.FrameStats:
        st = L.FrameStats()
        self.check(self.lib.cr_last_frame_stats(self.handle, cloud.handle, C.byref(params),
                                                C.byref(st)), "frame stats")
        return st

    def resolve(self, cloud, params: L.RenderParams, fb: "Framebuffer", stream=None):
        self.check(self.lib.cr_resolve(self.handle, cloud.handle if cloud else None,
                                       C.byref(params), fb.handle, stream), "cr_resolve")


class Cloud:
    def __init__(self, ctx: Context, handle, n, nb, nfiles, plain=False):
        self.ctx, self.handle = ctx, handle
        self.n, self.nb, self.nfiles, self.plain = int(n), int(nb), int(nfiles), plain

    def upload(self, batches, low, med, hig, rgba, box_min, stream=None):
        arrs = []
        for a in (low, med, hig, rgba):
            if a is None:
                arrs.append(None)
                continue
            a = np.ascontiguousarray(a, dtype=np.uint32)
            if a.size != self.n:
                raise ValueError(f"stream has {a.size} words, cloud holds {self.n} points")
            arrs.append(a)
        b = None if batches is None else np.ascontiguousarray(batches, dtype=L.BATCH_DTYPE)
        bm = None if box_min is None else np.ascontiguousarray(box_min, dtype=np.float64).reshape(-1)
        self.ctx.check(self.ctx.lib.cr_cloud_upload(
            self.ctx.handle, self.handle, ptr(b), *(ptr(a) for a in arrs), ptr(bm), stream),
            "cloud upload")
        self.ctx.sync(stream)

    def set_loaded(self, points: int = -1, batches: int = -1):
        """Frames draw only the first `batches` records / `points` points (the
        loader's numBatchesLoaded / numPointsLoaded); -1, -1 = everything."""
        self.ctx.check(self.ctx.lib.cr_cloud_set_loaded(self.ctx.handle, self.handle, int(points),
                                                        int(batches)), "set loaded")

    def set_files(self, box_min):
        bm = np.ascontiguousarray(box_min, dtype=np.float64).reshape(-1)
        self.ctx.check(self.ctx.lib.cr_cloud_set_files(self.ctx.handle, self.handle, ptr(bm)),
                       "set files")

    def read(self, which: int, stream=None) -> np.ndarray:
        """Download one array of the layout (STREAM_LOW/MED/HIG/RGBA, or 0: batches)."""
        if which == 0:
            out = np.empty(self.nb, dtype=L.BATCH_DTYPE)
        else:
            out = np.empty(self.n, dtype=np.uint32)
        self.ctx.check(self.ctx.lib.cr_cloud_read(self.ctx.handle, self.handle, int(which),
                                                  ptr(out), out.nbytes, stream), "cloud read")
        self.ctx.sync(stream)
        return out

    def device_pointers(self) -> dict:
        ps = [C.c_void_p() for _ in range(5)]
        self.ctx.check(self.ctx.lib.cr_cloud_device(self.handle, *(C.byref(p) for p in ps)),
                       "cloud device")
        return dict(zip(("batches", "low", "med", "hig", "rgba"), (p.value for p in ps)))

    def vertices_pointer(self) -> int:
        p = C.c_void_p()
        self.ctx.check(self.ctx.lib.cr_cloud_device_plain(self.handle, C.byref(p)), "plain ptr")
        return p.value

    def close(self):
        if self.handle:
            self.ctx.lib.cr_cloud_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Framebuffer:
    def __init__(self, ctx: Context, handle, W, H, kind):
        self.ctx, self.handle, self.W, self.H, self.kind = ctx, handle, W, H, kind

    @property
    def words(self) -> int:
        return self.W * self.H + self.W + 1

    def clear(self, value: int = L.DEFAULT_CLEAR, stream=None):
        self.ctx.check(self.ctx.lib.cr_fb_clear(self.ctx.handle, self.handle, C.c_uint64(value),
                                                stream), "fb clear")

    def nbytes(self, what: int) -> int:
        return int(self.ctx.lib.cr_fb_bytes(self.handle, int(what)))

    def read(self, what: int, stream=None) -> np.ndarray:
        dtype = {L.FB_WORDS: np.uint64, L.FB_DEPTH: np.uint32, L.FB_ACCUM: np.uint64,
                 L.FB_IMAGE: np.uint32}[what]
        nbytes = self.nbytes(what)
        out = np.empty(nbytes // np.dtype(dtype).itemsize, dtype=dtype)
        self.ctx.check(self.ctx.lib.cr_fb_read(self.ctx.handle, self.handle, int(what),
                                               ptr(out), nbytes, stream), "fb read")
        self.ctx.sync(stream)
        return out

    def device_pointer(self, what: int) -> int:
        p = C.c_void_p()
        self.ctx.check(self.ctx.lib.cr_fb_device(self.handle, int(what), C.byref(p)), "fb ptr")
        return p.value

    def close(self):
        if self.handle:
            self.ctx.lib.cr_fb_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
