"""Frame server over the C ABI of include/cr_serve.h.

`Server` owns one cr_server: resident clouds, a framebuffer + image pool with
memory-based admission, and a native dispatcher thread that batches queued
requests for the same cloud into multi-view launches (or, with
plain_launches=True, renders every request by itself with the single-view
kernels).  Each served image equals Context.render + resolve of the same view
alone.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import CRError


def request_bytes(width: int, height: int) -> int:
    """Pool bytes a request holds while in flight: its u64 framebuffer (with
    the W+1 guard words) and its RGBA8 image, each rounded to 256 B."""
    r = lambda n: (n + 255) // 256 * 256
    return r((width * height + width + 1) * 8) + r(width * height * 4)


class Server:
    def __init__(self, ctx, *, pool_bytes: int = 8 << 30, max_batch_views: int = 16,
                 max_inflight: int = 4, max_queued: int = 65536, plain_launches: bool = False,
                 method: int = L.METHOD_LOOP_LAS, payload: int = L.PAYLOAD_COLOR,
                 quirks: int = L.QUIRKS_METHOD_DEFAULT, frustum_culling: bool = True,
                 views_per_group: int = 8, block_threads: int = 0):
        self.ctx = ctx
        self.lib = ctx.lib
        cfg = L.ServerConfig()
        cfg.pool_bytes = int(pool_bytes)
        cfg.max_batch_views = int(max_batch_views)
        cfg.max_inflight = int(max_inflight)
        cfg.max_queued = int(max_queued)
        cfg.plain_launches = int(bool(plain_launches))
        cfg.method = int(method)
        cfg.payload = int(payload)
        cfg.quirks = int(quirks)
        cfg.frustum_culling = int(bool(frustum_culling))
        cfg.views_per_group = int(views_per_group)
        cfg.block_threads = int(block_threads)
        self.config = cfg
        h = C.c_void_p()
        st = self.lib.cr_server_create(ctx.handle, C.byref(cfg), C.byref(h))
        if st != L.OK:
            raise CRError(st, "cr_server_create: " + self.lib.cr_status_string(st).decode())
        self.handle = h
        self.clouds = []

    def _check(self, st, what):
        if st != L.OK:
            msg = self.lib.cr_server_last_error(self.handle).decode()
            raise CRError(st, f"{what}: {self.lib.cr_status_string(st).decode()}: {msg}")

    def add_cloud(self, cloud) -> int:
        cid = C.c_int32()
        self._check(self.lib.cr_server_add_cloud(self.handle, cloud.handle, C.byref(cid)),
                    "add_cloud")
        self.clouds.append(cloud)
        return cid.value

    def now_us(self) -> float:
        return self.lib.cr_server_now_us(self.handle)

    @staticmethod
    def request(cloud: int, view: L.View, host_image=None, user_tag: int = 0) -> L.Request:
        r = L.Request()
        r.cloud = int(cloud)
        r.view = view
        if host_image is not None:
            assert host_image.dtype == np.uint32 and host_image.size >= view.width * view.height
            assert host_image.flags["C_CONTIGUOUS"]
            r.host_image = host_image.ctypes.data
        r.user_tag = int(user_tag)
        return r

    def submit(self, req: L.Request) -> int:
        """Queues a request; raises CRError(ADMISSION_REJECTED) when refused."""
        t = C.c_uint64()
        self._check(self.lib.cr_server_submit(self.handle, C.byref(req), C.byref(t)), "submit")
        return t.value

    def try_submit(self, req: L.Request):
        """(status, ticket) without raising."""
        t = C.c_uint64()
        st = self.lib.cr_server_submit(self.handle, C.byref(req), C.byref(t))
        return st, t.value

    def poll(self, max_n: int = 256, wait_ms: int = 0) -> list:
        out = (L.Completion * max_n)()
        n = C.c_int32()
        self._check(self.lib.cr_server_poll(self.handle, out, int(max_n), C.byref(n), int(wait_ms)),
                    "poll")
        return [out[i] for i in range(n.value)]

    def drain(self, timeout_ms: int = -1):
        self._check(self.lib.cr_server_drain(self.handle, int(timeout_ms)), "drain")

    def replay(self, requests, arrival_us) -> np.ndarray:
        """Open-loop replay (requests at arrival_us after the call starts);
        returns a structured array of completions in request order."""
        n = len(requests)
        reqs = (L.Request * n)(*requests)
        arr = np.ascontiguousarray(np.asarray(arrival_us, dtype=np.float64))
        assert arr.shape == (n,)
        out = (L.Completion * n)()
        self._check(self.lib.cr_server_replay(self.handle, reqs,
                                              arr.ctypes.data_as(C.POINTER(C.c_double)), n, out),
                    "replay")
        return np.frombuffer(out, dtype=COMPLETION_DTYPE, count=n).copy()

    def inject(self, what: int, count: int):
        """Host-side fault injection (see cr_server_inject)."""
        self._check(self.lib.cr_server_inject(self.handle, int(what), int(count)), "inject")

    def stats(self) -> dict:
        s = L.ServerStats()
        self._check(self.lib.cr_server_stats_get(self.handle, C.byref(s)), "stats")
        return {k: getattr(s, k) for k, _ in L.ServerStats._fields_}

    def close(self):
        if getattr(self, "handle", None):
            self.lib.cr_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


COMPLETION_DTYPE = np.dtype([("ticket", "<u8"), ("user_tag", "<u8"), ("status", "<i4"),
                             ("batch_views", "<i4"), ("t_arrival_us", "<f8"),
                             ("t_launch_us", "<f8"), ("t_done_us", "<f8")])
assert COMPLETION_DTYPE.itemsize == C.sizeof(L.Completion)


def latency_summary(done: np.ndarray) -> dict:
    """p50/p99/mean latency (arrival -> done) over the completed requests."""
    ok = done[done["status"] == L.OK]
    if len(ok) == 0:
        return {"completed": 0}
    lat = (ok["t_done_us"] - ok["t_arrival_us"]) / 1000.0
    span = (ok["t_done_us"].max() - done["t_arrival_us"].min()) / 1e6
    return {
        "completed": int(len(ok)),
        "rejected": int((done["status"] == L.ADMISSION_REJECTED).sum()),
        "failed": int(((done["status"] != L.OK) & (done["status"] != L.ADMISSION_REJECTED)).sum()),
        "p50_ms": float(np.percentile(lat, 50)),
        "p99_ms": float(np.percentile(lat, 99)),
        "mean_ms": float(lat.mean()),
        "served_req_per_s": float(len(ok) / span) if span > 0 else None,
        "mean_batch_views": float(ok["batch_views"].mean()),
    }
