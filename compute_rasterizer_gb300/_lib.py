"""ctypes binding of include/cr_raster.h, cr_synth.h, cr_serve.h and cr_las.h.

The CUDA library is built in-tree (compute_rasterizer_gb300/_build/libcr_raster.so
by compute_rasterizer_gb300.build).  There is no CPU fallback: loading fails
loudly when the library is missing.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libcr_raster.so"

POINTS_PER_BATCH = 10240

# cr_status
OK, INVALID_ARG, OUT_OF_MEMORY, ADMISSION_REJECTED, TIMEOUT, CUDA_ERROR, DEVICE_FLAG, \
    UNSUPPORTED, NOT_FOUND, CORRUPT = range(10)

# methods / payloads / quirks / streams / fb kinds
METHOD_LOOP_LAS, METHOD_LOOP_LAS_PREFETCH, METHOD_LOOP_LAS_HQS, METHOD_EARLYZ, METHOD_DEDUP, \
    METHOD_EARLYZ_REDUCE, METHOD_LOOP_NODES = range(7)
PAYLOAD_INDEX, PAYLOAD_COLOR = 0, 1
QUIRK_L0_X12, QUIRK_INCLUSIVE_END, QUIRK_DISPATCH_BY_POINTS, QUIRK_UVEC4_BASE, QUIRK_RESOLVE_TILES = \
    1, 2, 4, 8, 16
QUIRK_NODE_LOOP, QUIRK_LEVEL4_80PX, QUIRK_ONE_WORLD, QUIRK_FLOAT_UNIFORMS = 32, 64, 128, 256
QUIRK_LITERAL_ARITH = 512
POTREE_QUIRK_12B_FROM_8B, POTREE_QUIRK_WRAP30, POTREE_QUIRKS_DEFAULT = 1, 2, -1
MAX_FILES = 65536
NOALLOC_MAX_BATCHES, NOALLOC_MAX_FILES, NOALLOC_SCRATCH_BYTES = 131064, 1024, 753664
QUIRKS_METHOD_DEFAULT = -1
STREAM_LOW, STREAM_MED, STREAM_HIG, STREAM_RGBA, STREAM_ALL = 1, 2, 4, 8, 15
FB_U64, FB_HQS = 0, 1
FB_WORDS, FB_DEPTH, FB_ACCUM, FB_IMAGE = 0, 1, 2, 3
SYNTH_TERRAIN, SYNTH_TERRAIN_BOXES = 0, 1
LAS_FORMAT2_BYTES = 26

DEFAULT_CLEAR = 0xFF800000FF800000
PLAIN_RECLEAR = 0xFFFFFFFFFF3C321E
BACKGROUND = 0x00443322

BATCH_DTYPE = np.dtype([
    ("state", "<i4"), ("min_x", "<f4"), ("min_y", "<f4"), ("min_z", "<f4"),
    ("max_x", "<f4"), ("max_y", "<f4"), ("max_z", "<f4"), ("num_points", "<i4"),
    ("first_point", "<i4"), ("file_index", "<i4"), ("padding", "<i4", (6,)),
])
assert BATCH_DTYPE.itemsize == 64
VERTEX_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("color", "<u4")])


class View(C.Structure):
    _fields_ = [("view", C.c_double * 16), ("proj", C.c_double * 16),
                ("width", C.c_int32), ("height", C.c_int32)]


class RenderParams(C.Structure):
    _fields_ = [("method", C.c_int32), ("payload", C.c_int32), ("quirks", C.c_int32),
                ("frustum_culling", C.c_int32), ("resolve", C.c_int32),
                ("clear_after", C.c_int32), ("clear_value", C.c_uint64),
                ("block_threads", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("views_per_group", C.c_int32), ("lod_skip_level", C.c_int32),
                ("reserved", C.c_int32 * 4)]


class LasHeader(C.Structure):
    _fields_ = [("num_points", C.c_int64), ("point_format", C.c_int32),
                ("bytes_per_point", C.c_int32), ("scale", C.c_double * 3),
                ("offset", C.c_double * 3), ("min", C.c_double * 3), ("max", C.c_double * 3)]


class FrameStats(C.Structure):
    _fields_ = [("batches_dispatched", C.c_int64), ("batches_visible", C.c_int64),
                ("batches_per_level", C.c_int64 * 5), ("points_per_level", C.c_int64 * 5),
                ("stream_bytes", C.c_int64)]


STAGE_CULL, STAGE_RASTER, STAGE_HQS_COLOR, STAGE_RESOLVE = range(4)


class SynthParams(C.Structure):
    _fields_ = [("kind", C.c_int32), ("octaves", C.c_int32), ("seed", C.c_uint64),
                ("extent", C.c_double), ("height", C.c_double), ("sigma", C.c_double),
                ("wavelength", C.c_double), ("las_scale", C.c_double),
                ("num_boxes", C.c_int32), ("points_per_box", C.c_int32),
                ("box_min_height", C.c_double), ("box_max_height", C.c_double),
                ("origin", C.c_double * 2)]


class ServerConfig(C.Structure):
    _fields_ = [("pool_bytes", C.c_int64), ("max_batch_views", C.c_int32),
                ("max_inflight", C.c_int32), ("max_queued", C.c_int32),
                ("plain_launches", C.c_int32), ("method", C.c_int32), ("payload", C.c_int32),
                ("quirks", C.c_int32), ("frustum_culling", C.c_int32),
                ("views_per_group", C.c_int32), ("block_threads", C.c_int32),
                ("reserved", C.c_int32 * 6)]


class Request(C.Structure):
    _fields_ = [("cloud", C.c_int32), ("reserved0", C.c_int32), ("view", View),
                ("host_image", C.c_void_p), ("user_tag", C.c_uint64)]


class Completion(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("user_tag", C.c_uint64), ("status", C.c_int32),
                ("batch_views", C.c_int32), ("t_arrival_us", C.c_double),
                ("t_launch_us", C.c_double), ("t_done_us", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("rejected", C.c_int64), ("completed", C.c_int64),
                ("failed", C.c_int64), ("launches", C.c_int64), ("views_launched", C.c_int64),
                ("pool_bytes", C.c_int64), ("pool_used_bytes", C.c_int64),
                ("pool_peak_bytes", C.c_int64), ("max_views_in_launch", C.c_int32),
                ("queued", C.c_int32), ("gpu_ms", C.c_double)]


class PotreeInfo(C.Structure):
    _fields_ = [("num_points", C.c_int64), ("num_nodes", C.c_int64), ("octree_bytes", C.c_int64),
                ("bytes_per_point", C.c_int32), ("rgb_offset", C.c_int32), ("max_level", C.c_int32),
                ("reserved", C.c_int32), ("max_node_points", C.c_int64),
                ("scale", C.c_double * 3), ("offset", C.c_double * 3),
                ("box_min", C.c_double * 3), ("box_max", C.c_double * 3), ("spacing", C.c_double)]


class PotreeNode(C.Structure):
    _fields_ = [("level", C.c_int32), ("type", C.c_int32), ("child_mask", C.c_int32),
                ("reserved", C.c_int32), ("num_points", C.c_int64), ("byte_offset", C.c_int64),
                ("byte_size", C.c_int64), ("min", C.c_double * 3), ("max", C.c_double * 3)]


class LasInfo(C.Structure):
    _fields_ = [("num_points", C.c_int64), ("offset_to_points", C.c_int64),
                ("version_major", C.c_int32), ("version_minor", C.c_int32),
                ("point_format", C.c_int32), ("bytes_per_point", C.c_int32),
                ("scale", C.c_double * 3), ("offset", C.c_double * 3),
                ("min", C.c_double * 3), ("max", C.c_double * 3)]


LAZ_MAX_ITEMS = 8
LAZ_ITEM_BYTE, LAZ_ITEM_POINT10, LAZ_ITEM_GPSTIME11, LAZ_ITEM_RGB12 = 0, 6, 7, 8
LAZ_ITEM_POINT14, LAZ_ITEM_RGB14, LAZ_ITEM_RGBNIR14, LAZ_ITEM_BYTE14 = 10, 11, 12, 14
LAZ_POINTWISE, LAZ_POINTWISE_CHUNKED, LAZ_LAYERED_CHUNKED = 1, 2, 3
LAZ_DEFAULT_CHUNK, LAZ_VARIABLE_CHUNKS = 50000, -1


class LazInfo(C.Structure):
    _fields_ = [("las", LasInfo), ("compressor", C.c_int32), ("num_items", C.c_int32),
                ("item_type", C.c_int32 * LAZ_MAX_ITEMS), ("item_size", C.c_int32 * LAZ_MAX_ITEMS),
                ("item_version", C.c_int32 * LAZ_MAX_ITEMS),
                ("version_major", C.c_int32), ("version_minor", C.c_int32),
                ("chunk_size", C.c_int64), ("num_chunks", C.c_int64), ("points_at", C.c_int64)]


LAS_MIN_HEADER, LAS_14_HEADER = 227, 375
MAX_POINTS_PER_LOAD = 1024000

SERVE_MAX_POOL_BYTES = 16 << 30
SERVE_MAX_BATCH_VIEWS = 256
INJECT_NONE, INJECT_LAUNCH_ALLOC = 0, 1

P = C.c_void_p
I32, I64, U64, DBL, FLT = C.c_int32, C.c_int64, C.c_uint64, C.c_double, C.c_float
PP = C.POINTER(C.c_void_p)

# name: (restype, argtypes)
_SIGS = {
    "cr_abi_version": (I32, []),
    "cr_status_string": (C.c_char_p, [I32]),
    "cr_method_name": (C.c_char_p, [I32]),
    "cr_method_group": (C.c_char_p, [I32]),
    "cr_method_description": (C.c_char_p, [I32]),
    "cr_method_find": (I32, [C.c_char_p, C.POINTER(I32)]),
    "cr_render_params_default": (None, [I32, C.POINTER(RenderParams)]),
    "cr_ctx_create": (I32, [I32, PP]),
    "cr_ctx_destroy": (I32, [P]),
    "cr_last_error": (C.c_char_p, [P]),
    "cr_ctx_check": (I32, [P, P]),
    "cr_check_reciprocal": (I32, [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]),
    "cr_ctx_num_sms": (I32, [P]),
    "cr_cloud_create": (I32, [P, I64, I64, I32, I32, PP]),
    "cr_cloud_upload": (I32, [P, P, P, P, P, P, P, P, P]),
    "cr_cloud_device": (I32, [P, PP, PP, PP, PP, PP]),
    "cr_cloud_set_files": (I32, [P, P, P]),
    "cr_cloud_read": (I32, [P, P, I32, P, I64, P]),
    "cr_cloud_num_points": (I64, [P]),
    "cr_cloud_set_loaded": (I32, [P, P, I64, I64]),
    "cr_cloud_num_batches": (I64, [P]),
    "cr_cloud_destroy": (I32, [P, P]),
    "cr_cloud_wrap": (I32, [P, I64, I64, I32, P, P, P, P, P, I64, PP]),
    "cr_cloud_create_plain": (I32, [P, I64, PP]),
    "cr_cloud_upload_plain": (I32, [P, P, P, P]),
    "cr_cloud_device_plain": (I32, [P, PP]),
    "cr_fb_create": (I32, [P, I32, I32, I32, PP]),
    "cr_fb_destroy": (I32, [P, P]),
    "cr_fb_clear": (I32, [P, P, U64, P]),
    "cr_fb_bytes": (I64, [P, I32]),
    "cr_fb_read": (I32, [P, P, I32, P, I64, P]),
    "cr_fb_device": (I32, [P, I32, PP]),
    "cr_render": (I32, [P, P, C.POINTER(View), C.POINTER(RenderParams), P, P]),
    "cr_resolve": (I32, [P, P, C.POINTER(RenderParams), P, P]),
    "cr_render_batched_noalloc": (I32, [P, I64, I64, P, P, P, P, I64, P, I32, C.POINTER(View),
                                        C.POINTER(RenderParams), P, P]),
    "cr_noalloc_scratch": (I32, [PP, C.POINTER(I64)]),
    "cr_mv_create": (I32, [P, P, I32, P, P, C.POINTER(RenderParams), PP]),
    "cr_mv_destroy": (I32, [P]),
    "cr_mv_last_error": (C.c_char_p, [P]),
    "cr_mv_set_params": (I32, [P, C.POINTER(RenderParams)]),
    "cr_mv_get_params": (I32, [P, C.POINTER(RenderParams)]),
    "cr_mv_shared_pairs": (I32, [P, C.POINTER(I32)]),
    "cr_mv_set_views": (I32, [P, C.POINTER(View)]),
    "cr_mv_render": (I32, [P, I32, P]),
    "cr_mv_clear": (I32, [P, U64, P]),
    "cr_mv_read": (I32, [P, I32, I32, P, I64, P]),
    "cr_mv_autotune": (I32, [P, I32, P, C.POINTER(RenderParams), C.c_char_p, I32]),
    "cr_timing_enable": (I32, [P, I32]),
    "cr_timing_read": (I32, [P, I32, C.POINTER(C.c_float), I32]),
    "cr_last_frame_stats": (I32, [P, P, C.POINTER(RenderParams), C.POINTER(FrameStats)]),
    "cr_num_batches": (I64, [I64]),
    "cr_encode_las": (I32, [P, I64, I32, I32, P, P, P, I64, I32, P, P, P, P, P]),
    "cr_encode_standard": (I32, [P, I64, I32, I32, P, P, P, P]),
    "cr_perspective": (None, [DBL, DBL, DBL, DBL, P]),
    "cr_look_at": (None, [P, P, P, P]),
    "cr_orbit_view": (None, [DBL, DBL, DBL, P, P]),
    # cr_synth.h
    "cr_synth_params_default": (None, [I32, DBL, U64, C.POINTER(SynthParams)]),
    "cr_synth_points_host": (I32, [C.POINTER(SynthParams), I64, P, C.POINTER(LasHeader)]),
    "cr_morton_sort_host": (I32, [P, I64, I32, C.POINTER(LasHeader)]),
    "cr_synth_points_device": (I32, [P, C.POINTER(SynthParams), I64, P, C.POINTER(LasHeader), P]),
    "cr_morton_sort_device": (I32, [P, P, I64, I32, C.POINTER(LasHeader), P]),
    "cr_encode_las_device": (I32, [P, P, I64, I32, I32, P, P, P, I64, I32, P, P, P, P, P, P]),
    "cr_synth_cloud_device": (I32, [P, C.POINTER(SynthParams), I64, P, C.POINTER(LasHeader), P]),
    "cr_synth_uniform_host": (I32, [U64, I64, FLT, P]),
    "cr_synth_uniform_device": (I32, [P, U64, I64, FLT, P, P]),
    # cr_las.h
    "cr_las_parse_header": (I32, [P, I64, C.POINTER(LasInfo)]),
    "cr_potree_open": (I32, [C.c_char_p, PP, C.POINTER(PotreeInfo)]),
    "cr_potree_close": (I32, [P]),
    "cr_potree_nodes": (I32, [P, P, I64]),
    "cr_potree_encode": (I32, [P, P, I64, I32, P, P, P, P, P]),
    "cr_potree_load": (I32, [P, P, I32, PP, P]),
    "cr_cloud_load_las": (I32, [P, P, P, I64, C.POINTER(LasInfo), I64, I64, I32, P]),
    "cr_las_num_batches": (I64, [I64]),
    # cr_laz.h
    "cr_laz_open": (I32, [P, I64, PP, C.POINTER(LazInfo)]),
    "cr_laz_close": (I32, [P]),
    "cr_laz_decode": (I32, [P, I64, I64, P, I32]),
    "cr_cloud_load_laz": (I32, [P, P, P, I64, I64, I32, I32, P]),
    "cr_laz_vlr": (I32, [I32, I32, I64, P, I64, C.POINTER(I64)]),
    "cr_laz_compress": (I32, [P, I64, I32, I32, I64, I64, I64, P, I64, C.POINTER(I64), I32]),
    "cr_laz_compress_bound": (I64, [I64, I32, I64]),
    # cr_serve.h
    "cr_server_create": (I32, [P, C.POINTER(ServerConfig), PP]),
    "cr_server_destroy": (I32, [P]),
    "cr_server_last_error": (C.c_char_p, [P]),
    "cr_server_now_us": (DBL, [P]),
    "cr_server_add_cloud": (I32, [P, P, C.POINTER(I32)]),
    "cr_server_submit": (I32, [P, C.POINTER(Request), C.POINTER(U64)]),
    "cr_server_poll": (I32, [P, C.POINTER(Completion), I32, C.POINTER(I32), I32]),
    "cr_server_drain": (I32, [P, I32]),
    "cr_server_replay": (I32, [P, C.POINTER(Request), C.POINTER(DBL), I64, C.POINTER(Completion)]),
    "cr_server_stats_get": (I32, [P, C.POINTER(ServerStats)]),
    "cr_server_inject": (I32, [P, I32, I32]),
}

EXPORTED = tuple(_SIGS)

_lib = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load libcr_raster.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with compute_rasterizer_gb300.build.build()")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class CRError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


def ptr(a) -> int | None:
    """Address of a numpy array, a ctypes object or an int device pointer."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return C.addressof(a)
