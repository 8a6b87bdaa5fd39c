"""ctypes binding of the oracle (oracle.c): TEST INFRASTRUCTURE.

Imported only by tests/, __graft_entry__.smoke() and the CPU-baseline leg of
bench.py, always as the checker.  `build()` runs oracle/Makefile.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
GLMREF = HERE / "_ref" / "libglmref.so"
SFREF = HERE / "_ref" / "libsfref.so"
LAZREF = HERE / "_ref" / "liblaszipref.so"
SHADERREF = HERE / "_ref" / "libshaderref.so"

L0_X12, INCLUSIVE_END, DISPATCH_BY_POINTS, UVEC4_BASE, RESOLVE_TILES = 1, 2, 4, 8, 16
NODE_LOOP, LEVEL4_80PX, ONE_WORLD = 32, 64, 128
PAYLOAD_INDEX, PAYLOAD_COLOR = 0, 1
ARITH_CONTRACT, ARITH_LITERAL = 0, 1


class FileFrame(C.Structure):
    _fields_ = [("transform", C.c_float * 16), ("planes", C.c_float * 24),
                ("view_world", C.c_float * 16)]


class Frame(C.Structure):
    _fields_ = [("proj", C.c_float * 16), ("width", C.c_int32), ("height", C.c_int32),
                ("frustum_culling", C.c_int32), ("quirks", C.c_int32), ("payload", C.c_int32),
                ("lod_skip_level", C.c_int32), ("num_files", C.c_int32),
                ("files", C.POINTER(FileFrame))]


def reference_dir() -> str:
    """The reference checkout the probes are compiled from: the CR_REFERENCE
    environment variable, else a checkout named "reference" beside this
    repository; "" when neither holds one (the probes are then not built and
    their tests skip)."""
    import os
    for ref in (os.environ.get("CR_REFERENCE"), str(HERE.parent.parent / "reference")):
        if ref and Path(ref, "libs", "glm", "glm").is_dir():
            return ref
    return ""


def build() -> None:
    subprocess.run(["make", "-s", "-C", str(HERE), f"REF={reference_dir()}"], check=True)


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
        P, I64, I32 = C.c_void_p, C.c_int64, C.c_int32
        sig = {
            "or_file_setup": [P, P, P, C.POINTER(FileFrame)],
            "or_file_setup_float": [P, P, P, C.POINTER(FileFrame)],
            "or_resolve_index_tiles": [I32, I32, P, P, P],
            "or_proj_float": [P, P],
            "or_raster_batched": [C.POINTER(Frame), P, I64, I64, P, P, P, P, P],
            "or_raster_batched_mt": [C.POINTER(Frame), P, I64, I64, P, P, P, P, P, C.c_int],
            "or_resolve_index": [I32, I32, P, P, P],
            "or_resolve_color": [I32, I32, P, P],
            "or_hqs_depth": [C.POINTER(Frame), P, I64, I64, P, P, P, P],
            "or_hqs_color": [C.POINTER(Frame), P, I64, I64, P, P, P, P, P, P],
            "or_hqs_resolve": [I32, I32, P, P],
            "or_plain_transform": [P, P, P],
            "or_raster_plain": [P, I32, I32, P, I64, P],
            "or_raster_plain_warp": [P, I32, I32, P, I64, P, I32],
            "or_resolve_plain": [I32, I32, P, P, C.c_uint64, I32, I32],
            "or_encode_las": [P, I64, I32, I32, P, P, P, I64, I32, P, P, P, P, P],
            "or_encode_standard": [P, I64, I32, I32, P, P, P, P],
            "or_precision_level": [C.POINTER(Frame), C.POINTER(FileFrame), P, P],
            "or_intersects_frustum": [P, P, P],
            "or_perspective": [C.c_double] * 4 + [P],
            "or_look_at": [P, P, P, P],
            "or_inverse": [P, P],
            "or_orbit_world": [C.c_double] * 3 + [P, P],
            "or_morton3": [C.c_uint32] * 3,
            "or_fnv1a64": [P, I64],
            "or_dispatch_batches": [I64, I64, I32],
            "or_set_arith": [C.c_int],
        }
        for k, v in sig.items():
            getattr(_lib, k).argtypes = v
            getattr(_lib, k).restype = None
        for k in ("or_precision_level", "or_intersects_frustum"):
            getattr(_lib, k).restype = C.c_int
        _lib.or_morton3.restype = C.c_uint64
        _lib.or_fnv1a64.restype = C.c_uint64
        _lib.or_dispatch_batches.restype = C.c_int64
        _lib.or_set_arith.restype = C.c_int
    return _lib


class arith:
    """with arith(ARITH_LITERAL): ... -- the oracle's arithmetic interpretation
    (oracle.h) for the frames set up and rasterized inside the block."""

    def __init__(self, mode: int):
        self.mode, self.old = int(mode), None

    def __enter__(self):
        self.old = lib().or_set_arith(self.mode)
        return self

    def __exit__(self, *exc):
        lib().or_set_arith(self.old)


def _p(a):
    return None if a is None else a.ctypes.data


def glmref() -> C.CDLL:
    """The glm probe built from the reference's vendored glm (oracle/_ref)."""
    g = C.CDLL(str(GLMREF))
    P, D, I = C.c_void_p, C.c_double, C.c_int
    sig = {"glmref_camera": [D, I, I, D, D, P, P, P],
           "glmref_orbit_world": [D, D, D, P, P],
           "glmref_look_at": [P, P, P, P],
           "glmref_inverse": [P, P],
           "glmref_file_record": [P, P, P, P, P, P, P],
           "glmref_plain_transform": [P, P, P]}
    for k, v in sig.items():
        getattr(g, k).argtypes = v
        getattr(g, k).restype = None
    return g


def sfref() -> C.CDLL:
    """The Sort_Frugal probe built from the reference's sorter (oracle/_ref)."""
    g = C.CDLL(str(SFREF))
    g.sfref_morton.argtypes = [C.c_uint32] * 3
    g.sfref_morton.restype = C.c_uint64
    return g


def laszipref() -> C.CDLL:
    """The LASzip probe built from the reference's vendored LASzip (oracle/_ref)."""
    g = C.CDLL(str(LAZREF))
    P, I, I64, U32 = C.c_void_p, C.c_int, C.c_int64, C.c_uint32
    g.lzref_vlr.argtypes = [I, I, I, U32, I, P, C.c_int32]
    g.lzref_vlr.restype = C.c_int
    g.lzref_compress.argtypes = [P, I64, P, I64, I, I, I, U32, I, I64, P, I64]
    g.lzref_compress.restype = I64
    g.lzref_decompress.argtypes = [P, I64, I64, P, C.c_int32, I64, I, P]
    g.lzref_decompress.restype = I64
    return g


def shaderref() -> C.CDLL:
    """The reference's GLSL shaders translated to C++ and run on the CPU
    (oracle/shader_ref.cpp, built into oracle/_ref)."""
    g = C.CDLL(str(SHADERREF))
    P, I32, I64 = C.c_void_p, C.c_int32, C.c_int64
    g.ref_loop_las_render.argtypes = [P, I64, P, P, P, P, P, P, I32, I32, I32, I64, P]
    g.ref_loop_las_render.restype = C.c_int
    g.ref_loop_las2_render.argtypes = [P, I64, P, P, P, P, P, P, I32, I32, I32, I64, P]
    g.ref_loop_las2_render.restype = C.c_int
    g.ref_hqs_render.argtypes = [P, I64, P, P, P, P, P, P, P, I32, I32, I32, I64, P, P]
    g.ref_hqs_render.restype = C.c_int
    g.ref_loop_las_resolve.argtypes = [P, P, I32, I32, P]
    g.ref_hqs_resolve.argtypes = [P, I32, I32, P]
    g.ref_earlyz_render.argtypes = [P, I64, P, I32, I32, P]
    g.ref_earlyz_resolve.argtypes = [P, I32, I32, P]
    g.ref_loop_nodes_render.argtypes = [P, I64, P, P, P, P, P, P, I32, I32, I32, I64, P]
    g.ref_dedup_render.argtypes = [P, I64, P, I32, I32, P]
    g.ref_reduce_render.argtypes = [P, I64, P, I32, I32, P]
    for k in ("ref_loop_las_resolve", "ref_hqs_resolve", "ref_earlyz_render", "ref_earlyz_resolve",
              "ref_loop_nodes_render", "ref_dedup_render", "ref_reduce_render"):
        getattr(g, k).restype = C.c_int
    return g


def fnv(a: np.ndarray) -> int:
    a = np.ascontiguousarray(a)
    return int(lib().or_fnv1a64(_p(a), a.nbytes))


def make_frame(view, proj, width, height, box_mins, culling=1, quirks=0, payload=0, lod_skip_level=0,
               float_uniforms=False):
    """Frame + per-file records from double matrices (compute_loop_las.h:141-200;
    float_uniforms: the float products of compute_loop_nodes.h:128-139)."""
    o = lib()
    view = np.ascontiguousarray(view, np.float64).reshape(16)
    proj = np.ascontiguousarray(proj, np.float64).reshape(16)
    box_mins = np.ascontiguousarray(box_mins, np.float64).reshape(-1, 3)
    files = (FileFrame * len(box_mins))()
    setup = o.or_file_setup_float if float_uniforms else o.or_file_setup
    for i, bm in enumerate(box_mins):
        bm = np.ascontiguousarray(bm)
        setup(_p(view), _p(proj), _p(bm), C.byref(files[i]))
    fr = Frame()
    o.or_proj_float(_p(proj), C.cast(fr.proj, C.c_void_p))
    fr.width, fr.height = int(width), int(height)
    fr.frustum_culling, fr.quirks, fr.payload = int(culling), int(quirks), int(payload)
    fr.lod_skip_level = int(lod_skip_level)
    fr.num_files = len(box_mins)
    fr.files = files
    fr._keep = files
    return fr


def fb_words(width, height) -> int:
    return width * height + width + 1


def pad_stream(a, pad=64, n=None) -> np.ndarray:
    """A stream with zeroed words past N (the device streams carry the same).
    A stream that already holds n + pad words is returned as it is."""
    if n is not None and len(a) >= n + pad:
        return a
    out = np.zeros(len(a) + pad, dtype=np.uint32)
    out[:len(a)] = a
    return out


def raster_batched(frame, batches, n, low, med, hig, rgba, clear=0xFF800000FF800000,
                   threads=1) -> np.ndarray:
    fb = np.full(fb_words(frame.width, frame.height), clear, dtype=np.uint64)
    low, med, hig = pad_stream(low, n=n), pad_stream(med, n=n), pad_stream(hig, n=n)
    rgba = pad_stream(rgba, n=n) if rgba is not None else None
    b = np.ascontiguousarray(batches)
    if threads > 1:
        lib().or_raster_batched_mt(C.byref(frame), _p(b), len(b), n, _p(low), _p(med), _p(hig),
                                   _p(rgba), _p(fb), threads)
    else:
        lib().or_raster_batched(C.byref(frame), _p(b), len(b), n, _p(low), _p(med), _p(hig),
                                _p(rgba), _p(fb))
    return fb


def resolve_index(width, height, fb, rgba) -> np.ndarray:
    out = np.empty(width * height, dtype=np.uint32)
    r = pad_stream(rgba)
    lib().or_resolve_index(width, height, _p(fb), _p(r), _p(out))
    return out


def resolve_index_tiles(width, height, fb, rgba, image=None) -> np.ndarray:
    """resolve_index over full 16x16 tiles only; other pixels keep `image`'s
    words (zeros by default)."""
    out = np.zeros(width * height, np.uint32) if image is None else np.array(image, np.uint32)
    r = pad_stream(rgba)
    lib().or_resolve_index_tiles(width, height, _p(fb), _p(r), _p(out))
    return out


def resolve_color(width, height, fb) -> np.ndarray:
    out = np.empty(width * height, dtype=np.uint32)
    lib().or_resolve_color(width, height, _p(fb), _p(out))
    return out


def hqs(frame, batches, n, low, med, hig, rgba):
    depth = np.full(fb_words(frame.width, frame.height), 0xFF800000, dtype=np.uint32)
    accum = np.zeros(2 * fb_words(frame.width, frame.height), dtype=np.uint64)
    low, med, hig, rgba = (pad_stream(x, n=n) for x in (low, med, hig, rgba))
    b = np.ascontiguousarray(batches)
    lib().or_hqs_depth(C.byref(frame), _p(b), len(b), n, _p(low), _p(med), _p(hig), _p(depth))
    lib().or_hqs_color(C.byref(frame), _p(b), len(b), n, _p(low), _p(med), _p(hig), _p(rgba),
                       _p(depth), _p(accum))
    img = np.empty(frame.width * frame.height, dtype=np.uint32)
    lib().or_hqs_resolve(frame.width, frame.height, _p(accum), _p(img))
    return depth, accum, img


def plain(view, proj, width, height, vertices, clear=0xFFFFFFFFFFFFFFFF,
          reclear=0xFFFFFFFFFF3C321E, variant=0, quirks=RESOLVE_TILES, fb=None, image=None):
    """The plain 16 B path: variant 0 early-z, 1 dedup, 2 early-z & reduce.
    quirks: RESOLVE_TILES (the methods' default) or 0.  `fb` / `image`: the
    previous frame's framebuffer and image (pixels outside the resolved tiles
    keep them); a fresh fb filled with `clear` and a zero image by default.
    Returns (fb after the raster, image, fb after the resolve)."""
    T = np.empty(16, np.float32)
    view = np.ascontiguousarray(view, np.float64).reshape(16)
    proj = np.ascontiguousarray(proj, np.float64).reshape(16)
    lib().or_plain_transform(_p(view), _p(proj), _p(T))
    fb = (np.full(fb_words(width, height), clear, dtype=np.uint64) if fb is None
          else np.array(fb, dtype=np.uint64))
    v = np.ascontiguousarray(vertices)
    if variant == 0:
        lib().or_raster_plain(_p(T), width, height, _p(v), len(v), _p(fb))
    else:
        lib().or_raster_plain_warp(_p(T), width, height, _p(v), len(v), _p(fb), int(variant))
    fb_before = fb.copy()
    img = (np.zeros(width * height, dtype=np.uint32) if image is None
           else np.array(image, dtype=np.uint32))
    lib().or_resolve_plain(width, height, _p(fb), _p(img), reclear, int(quirks),
                           0 if variant == 1 else 1)
    return fb_before, img, fb


def encode_las(records, n, bpp, fmt, scale, offset, box_min, sparse_offset=0, file_index=0):
    nb = (n + 10239) // 10240
    from compute_rasterizer_gb300._lib import BATCH_DTYPE
    batches = np.zeros(nb, dtype=BATCH_DTYPE)
    streams = [np.zeros(n, dtype=np.uint32) for _ in range(4)]
    sc, of, bm = (np.ascontiguousarray(x, np.float64) for x in (scale, offset, box_min))
    lib().or_encode_las(_p(records), n, bpp, fmt, _p(sc), _p(of), _p(bm), sparse_offset,
                        file_index, _p(batches), *(_p(s) for s in streams))
    return (batches, *streams)
