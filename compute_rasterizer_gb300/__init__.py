"""GB300-native point-rasterizer hot path of m-schuetz/compute_rasterizer.

The product is libcr_raster.so (CUDA kernels for sm_103a behind the C ABI in
include/cr_raster.h and include/cr_synth.h).  This package builds it in-tree
and binds it with ctypes; `methods` mirrors the reference's Method plugins.
"""
from . import _lib
from ._lib import CRError
from .raster import Cloud, Context, Framebuffer, default_params, make_view

__all__ = ["CRError", "Cloud", "Context", "Framebuffer", "default_params", "make_view", "_lib"]
