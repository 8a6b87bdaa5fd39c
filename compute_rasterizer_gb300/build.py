"""In-tree build of the CUDA library (libcr_raster.so) for sm_103a.

The sources under csrc/ are compiled in parallel with nvcc and linked into
compute_rasterizer_gb300/_build/libcr_raster.so; nothing is installed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libcr_raster.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

SOURCES = ["cr_api.cpp", "cr_kernels.cu", "cr_synth.cu", "cr_noalloc.cu", "cr_multiview.cu", "cr_serve.cpp",
           "cr_las.cpp", "cr_potree.cpp", "cr_laz.cpp"]

# -fmad=false: no implicit contraction; explicit __fmaf_rn only.
NVCC_FLAGS = [
    ARCH, "-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--prec-div=true",
    "--prec-sqrt=true", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-Xcompiler", "-fno-fast-math", "-Xcompiler", "-Wall",
]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcr_raster.so")
    return exe


def _compile(src: str, extra: list[str]) -> Path:
    obj = OUT / (Path(src).stem + ".o")
    cmd = [nvcc(), *NVCC_FLAGS, *extra, "-c", str(CSRC / src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose_ptxas: bool = False, force: bool = False) -> Path:
    """Compile and link libcr_raster.so; returns its path."""
    OUT.mkdir(parents=True, exist_ok=True)
    srcs = [CSRC / s for s in SOURCES]
    # every header a source includes: the package's own and the public ones
    deps = srcs + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + \
        list((PKG.parent / "include").glob("*.h")) + list((PKG.parent / "include").glob("*.hpp"))
    if LIB.exists() and not force and not verbose_ptxas:
        newest = max(p.stat().st_mtime for p in deps if p.exists())
        if LIB.stat().st_mtime >= newest:
            return LIB
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cudalib = Path(nvcc()).resolve().parent.parent / "lib64"
    cmd = [nvcc(), ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-lpthread",
           "-Xlinker", "-rpath", "-Xlinker", str(cudalib)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
