"""CPU tests of the C ABI: the library loads, exports every function declared in
include/*.h, and its host-only entry points behave (no GPU calls here)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from compute_rasterizer_gb300 import _lib as L

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(cr_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) > 30
    out = subprocess.run(["nm", "-D", "--defined-only", str(L.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = names - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    lib = L.load()
    for n in names:
        assert getattr(lib, n)


def test_binding_covers_declarations():
    assert declared_functions() <= set(L.EXPORTED)


def test_method_registry_and_defaults():
    lib = L.load()
    want = {"loop_las": 0, "loop_las_prefetch": 1, "loop_las_hqs": 2, "(2021) early-z": 3}
    for name, mid in want.items():
        m = C.c_int32(-1)
        assert lib.cr_method_find(name.encode(), C.byref(m)) == L.OK and m.value == mid
        assert lib.cr_method_name(mid).decode() == name
    assert lib.cr_method_group(0).decode() == "10-10-10 bit encoded"
    m = C.c_int32()
    assert lib.cr_method_find(b"nope", C.byref(m)) == L.NOT_FOUND
    p = L.RenderParams()
    lib.cr_render_params_default(L.METHOD_LOOP_LAS, C.byref(p))
    assert (p.payload, p.quirks, p.frustum_culling, p.resolve, p.clear_after) == (
        L.PAYLOAD_INDEX, L.QUIRKS_METHOD_DEFAULT, 1, 1, 1)
    assert p.clear_value == L.DEFAULT_CLEAR
    lib.cr_render_params_default(L.METHOD_EARLYZ, C.byref(p))
    assert p.clear_value == L.PLAIN_RECLEAR
    assert lib.cr_abi_version() == 2
    assert lib.cr_status_string(L.DEVICE_FLAG) == b"device error flag raised"


def test_null_and_bad_arguments_are_rejected():
    lib = L.load()
    assert lib.cr_ctx_create(0, None) == L.INVALID_ARG
    assert lib.cr_ctx_destroy(None) == L.INVALID_ARG
    assert lib.cr_render(None, None, None, None, None, None) == L.INVALID_ARG
    assert lib.cr_encode_las(None, -1, 26, 2, None, None, None, 0, 0, None, None, None, None,
                             None) == L.INVALID_ARG
    assert lib.cr_num_batches(0) == 0 and lib.cr_num_batches(10241) == 2
    assert lib.cr_last_error(None) == b""


def test_no_gpu_context_fails_cleanly():
    """Without a GPU (this container) context creation returns a status, no abort."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = L.load()
    h = C.c_void_p()
    assert lib.cr_ctx_create(0, C.byref(h)) == L.CUDA_ERROR and not h.value


def test_bench_workloads_are_defined():
    """Every workload bench.py runs after the headline frame is defined (the
    extras run on a GPU only, so a missing one would show up there late)."""
    import ast
    src = (ROOT / "bench.py").read_text()
    defined = {n.name for n in ast.parse(src).body if isinstance(n, ast.FunctionDef)}
    for fn in ("extras", "multiview_64", "small_configs", "serving", "e2e", "cpu_baseline",
               "reference_arm", "main"):
        assert fn in defined, fn


def test_quirk_constants_match_the_header():
    """The Python quirk constants and the oracle's shared quirk bits are the
    values include/cr_raster.h declares."""
    import re
    from pathlib import Path
    from oracle import oracle as O
    text = (Path(__file__).resolve().parent.parent / "include" / "cr_raster.h").read_text()
    enum = text[text.index("typedef enum cr_quirk"):text.index("} cr_quirk;")]
    declared = {m.group(1): int(m.group(2)) for m in re.finditer(r"CR_QUIRK_(\w+)\s*=\s*(\d+)", enum)}
    assert declared["LITERAL_ARITH"] == 512
    for name, value in declared.items():
        assert getattr(L, "QUIRK_" + name) == value, name
    for name in ("L0_X12", "INCLUSIVE_END", "DISPATCH_BY_POINTS", "UVEC4_BASE", "RESOLVE_TILES",
                 "NODE_LOOP", "LEVEL4_80PX", "ONE_WORLD"):
        assert getattr(O, name) == declared[name], name
