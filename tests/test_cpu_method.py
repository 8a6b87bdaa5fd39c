"""The C++ Method adapter (include/cr_method.hpp) compiles warning-free and
reports the registered names, groups and descriptions of the C ABI."""
import subprocess

from compute_rasterizer_gb300 import _lib as L
from helpers import build_method_demo


def test_adapter_reports_registered_methods(tmp_path):
    exe = build_method_demo(tmp_path)
    res = subprocess.run([str(exe), "info"], capture_output=True, text=True, timeout=60)
    assert res.returncode == 0, res.stderr
    lib = L.load()
    want = []
    for m in (L.METHOD_LOOP_LAS, L.METHOD_LOOP_LAS_PREFETCH, L.METHOD_LOOP_LAS_HQS, L.METHOD_EARLYZ,
              L.METHOD_DEDUP, L.METHOD_EARLYZ_REDUCE):
        want.append("|".join(x.decode() for x in (lib.cr_method_name(m), lib.cr_method_group(m),
                                                   lib.cr_method_description(m))))
    assert res.stdout.splitlines() == want
    assert want[0].split("|")[:2] == ["loop_las", "10-10-10 bit encoded"]
