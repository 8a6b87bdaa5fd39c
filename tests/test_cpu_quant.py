"""The GPU builders' integer form of the loaders' double quantisation
(compute_rasterizer_gb300/csrc/cr_quant.h) never disagrees with the double
chain it stands for: tests/cpp/quant_check.cpp draws encoder batch boxes
(LasLoaderSparse.cpp:93-105,146-148, 30-bit cells) and Morton cubes
(Sort_Frugal/src/main.cpp:82-105, 21-bit cells) over LAS scales, offsets and
extents, with points drawn uniformly and next to cell boundaries, and checks
every point the integer form decides.  The same header compiles into the CUDA
kernels, whose output the GPU builder tests compare with the host encoder and
host Morton sort (both on the double chain)."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _build(tmp_path):
    exe = tmp_path / "quant_check"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off",
           "-fno-fast-math", str(ROOT / "tests" / "cpp" / "quant_check.cpp"), "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def test_integer_quantisation_matches_double_chain(tmp_path):
    exe = _build(tmp_path)
    res = subprocess.run([str(exe), "200000"], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    # "encode checked N fast F; morton checked N fast F"
    words = res.stdout.split()
    enc_checked, enc_fast = int(words[2]), int(words[4].rstrip(";"))
    mor_checked, mor_fast = int(words[7]), int(words[9])
    assert enc_checked > 10**7 and mor_checked > 10**7
    # the integer form decides a good share even of these adversarial draws
    assert enc_fast > enc_checked // 4 and mor_fast > mor_checked // 4
