"""The literal pair body's division (f2_neg_div_rn: -RN(1/w), then two
Markstein corrections) restated on the host returns C's correctly rounded
quotient on the quotients cr_check_reciprocal draws (csrc/cr_divcheck.h):
every 97th float divisor with |w| in [2^-64, 2^64), both signs, two numerators
each, a quarter of them within 2^-18 ulp of a rounding midpoint or a float.
The bare product RN(a * RN(1/w)) misses on many of those, so the draws test
the corrections.  On the GPU, cr_check_reciprocal runs the device form against
__fdiv_rn over every divisor in the range (test_gpu_parity.py)."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_two_step_division_is_correctly_rounded(tmp_path):
    exe = tmp_path / "div_check"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off",
           "-fno-fast-math", str(ROOT / "tests" / "cpp" / "div_check.cpp"), "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    res = subprocess.run([str(exe), "97"], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    w = res.stdout.split()
    checked, hard, bad2, bad0 = int(w[1]), int(w[3]), int(w[5]), int(w[9])
    assert checked > 4 * 10**7 and hard > checked // 5
    assert bad2 == 0
    assert bad0 > hard // 10
