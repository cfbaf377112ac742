"""Host checks of the integer arithmetic that replaces FP64 instructions in
the row loops, built with g++ (the headers compile as plain C++):

- the fixed-point reciprocal of the Lennard-Jones pair loops
  (pagmo2_gb300/csrc/rcp_fixed.h, tests/cpp/test_rcp_fixed.cpp): 2 million
  random d in 2^-100 .. 2^100 and edge mantissas, seeds one unit either side
  of the rounded float reciprocal; every result within 0.5 + 2^-10 units of
  the last place of 1/d, every cube within 0.5 + 2^-5 units of 1/d^3;
- the sum-of-squares accumulator of the Rosenbrock rows
  (pagmo2_gb300/csrc/isum.h, tests/cpp/test_isum.cpp): 80 000 sums of 1..200
  squares spread over 2^200, one at a time and four at a time, within
  2^-53 + n 2^-60 of the exact sums; infinities, NaN, overflow, underflow
  and subnormal squares as FP64 gives them; and its signed variant (ZDT and
  DTLZ sums): 40 000 sums of both signs within 2^-53 of the result plus
  n 2^-60 of the largest magnitude, cancellation and infinities included;
- the fixed-point sin/cos(2 pi x) of the rastrigin and ackley rows
  (pagmo2_gb300/csrc/trig_fixed.h, tests/cpp/test_trig_fixed.cpp): 2.8 million
  x over every binade of 2^-60 .. 2^40 and next to the multiples of 1/4,
  cos within 2^-53 absolute and sin within 2^-52 relative of long double."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def build_and_run(tmp_path, name):
    exe = tmp_path / name
    cmd = ["g++", "-std=c++17", "-O2", "-I", str(ROOT / "pagmo2_gb300" / "csrc"),
           str(ROOT / "tests" / "cpp" / f"{name}.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout.split()


def test_fixed_point_reciprocal_is_faithful(tmp_path):
    values, worst, not_cr, worst3 = build_and_run(tmp_path, "test_rcp_fixed")
    assert int(values) > 2_000_000
    assert float(worst) <= 0.5 + 2.0 ** -10
    # correctly rounded but for values within 2^-10 units of a midpoint
    assert int(not_cr) <= int(values) // 10_000
    assert float(worst3) <= 0.5 + 2.0 ** -5


def test_integer_sum_of_squares(tmp_path):
    sums, worst, worst_signed = build_and_run(tmp_path, "test_isum")
    assert int(sums) == 80_000
    assert float(worst) <= 2.0 ** -53 + 200 * 2.0 ** -60
    # signed sums: the worst error as a fraction of 2^-53 |sum| + n 2^-60 max |term|
    assert float(worst_signed) <= 1.0


def test_fixed_point_sin_cos_2pi(tmp_path):
    values, worst_c, worst_s = build_and_run(tmp_path, "test_trig_fixed")
    assert int(values) > 2_700_000
    assert float(worst_c) <= 2.0 ** -53 and float(worst_s) <= 2.0 ** -52
