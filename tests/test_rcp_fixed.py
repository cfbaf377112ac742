"""Host check of the integer fixed-point reciprocal of the Lennard-Jones pair
loops (pagmo2_gb300/csrc/rcp_fixed.h), built with g++ from
tests/cpp/test_rcp_fixed.cpp: 2 million random d in 2^-100 .. 2^100 and edge
mantissas, seeds one unit either side of the rounded float reciprocal; every
result within 0.5 + 2^-10 units of the last place of 1/d, every cube within
0.5 + 2^-5 units of the last place of 1/d^3."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_fixed_point_reciprocal_is_faithful(tmp_path):
    exe = tmp_path / "test_rcp_fixed"
    cmd = ["g++", "-std=c++17", "-O2", "-I", str(ROOT / "pagmo2_gb300" / "csrc"),
           str(ROOT / "tests" / "cpp" / "test_rcp_fixed.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    values, worst, not_cr, worst3 = r.stdout.split()
    assert int(values) > 2_000_000
    assert float(worst) <= 0.5 + 2.0 ** -10
    # correctly rounded but for values within 2^-10 units of a midpoint
    assert int(not_cr) <= int(values) // 10_000
    assert float(worst3) <= 0.5 + 2.0 ** -5
