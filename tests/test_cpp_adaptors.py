"""Builds and runs tests/cpp/test_adaptors.cpp: the C++ pagmo adaptors
(include/pagmo_gb300/) compiled against pagmo's own headers and linked with
the reference's compiled sources (oracle/_ref/libpagmo_ref.so) and libpgx.
Needs the reference tree (its headers); skipped where it is absent."""
import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def build_and_run(tmp_path, have_gpu: bool):
    import oracle

    ref_inc = oracle.REF_ROOT / "include"
    if not ref_inc.exists():
        pytest.skip("pagmo headers (the reference tree) are not present")
    if oracle.reference() is None:
        oracle.build(reference=True)
    lib = ROOT / "pagmo2_gb300" / "_lib"
    exe = tmp_path / "test_adaptors"
    cmd = ["g++", "-std=c++17", "-O1", "-I", str(ROOT / "oracle" / "shim"), "-I", str(ref_inc), "-I",
           str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "test_adaptors.cpp"), "-o", str(exe),
           str(oracle.REF_SO), "-L", str(lib), "-lpgx", f"-Wl,-rpath,{lib}",
           f"-Wl,-rpath,{oracle.REF_SO.parent}", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    env = dict(os.environ, PGX_TEST_HAVE_GPU="1" if have_gpu else "0")
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_adaptors_without_gpu(tmp_path):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present; see the gpu-marked variant")
    out = build_and_run(tmp_path, have_gpu=False)
    assert "adaptor checks passed" in out


@pytest.mark.gpu
def test_adaptors_with_gpu(tmp_path):
    out = build_and_run(tmp_path, have_gpu=True)
    assert "adaptor checks passed (with GPU)" in out
