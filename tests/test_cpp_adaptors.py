"""Builds and runs the C++ programs under tests/cpp/ that use the pagmo
adaptors (include/pagmo_gb300/) against pagmo's own headers, linked with the
reference's compiled sources (oracle/_ref/libpagmo_ref.so) and libpgx:

- test_adaptors.cpp: traits, messages, fevals accounting, and (with a GPU)
  gpu_bfe / the gpu_* UDPs against bfe{thread_bfe{}} and problem::gradient;
- test_udas_gpu_bfe.cpp: pagmo's nsga2, moead_gen, nspso, maco, pso_gen and
  gaco run with bfe{thread_bfe{}} and with bfe{gpu_bfe{}} on the same seeds.

Needs the reference's sources (for its headers and library); skipped where
they are absent."""
import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def build_and_run(tmp_path, source: str, have_gpu: bool):
    import oracle

    if oracle.REF_ROOT is None or not (oracle.REF_ROOT / "include").exists():
        pytest.skip("pagmo headers (the reference tree) are not present")
    ref_inc = oracle.REF_ROOT / "include"
    if oracle.reference() is None:
        oracle.build(reference=True)
    lib = ROOT / "pagmo2_gb300" / "_lib"
    exe = tmp_path / Path(source).stem
    cmd = ["g++", "-std=c++17", "-O1", "-I", str(ROOT / "oracle" / "shim"), "-I", str(ref_inc), "-I",
           str(ROOT / "include"), str(ROOT / "tests" / "cpp" / source), "-o", str(exe),
           str(oracle.REF_SO), "-L", str(lib), "-lpgx", f"-Wl,-rpath,{lib}",
           f"-Wl,-rpath,{oracle.REF_SO.parent}", "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    env = dict(os.environ, PGX_TEST_HAVE_GPU="1" if have_gpu else "0")
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def _no_gpu():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present; see the gpu-marked variant")


def test_adaptors_without_gpu(tmp_path):
    _no_gpu()
    out = build_and_run(tmp_path, "test_adaptors.cpp", have_gpu=False)
    assert "adaptor checks passed" in out


def test_udas_thread_bfe_without_gpu(tmp_path):
    _no_gpu()
    out = build_and_run(tmp_path, "test_udas_gpu_bfe.cpp", have_gpu=False)
    assert "uda checks passed (thread_bfe only)" in out


@pytest.mark.gpu
def test_adaptors_with_gpu(tmp_path):
    out = build_and_run(tmp_path, "test_adaptors.cpp", have_gpu=True)
    assert "adaptor checks passed (with GPU)" in out


@pytest.mark.gpu
def test_udas_with_gpu_bfe(tmp_path):
    """pagmo's algorithms take the same decisions with the GPU bfe as with
    thread_bfe, and log the same values to within 1e-12 relative."""
    out = build_and_run(tmp_path, "test_udas_gpu_bfe.cpp", have_gpu=True)
    assert "uda checks passed (with GPU)" in out
