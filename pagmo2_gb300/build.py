"""Build recipe for the native library (libpgx.so), in-tree.

Every CUDA translation unit in ``csrc/`` is compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into
``pagmo2_gb300/_lib/libpgx.so``. No torch extension machinery is involved: the
library exports the plain C ABI of ``include/pgx.h``.

Run ``python -m pagmo2_gb300.build`` (or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libpgx.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpgx")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _fingerprint() -> str:
    h = hashlib.sha256()
    for p in sorted(list(CSRC.glob("*")) + [ROOT / "include" / "pgx.h"]):
        if p.is_file():
            h.update(p.name.encode())
            h.update(p.read_bytes())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile libpgx.so if its sources changed since the last build."""
    OUT.mkdir(exist_ok=True)
    stamp = OUT / "libpgx.stamp"
    fp = _fingerprint()
    if not force and LIB.exists() and stamp.exists() and stamp.read_text() == fp:
        return LIB
    nvcc = _nvcc()
    objs = []

    # the build's identity (a digest of every source and flag): the autotuner
    # keys its cached choices by it, so a rebuilt library never reuses them
    build_id = f'-DPGX_BUILD_ID="{fp[:16]}"'

    def compile_one(src: Path) -> Path:
        obj = OUT / (src.stem + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, build_id, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = OUT / "libpgx.so.tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of libpgx.so failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    for o in objs:
        o.unlink(missing_ok=True)
    stamp.write_text(fp)
    return LIB


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose=True)
    print(p)
