"""The allocation-free survival entry point against the regular one.

pgx_nsga2_survival_device_noalloc serves callers that cannot call cudaMalloc
when they evaluate a population (their device memory is held by another
allocator, or they must not risk the device-wide synchronisation cudaMalloc
and cudaFree can cause); its scratch is a fixed array inside the library.
This file is collected last on purpose and must pass both alone in a fresh
process and after the other tests: the entry point's first call on a device
does a one-time set-up, and every call reuses the same array, so two calls in
a row with different inputs check that nothing leaks from one to the next.
"""
import numpy as np
import pytest

from pagmo2_gb300 import _native as N
from pagmo2_gb300 import workloads as W

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _outputs(n):
    i32 = lambda k: torch.full((k,), -7, dtype=torch.int32, device="cuda")  # noqa: E731
    return {"rank": i32(n), "dc": i32(n), "off": i32(n + 1), "idx": i32(n), "nf": i32(1),
            "cd": torch.full((n,), -7.0, dtype=torch.float64, device="cuda")}


def _run(entry, pts, ctx=None):
    n, m = pts.shape
    d = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    o = _outputs(n)
    stream = torch.cuda.current_stream().cuda_stream
    args = [d.data_ptr(), n, m, o["rank"].data_ptr(), o["dc"].data_ptr(), o["off"].data_ptr(), o["idx"].data_ptr(),
            o["nf"].data_ptr(), o["cd"].data_ptr(), stream]
    if ctx is not None:
        args = [ctx.handle] + args
    N.check(entry(*args))
    torch.cuda.synchronize()
    nf = int(o["nf"].item())
    return {"nf": nf, "rank": o["rank"].cpu().numpy(), "dc": o["dc"].cpu().numpy(),
            "off": o["off"].cpu().numpy()[:nf + 1], "idx": o["idx"].cpu().numpy(), "cd": o["cd"].cpu().numpy()}


def _same(a, b):
    assert a["nf"] == b["nf"] and a["nf"] > 0
    for k in ("rank", "dc", "off", "idx"):
        assert np.array_equal(a[k], b[k]), k
    # crowding: the same kernels on the same inputs, so bit-exact
    assert np.array_equal(a["cd"], b["cd"], equal_nan=True)


def test_noalloc_matches_regular_entry_twice_in_a_row():
    lib = N.lib()
    ctx = N.Context(0)
    try:
        first = W.nsga2_points(4096, 3, layers=12, seed=21)   # the largest accepted shape class
        rs = np.random.RandomState(22)
        second = rs.random_sample((1500, 2))                  # smaller, different m: stale data would show
        second[rs.randint(0, 1500, 100)] = second[rs.randint(0, 1500, 100)]
        for pts in (first, second):
            got = _run(lib.pgx_nsga2_survival_device_noalloc, pts)
            want = _run(lib.pgx_nsga2_survival_device, pts, ctx)
            _same(got, want)
    finally:
        ctx.close()


def test_noalloc_rejects_sizes_beyond_its_array():
    lib = N.lib()
    for n, m in ((4097, 3), (100, 9)):
        with pytest.raises(OverflowError, match="at most 4096 points and 8 objectives"):
            N.check(lib.pgx_nsga2_survival_device_noalloc(None, n, m, None, None, None, None, None, None, None))
    with pytest.raises(ValueError):
        N.check(lib.pgx_nsga2_survival_device_noalloc(None, 1, 3, None, None, None, None, None, None, None))


_FRESH_PROCESS = r"""
import numpy as np, torch
from pagmo2_gb300 import _native as N
from pagmo2_gb300 import workloads as W

lib = N.lib()
stream = torch.cuda.current_stream().cuda_stream

def buffers(pts):
    n, m = pts.shape
    d = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    i32 = lambda k: torch.full((k,), -7, dtype=torch.int32, device="cuda")
    return d, [i32(n), i32(n), i32(n + 1), i32(n), i32(1), torch.full((n,), -7.0, dtype=torch.float64, device="cuda")]

def call(pts, bufs):
    d, o = bufs
    n, m = pts.shape
    N.check(lib.pgx_nsga2_survival_device_noalloc(d.data_ptr(), n, m, *[t.data_ptr() for t in o], stream))

big = W.nsga2_points(4096, 8, layers=6, seed=31)          # the largest accepted shape
rs = np.random.RandomState(32)
small = rs.random_sample((1500, 2))
b_big, b_small = buffers(big), buffers(small)              # inputs and outputs first: torch's allocations
call(small, b_small)                                       # the first call on this device: the set-up
torch.cuda.synchronize()
free0 = torch.cuda.mem_get_info()[0]
for _ in range(3):
    call(big, b_big)
    call(small, b_small)
torch.cuda.synchronize()
free1 = torch.cuda.mem_get_info()[0]
print("FREE", free0, free1)
# the same results as the regular entry point (whose context allocates: only now)
ctx = N.Context(0)
for pts, (d, o) in ((big, b_big), (small, b_small)):
    n, m = pts.shape
    ref = [torch.full_like(t, -7) for t in o]
    N.check(lib.pgx_nsga2_survival_device(ctx.handle, d.data_ptr(), n, m, *[t.data_ptr() for t in ref], stream))
    torch.cuda.synchronize()
    nf = int(o[4].item())
    assert nf == int(ref[4].item()) and nf > 0
    for k in (0, 1, 3):
        assert torch.equal(o[k], ref[k]), k
    assert torch.equal(o[2][:nf + 1], ref[2][:nf + 1])
    assert torch.equal(o[5], ref[5])
ctx.close()
print("SAME")
"""


def test_noalloc_allocates_nothing_after_its_first_call_in_a_fresh_process():
    """In a process of its own (no pgx context, no earlier pgx call): after the
    first call on the device, calls of the largest accepted shape and of a
    smaller one leave the device's free memory unchanged, and their results
    equal the regular entry point's."""
    import os
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    env = dict(os.environ, PYTHONPATH=str(root))
    r = subprocess.run([sys.executable, "-c", _FRESH_PROCESS], capture_output=True, text=True, env=env, cwd=root,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    free0, free1 = (int(v) for v in r.stdout.split("FREE")[1].split()[:2])
    assert free0 == free1, (free0, free1)
    assert "SAME" in r.stdout
