"""The fused archipelago epoch (through the C ABI) against the island-by-island
path and the long-double oracle, including two epochs in flight."""
from pathlib import Path

import numpy as np
import pytest

from pagmo2_gb300 import _native as N
from pagmo2_gb300 import archipelago as A
from pagmo2_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-13


def shapes_and_batches(islands=18, seed=5, grad_every=1):
    reqs = W.archipelago(islands, seed=seed, pop_hi=1024)
    shapes = [(r.kind, r.param, r.n, i % grad_every == 0) for i, r in enumerate(reqs)]
    return shapes, [r.dvs for r in reqs]


def check(orc, shapes, batches, outs):
    for (k, p, n, g), x, (f, gr) in zip(shapes, batches, outs):
        rows = np.unique(np.linspace(0, n - 1, min(n, 6)).astype(int))
        fl, fs = orc.batch_fitness_ld(k, p, x[rows])
        assert np.max(np.abs(f[rows] - fl) / fs) <= TOL, (k, p)
        if g:
            gl, gs = orc.batch_gradient_ld(k, p, x[rows])
            assert np.max(np.abs(gr[rows] - gl) / np.maximum(gs, 1e-300)) <= TOL, (k, p)


def test_epoch_matches_plain_and_oracle(ctx, orc):
    shapes, batches = shapes_and_batches(grad_every=3)  # some islands fitness only
    ep = A.Epoch(shapes, ctx)
    try:
        fused = ep.run(batches)
        plain = A.run_plain(shapes, batches, ctx)
        check(orc, shapes, batches, fused)
        for (k, p, n, g), x, (f1, g1), (f2, g2) in zip(shapes, batches, fused, plain):
            fl, fs = orc.batch_fitness_ld(k, p, x)
            assert np.max(np.abs(f1 - f2) / fs) <= 2 * TOL
            if k == N.RASTRIGIN:  # the same values whatever lanes the plan gave the rows
                assert np.array_equal(f1, f2) and (g1 is None or np.array_equal(g1, g2))
        for i in range(len(shapes)):
            lanes, tiles = ep.info(i)
            assert tiles >= 1 and lanes in (0, 1, 2, 4, 8, 16, 32)
    finally:
        ep.close()


def test_epochs_in_flight(ctx, orc):
    shapes, b1 = shapes_and_batches(islands=9, seed=7)
    b2 = [W.uniform_batch(k, p, n, seed=100 + i) for i, (k, p, n, g) in enumerate(shapes)]
    b3 = [W.uniform_batch(k, p, n, seed=200 + i) for i, (k, p, n, g) in enumerate(shapes)]
    ep = A.Epoch(shapes, ctx)
    try:
        o1 = ep.submit(b1)
        o2 = ep.submit(b2)
        o3 = ep.submit(b3)
        with pytest.raises(ValueError):
            ep.submit(b1)  # every staging set busy
        r1 = ep.collect()
        r2 = ep.collect()
        r3 = ep.collect()
        assert r1 is o1 and r2 is o2 and r3 is o3
        check(orc, shapes, b1, r1)
        check(orc, shapes, b2, r2)
        check(orc, shapes, b3, r3)
        # repeat run gives identical results (deterministic tiles and order)
        again = ep.run(b1)
        for (f1, g1), (f2, g2) in zip(r1, again):
            assert np.array_equal(f1, f2) and (g1 is None or np.array_equal(g1, g2))
    finally:
        ep.close()


def test_epoch_shape_mismatch_is_rejected(ctx):
    shapes, batches = shapes_and_batches(islands=3, seed=9)
    ep = A.Epoch(shapes, ctx)
    try:
        bad = (N.pgx_request * 3)()
        for i, (k, p, n, g) in enumerate(shapes):
            bad[i].kind, bad[i].param, bad[i].n_dvs = k, p, n + 1
        with pytest.raises(ValueError, match="does not match the epoch plan"):
            N.check(N.lib().pgx_epoch_run(ep.handle, bad))
    finally:
        ep.close()


def test_collector_threads_on_gpu(ctx, orc):
    import threading

    shapes, batches = shapes_and_batches(islands=6, seed=11)
    col = A.Collector(shapes, deadline_s=5.0, ctx=ctx)
    out = {}

    def island(i):
        out[i] = col.evaluate(i, batches[i])

    ts = [threading.Thread(target=island, args=(i,)) for i in range(6)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=60)
    assert col.epochs_run == 1 and sorted(out) == list(range(6))
    check(orc, shapes, batches, [out[i] for i in range(6)])


def test_in_place_staged_and_unaligned_epochs_agree(ctx, monkeypatch):
    """The in-place epochs (the kernel reading and writing the islands' arrays
    over NVLink-C2C), the staged ones (PGX_EPOCH_STAGED=1: packing, copies,
    unpacking) and in-place plans handed arrays that are not 16-byte aligned
    (they fall back to the staged graph) give bit-identical results: the same
    kernel evaluates the same rows."""
    shapes, batches = shapes_and_batches(islands=12, seed=11, grad_every=2)
    ep = A.Epoch(shapes, ctx)
    try:
        direct = ep.run(batches)
        # arrays at an 8-byte offset inside larger buffers: not 16-byte aligned
        raw_x = [np.empty(x.size + 1) for x in batches]
        shifted = []
        for r, x in zip(raw_x, batches):
            v = r[1:] if r.ctypes.data % 16 == 0 else r[:-1]
            v[:] = x.ravel()
            shifted.append(v.reshape(x.shape))
        outs = []
        for k, p, n, g in shapes:
            rf = np.empty(n + 1)
            f = rf[1:] if rf.ctypes.data % 16 == 0 else rf[:-1]
            gr = None
            if g:
                nx = shifted[len(outs)].shape[1]
                rg = np.empty(n * nx + 1)
                gr = (rg[1:] if rg.ctypes.data % 16 == 0 else rg[:-1]).reshape(n, nx)
            outs.append((f, gr))
        unaligned = ep.run(shifted, outs)
    finally:
        ep.close()
    monkeypatch.setenv("PGX_EPOCH_STAGED", "1")
    ep = A.Epoch(shapes, ctx)
    try:
        staged = ep.run(batches)
    finally:
        ep.close()
    for (f1, g1), (f2, g2), (f3, g3) in zip(direct, staged, unaligned):
        assert np.array_equal(f1, f2) and np.array_equal(f1, f3)
        if g1 is not None:
            assert np.array_equal(g1, g2) and np.array_equal(g1, g3)


def test_gradients_written_over_their_inputs(ctx):
    """A request whose gradient array is its own decision-vector array: the
    epoch must read every input before writing (the in-place path detects the
    overlap and takes the staged one)."""
    shapes, batches = shapes_and_batches(islands=6, seed=13, grad_every=1)
    ep = A.Epoch(shapes, ctx)
    try:
        want = ep.run(batches)
        xs = [np.array(x, dtype=np.float64, copy=True) for x in batches]
        outs = [(np.empty(n), xs[i]) for i, (k, p, n, g) in enumerate(shapes)]
        got = ep.run(xs, outs)
    finally:
        ep.close()
    for (f1, g1), (f2, g2) in zip(want, got):
        assert np.array_equal(f1, f2) and np.array_equal(g1, g2)


def test_autotune_cache_is_keyed_by_the_build(tmp_path):
    """The autotuner's cached choices carry the library's build identity: a
    line written by another build of the kernels is neither used nor kept (the
    shape is re-tuned), a line of this build is used as written. Runs in a
    fresh process, since a process loads the cache file once."""
    import os
    import subprocess
    import sys

    import torch

    bid = N.lib().pgx_build_id().decode()
    prop = torch.cuda.get_device_properties(0)
    tail = f"{prop.multi_processor_count}:{prop.major}{prop.minor}"
    stale_key = f"0123456789abcdef/{N.RASTRIGIN}:37:37:1:{tail}"
    fresh_key = f"{bid}/{N.ROSENBROCK}:41:41:1:{tail}"
    cache = tmp_path / "autotune.txt"
    cache.write_text(f"{stale_key} 2 1\n{fresh_key} 4 1\n")
    code = ("from pagmo2_gb300 import archipelago as A, _native as N\n"
            "ep = A.Epoch([(N.RASTRIGIN, 37, 100, True), (N.ROSENBROCK, 41, 100, True)])\n"
            "print('LANES', ep.info(0)[0], ep.info(1)[0])\n"
            "ep.close()\n")
    root = Path(__file__).resolve().parents[1]
    env = dict(os.environ, PGX_AUTOTUNE_CACHE=str(cache), PYTHONPATH=str(root))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=300, cwd=root)
    assert r.returncode == 0, r.stdout + r.stderr
    lanes = [int(v) for v in r.stdout.split("LANES")[1].split()]
    assert lanes[1] == 4  # this build's cached choice
    lines = cache.read_text().splitlines()
    assert not any(ln.startswith("0123456789abcdef/") for ln in lines)
    assert any(ln.startswith(f"{bid}/{N.RASTRIGIN}:37:37:1:") for ln in lines)  # re-tuned and stored
    assert any(ln.startswith(fresh_key + " 4 ") for ln in lines)
