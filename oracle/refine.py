"""Host restatement of the batched refinement of pgx_refine_batch -- TEST
INFRASTRUCTURE ONLY (the checker of tests/test_gpu_refine.py).

The loop of csrc/refine.cu, step for step, in Python doubles (every operation
rounded once, as the kernel rounds it; |d|^2 summed in the kernel's lane
order), driven by caller-supplied fitness-and-gradient evaluations of one
point: fed the GPU's own per-point values it must reproduce the GPU result bit
for bit; fed the reference's problem::fitness / problem::gradient
(src/problem.cpp:353, :456) it is the same algorithm on pagmo's own arithmetic.
The scheme is pagmo's monotonic basin hopping (src/algorithms/mbh.cpp:102-200,
the perturbation of :164-170) applied per individual, with projected-gradient
descent as the inner optimiser.
"""
from __future__ import annotations

import math

import numpy as np

_M64 = (1 << 64) - 1


def _mix(z: int) -> int:
    """splitmix64's finaliser (Steele, Lea and Flood, 2014)."""
    z = (z + 0x9E3779B97F4A7C15) & _M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
    return z ^ (z >> 31)


def uniform(seed: int, row: int, trial: int, coord: int) -> float:
    h = _mix(_mix((seed ^ _mix(row)) & _M64) ^ (((trial << 32) | coord) & _M64))
    return float(h >> 11) * 2.0 ** -53


def lanes_per_row(nx: int) -> int:
    """The row kernels' lanes per row for dimension nx (csrc/fitness.cu)."""
    g = 32
    while g >= 2:
        steps = (nx + g - 1) // g
        if nx >= g and 100 * nx >= 94 * g * steps:
            return g
        g >>= 1
    return 2 if nx >= 2 else 1


def refine_lanes(kind: int, nx: int) -> int:
    """Lanes per individual of the refinement kernel (csrc/refine.cu)."""
    if kind == 3:
        return 32
    own = lanes_per_row(nx)
    if kind == 1:
        return 32 if own >= 32 else (16 if own >= 16 else 8)
    return own


def _lane_sum(vals, lanes: int) -> float:
    part = [0.0] * lanes
    for i, v in enumerate(vals):
        part[i % lanes] = part[i % lanes] + v
    o = lanes // 2
    while o >= 1:
        part = [part[lane] + part[lane ^ o] for lane in range(lanes)]
        o //= 2
    return part[0]


def refine_one(fg, x0, lb, ub, row: int, hops: int, stop: int, steps: int, perturb: float, step0: float,
               step_min: float, seed: int, lanes: int):
    """One individual's chain. fg(x) -> (f, g) evaluates one point.
    Returns (best x, best f, evaluations)."""
    lb = [float(v) for v in lb]
    ub = [float(v) for v in ub]
    nx = len(lb)
    xb = [float(v) for v in x0]
    fb, _ = fg(np.array(xb))
    fb = float(fb)
    evals = 1
    failed = 0
    trial = 0
    while trial < hops and failed < stop:
        xc = []
        for i in range(nx):
            w = perturb * (ub[i] - lb[i])
            xl = max(xb[i] - w, lb[i])
            xu = min(xb[i] + w, ub[i])
            xc.append(xl + (xu - xl) * uniform(seed, row, trial, i))
        fc, gc = fg(np.array(xc))
        fc = float(fc)
        gc = [float(v) for v in gc]
        evals += 1
        eta = step0
        k = 0
        while k < steps and eta >= step_min:
            d2 = []
            for i in range(nx):
                d = (ub[i] - lb[i]) * gc[i]
                d2.append(d * d)
            q = _lane_sum(d2, lanes)
            if not (q > 0.0) or not math.isfinite(q):
                break
            c = eta / math.sqrt(q)
            xt = []
            for i in range(nx):
                s = ub[i] - lb[i]
                t = (c * s) * (s * gc[i])
                xt.append(min(max(xc[i] - t, lb[i]), ub[i]))
            ft, gt = fg(np.array(xt))
            ft = float(ft)
            evals += 1
            if ft < fc:
                xc, gc, fc = xt, [float(v) for v in gt], ft
                eta = min(2.0 * eta, 1.0)
            else:
                eta *= 0.5
            k += 1
        if fc < fb:
            xb, fb = list(xc), fc
            failed = 0
        else:
            failed += 1
        trial += 1
    return np.array(xb), fb, evals
