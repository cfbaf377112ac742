"""Runs one kernel of the batch-evaluation path on a chosen workload, for profilers.

    python profile_case.py --case rosenbrock_fg --rows 16384
    ncu --set full --clock-control none -k regex:rosenbrock -s 2 -c 1 \
        python profile_case.py --case rosenbrock_fg --rows 16384

Inputs are seeded synthetic batches resident on the device; --warmup launches
are followed by --launches timed ones (CUDA events; numbers printed under a
profiler are not benchmark values). Cases:

  rastrigin_fg / rastrigin_f    dim 50 (--dim)
  rosenbrock_fg / rosenbrock_f  dim 1000 (--dim)
  lj_fg / lj_f                  150 atoms (--atoms)
  ackley_f / griewank_f / schwefel_f   dim 50 (--dim), fitness only
  zdt<k>_f                      ZDT k, param 30 (--dim), objectives n x 2
  dtlz<k>_f                     DTLZ k, dim 12 (--dim), 3 objectives (--fdim)
  survival                      NSGA-II survival of --rows nested-front points x 3
  select_best                   select_best_N_mo(--rows nested-front points x 3, rows / 2)
  sort_population               sort_population_mo(--rows nested-front points x 3)
  hypervolume                   hypervolume of --rows nested-front points x 3 (reference point max + 0.5)
  hv_wfg / hv_contributions     hypervolume / every point's contribution of --rows points on a sphere front of
                                --fdim objectives (default 5; reference point 1.1)
  archipelago                   the fused kernel of a 64-island mixed epoch (--rows unused)
  refine_rastrigin / refine_rosenbrock / refine_lj   batched basin hopping with gradient descent
                                (10 trials, stop 5, 20 steps) on --rows individuals
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", required=True)
    ap.add_argument("--rows", type=int, default=16384)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--launches", type=int, default=3)
    ap.add_argument("--atoms", type=int, default=150, help="lennard_jones cluster size (lj_* cases)")
    ap.add_argument("--dim", type=int, default=0, help="rastrigin/rosenbrock dimension (default 50 / 1000)")
    ap.add_argument("--fdim", type=int, default=3, help="DTLZ objectives (dtlz* cases)")
    ap.add_argument("--layers", type=int, default=30, help="nested fronts of the survival/select_best/sort cases")
    a = ap.parse_args()

    import numpy as np
    import torch

    from pagmo2_gb300 import _native as N
    from pagmo2_gb300 import workloads as W

    ctx = N.Context(0)
    L = N.lib()
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    n = a.rows
    if a.case == "archipelago":
        from pagmo2_gb300 import archipelago as A

        reqs = W.archipelago(64)
        ep = A.Epoch([(r.kind, r.param, r.n, True) for r in reqs], ctx)
        ep.run([r.dvs for r in reqs])

        def run():
            ep.launch_device(sp)
    elif a.case.startswith("refine_"):
        import ctypes as C

        kind, param, x = {"refine_rastrigin": (N.RASTRIGIN, a.dim or 50, lambda: W.rastrigin_batch(n, a.dim or 50)),
                          "refine_rosenbrock": (N.ROSENBROCK, a.dim or 1000,
                                                lambda: W.rosenbrock_batch(n, a.dim or 1000)),
                          "refine_lj": (N.LENNARD_JONES, a.atoms, lambda: W.lj_batch(n, a.atoms))}[a.case]
        d0 = torch.from_numpy(x()).cuda()
        dx = torch.empty_like(d0)
        df = torch.empty(n, dtype=torch.float64, device="cuda")
        de = torch.zeros(1, dtype=torch.int64, device="cuda")
        params = N.pgx_refine_params(10, 5, 20, 0.02, 0.05, 1e-7, 7)

        def run():
            with torch.cuda.stream(stream):
                dx.copy_(d0)
            N.check(L.pgx_refine_batch_device(ctx.handle, kind, param, C.byref(params), dx.data_ptr(), n,
                                              df.data_ptr(), de.data_ptr(), sp))
    elif a.case == "survival":
        p = W.nsga2_points(n, 3, layers=a.layers)
        dp = torch.from_numpy(p).cuda()
        i32 = lambda k: torch.empty(k, dtype=torch.int32, device="cuda")  # noqa: E731
        rank, dc, off, idx, nf = i32(n), i32(n), i32(n + 1), i32(n), i32(1)
        cd = torch.empty(n, dtype=torch.float64, device="cuda")

        def run():
            N.check(L.pgx_nsga2_survival_device(ctx.handle, dp.data_ptr(), n, 3, rank.data_ptr(), dc.data_ptr(),
                                                off.data_ptr(), idx.data_ptr(), nf.data_ptr(), cd.data_ptr(), sp))
    elif a.case == "hypervolume":
        p = W.nsga2_points(n, 3, layers=a.layers)
        r = np.ascontiguousarray(p.max(axis=0) + 0.5)
        dp = torch.from_numpy(np.ascontiguousarray(p)).cuda()
        dhv = torch.empty(1, dtype=torch.float64, device="cuda")

        def run():
            N.check(L.pgx_hypervolume_device(ctx.handle, dp.data_ptr(), n, 3, N.ptr(r), dhv.data_ptr(), sp))
    elif a.case in ("hv_wfg", "hv_contributions"):
        m = a.fdim if a.fdim != 3 else 5
        p = W.sphere_front(n, m)
        r = np.full(m, 1.1)
        dp = torch.from_numpy(p).cuda()
        dout = torch.empty(n, dtype=torch.float64, device="cuda")

        def run():
            if a.case == "hv_wfg":
                N.check(L.pgx_hypervolume_device(ctx.handle, dp.data_ptr(), n, m, N.ptr(r), dout.data_ptr(), sp))
            else:
                N.check(L.pgx_hypervolume_contributions_device(ctx.handle, dp.data_ptr(), n, m, N.ptr(r),
                                                               dout.data_ptr(), sp))
    elif a.case in ("select_best", "sort_population"):
        p = W.nsga2_points(n, 3, layers=a.layers)
        dp = torch.from_numpy(p).cuda()
        sel = torch.empty(n, dtype=torch.int32, device="cuda")
        st = torch.empty(1, dtype=torch.int32, device="cuda")

        def run():
            if a.case == "select_best":
                N.check(L.pgx_select_best_n_mo_device(ctx.handle, dp.data_ptr(), n, 3, n // 2, sel.data_ptr(),
                                                      st.data_ptr(), sp))
            else:
                N.check(L.pgx_sort_population_mo_device(ctx.handle, dp.data_ptr(), n, 3, sel.data_ptr(),
                                                        st.data_ptr(), sp))
    elif a.case.startswith(("zdt", "dtlz")):
        import ctypes as C

        fam = N.ZDT if a.case.startswith("zdt") else N.DTLZ
        pid = int(a.case.split("_")[0][3 if fam == N.ZDT else 4:])
        param = a.dim or (30 if fam == N.ZDT else 12)
        spec = N.mo_problem(fam, pid, param, a.fdim if fam == N.DTLZ else 0, 100)
        nx, nobj, _ = N.mo_problem_dims(spec)
        x = W.mo_uniform_batch(fam, pid, param, n, seed=47, fdim=a.fdim)
        dx = torch.from_numpy(x).cuda()
        df = torch.empty((n, nobj), dtype=torch.float64, device="cuda")

        def run():
            N.check(L.pgx_mo_batch_fitness_device(ctx.handle, C.byref(spec), dx.data_ptr(), n, df.data_ptr(), sp))
    else:
        name, mode = a.case.rsplit("_", 1)
        kind, param, x = {
            "rastrigin": (N.RASTRIGIN, a.dim or 50, lambda: W.rastrigin_batch(n, a.dim or 50)),
            "rosenbrock": (N.ROSENBROCK, a.dim or 1000, lambda: W.rosenbrock_batch(n, a.dim or 1000)),
            "lj": (N.LENNARD_JONES, a.atoms, lambda: W.lj_batch(n, a.atoms)),
            "ackley": (N.ACKLEY, a.dim or 50, lambda: W.uniform_batch(N.ACKLEY, a.dim or 50, n, 44)),
            "griewank": (N.GRIEWANK, a.dim or 50, lambda: W.uniform_batch(N.GRIEWANK, a.dim or 50, n, 45)),
            "schwefel": (N.SCHWEFEL, a.dim or 50, lambda: W.uniform_batch(N.SCHWEFEL, a.dim or 50, n, 46)),
        }[name]
        x = x()
        dx = torch.from_numpy(x).cuda()
        df = torch.empty(n, dtype=torch.float64, device="cuda")
        dg = torch.empty_like(dx) if mode == "fg" else None

        def run():
            N.check(L.pgx_batch_eval_device(ctx.handle, kind, param, dx.data_ptr(), n, df.data_ptr(),
                                            dg.data_ptr() if dg is not None else None, sp))
    for _ in range(a.warmup):
        run()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.launches):
        run()
    e1.record(stream)
    e1.synchronize()
    print(f"{a.case} rows={n}: {e0.elapsed_time(e1) / a.launches:.4f} ms per launch")
    ctx.close()


if __name__ == "__main__":
    main()
