"""One analysis + factorization + refined solve, for profiling.

    python -m sylver_gb300.profile_step [k] [fp32|fp64] [nrhs] [spd|indef]

spd (default): the 3D 27-point log-normal workload on a k^3 grid (default
80), Cholesky.  indef: the 3D 7-point Laplacian on k^3 minus sigma*I
(threshold-pivoted LDL^T, u = 0.01).  Runs once through the C-ABI:
spldlt_analyse, spldlt_factorize_mixed and spldlt_solve with FP64 refinement
to a backward error of 1e-14, and prints the timings, refinement statistics
and launch counts.  Use it under a profiler (ncu) to capture the launches of
exactly one step.
"""
from __future__ import annotations

import sys
import time

import numpy as np

from . import FP32, FP64, Analysis, Factor
from . import workloads as w


def main(argv=None):
    argv = list(sys.argv[1:] if argv is None else argv)
    k = int(argv[0]) if argv else 80
    prec = FP64 if (len(argv) > 1 and argv[1] == "fp64") else FP32
    nrhs = int(argv[2]) if len(argv) > 2 else 16
    indef = len(argv) > 3 and argv[3] == "indef"
    p = w.shifted_laplace3d(k, nrhs=nrhs) if indef else w.lognormal27(k, nrhs=nrhs)
    t0 = time.perf_counter()
    an = Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    t1 = time.perf_counter()
    f = Factor(an, not indef, p.a.val, precision=prec, ir_tol=1e-14, ir_max_iter=20)
    t2 = time.perf_counter()
    x = f.solve(p.rhs)
    t3 = time.perf_counter()
    be = w.backward_error(p.a.to_scipy_full(), x, p.rhs).max()
    it, be_dev = f.solve_stats()
    print(f"{p.name} n={p.a.n} precision={'fp32' if prec == FP32 else 'fp64'} flag={f.flag}"
          + (f" num_neg={f.inform.num_neg} (closed form {p.inertia[0]})" if indef else ""))
    print(f"analyse {t1 - t0:.3f}s factorize {t2 - t1:.3f}s solve {t3 - t2:.3f}s "
          f"ir_iters={it} bwd_err={be:.3e} (device {be_dev:.3e})")
    print("counters", f.counters())
    print("refinement history", ["%.2e" % v for v in f.solve_history()])
    ok = f.flag == 0 and np.isfinite(be) and be <= 1e-14
    if indef:
        ok = ok and f.inform.num_neg == p.inertia[0]
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
