"""Dataflow solve sweeps (FP32 factors).

The block steps of a level's large fronts run as one launch of persistent
CTAs that hand each step to the next through counters, with the products
P_ib = L_ib X_b formed after the factorization; schedule solve_dataflow < 0
restores one launch per block step.  LDL^T factors use the step launches
unless solve_dataflow > 0, so their case asks for the dataflow sweeps.  Both must give the same solutions to
FP32 accuracy (the sums run in different orders), the refined solve must
reach the 1e-14 backward error, and every partial job must agree.  The
bounded waits are checked on a synthetic sweep whose counter is never set:
the wait gives up with ST_TIMEOUT instead of hanging, and the device stays
usable afterwards."""
import ctypes

import numpy as np
import pytest

from sylver_gb300 import workloads as w

pytestmark = pytest.mark.gpu

ST_TIMEOUT = 32


def _solves(sylver, an, val, rhs, mode, posdef):
    sylver.set_schedule(solve_dataflow=mode)
    try:
        f = sylver.Factor(an, posdef, val, precision=sylver.FP32, ir_max_iter=0)
        assert f.flag >= 0
        out = {job: f.solve(rhs, job=job) for job in (0, 1, 3)}
        fr = sylver.Factor(an, posdef, val, precision=sylver.FP32, ir_max_iter=10)
        out["refined"] = fr.solve(rhs)
        return out
    finally:
        sylver.set_schedule()


@pytest.mark.parametrize("case", ["lognormal27_20", "lognormal27_24", "dense_700",
                                  "shifted_laplace3d_20"])
def test_dataflow_matches_step_launches(sylver, gpu, case):
    posdef, mode = True, 0
    if case.startswith("lognormal"):
        p = w.lognormal27(int(case.split("_")[1]), nrhs=1)
        a, order = p.a, p.order
    elif case.startswith("shifted"):
        p = w.shifted_laplace3d(20, nrhs=1)
        a, order, posdef, mode = p.a, p.order, False, 1
    else:
        import scipy.sparse as sp
        rng = np.random.default_rng(3)
        g = rng.standard_normal((700, 700))
        a = w.SymMatrix.from_scipy(sp.csc_matrix(g @ g.T / 700 + np.eye(700)))
        order = None
    an = sylver.Analysis(a.n, a.ptr, a.row, order=order)
    assert an.inform.maxfront > 256  # fronts with several 256-column blocks
    rhs = np.asfortranarray(np.random.default_rng(5).standard_normal((a.n, 16)))
    df = _solves(sylver, an, a.val, rhs, mode, posdef)
    st = _solves(sylver, an, a.val, rhs, -1, posdef)
    # the sweeps add in different orders (the backward one through atomics); on the
    # indefinite factor, entries of L up to 1/u = 100 under threshold pivoting amplify
    # those FP32 rounding differences (the backward sweep alone grows b by ~200 here)
    tol = 1e-4 if posdef else 1e-3
    for job in (0, 1, 3):
        scale = np.abs(st[job]).max()
        assert np.abs(df[job] - st[job]).max() <= tol * scale, job
    full = a.to_scipy_full()
    assert w.backward_error(full, df["refined"], rhs).max() <= 1e-14
    assert w.backward_error(full, st["refined"], rhs).max() <= 1e-14


def test_dataflow_bounded_wait_gives_up(sylver, gpu):
    lib = sylver.load()
    status, secs = ctypes.c_uint(99), ctypes.c_double(-1.0)
    assert lib.sylver_gb300_dataflow_selftest(0, ctypes.byref(status), ctypes.byref(secs)) == 0
    assert status.value == 0
    assert lib.sylver_gb300_dataflow_selftest(1, ctypes.byref(status), ctypes.byref(secs)) == 0
    assert status.value & ST_TIMEOUT
    assert 0.0 < secs.value < 10.0, secs.value
    # the context is still usable: a full factor + refined solve afterwards
    p = w.lognormal27(12, nrhs=2)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    f = sylver.Factor(an, True, p.a.val, precision=sylver.FP32, ir_max_iter=10)
    x = f.solve(p.rhs)
    assert w.backward_error(p.a.to_scipy_full(), x, p.rhs).max() <= 1e-14
