"""GPU Cholesky path through the C-ABI against the CPU oracle.

Bars (the benchmark spec): FP64 path -- backward error <= 1e-14 and the solution
agrees with the oracle's to 1e-10 relative; FP32 factors + FP64 iterative
refinement -- the same backward error after refinement."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from sylver_gb300 import workloads as w

pytestmark = pytest.mark.gpu

SPD = [n for n in golden_names() if load_golden(n)["posdef"] and load_golden(n)["flag"] == 0]


def run(sylver, g, precision, ir=0):
    an = sylver.Analysis(g["n"], g["ptr"], g["row"], order=g["order"])
    f = sylver.Factor(an, True, g["val"], precision=precision, ir_max_iter=ir)
    return an, f


@pytest.mark.parametrize("name", SPD)
@pytest.mark.parametrize("precision", [0, 1])
def test_spd_golden(sylver, orc, gpu, name, precision):
    g = load_golden(name)
    an, f = run(sylver, g, precision, ir=10)
    assert f.flag == 0, f.inform.as_dict()
    full = w.SymMatrix(g["n"], g["ptr"], g["row"], g["val"]).to_scipy_full()
    x = f.solve(g["rhs"])
    be = w.backward_error(full, x, g["rhs"]).max()
    assert be <= 1e-14, (be, f.solve_stats())
    o = orc.OracleFactor(True, an.symbolic(), g["val"])
    xo = o.solve(g["rhs"])
    xo = xo + o.solve(g["rhs"] - full @ xo)
    assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()
    if "x_true" in g:
        assert np.abs(x - g["x_true"]).max() <= 1e-10


@pytest.mark.parametrize("precision", [0, 1])
def test_spd_plain_solve_matches_oracle(sylver, orc, gpu, precision):
    """Without refinement the GPU factor solves like the FP64 oracle factor
    (FP64) or to FP32 accuracy (FP32)."""
    g = load_golden("lognormal27_7")
    an, f = run(sylver, g, precision, ir=0)
    o = orc.OracleFactor(True, an.symbolic(), g["val"])
    xo = o.solve(g["rhs"])
    if precision == 0:
        x = f.solve(g["rhs"])
        assert np.abs(x - xo).max() <= 1e-11 * np.abs(xo).max()
    # partial jobs: fwd then bwd equals the full solve of the same factor
    y = f.solve(g["rhs"], job=1)
    y = f.solve(y, job=3)
    yo = o.solve(o.solve(g["rhs"], job=1), job=3)
    tol = 1e-11 if precision == 0 else 2e-4
    assert np.abs(y - yo).max() <= tol * np.abs(yo).max()


def test_not_posdef_flag(sylver, gpu):
    g = load_golden("not_posdef_5")
    an, f = run(sylver, g, 0)
    assert f.flag == -6
    with pytest.raises(RuntimeError):
        f.solve(g["rhs"])  # call sequence error after a failed factorization


def test_solve_arg_errors(sylver, gpu):
    g = load_golden("laplace2d_12")
    an, f = run(sylver, g, 0)
    import ctypes
    lib = sylver.load()
    x = np.zeros((g["n"], 1), order="F")
    inf = sylver.Inform()
    o = sylver.default_options()
    P = ctypes.c_void_p
    lib.spldlt_solve(0, 1, x.ctypes.data_as(P), g["n"] - 1, an.akeep, f.fkeep, ctypes.byref(o),
                     ctypes.byref(inf))
    assert inf.flag == -10
    lib.spldlt_solve(0, 0, x.ctypes.data_as(P), g["n"], an.akeep, f.fkeep, ctypes.byref(o),
                     ctypes.byref(inf))
    assert inf.flag == -10
    lib.spldlt_solve(2, 1, x.ctypes.data_as(P), g["n"], an.akeep, f.fkeep, ctypes.byref(o),
                     ctypes.byref(inf))
    assert inf.flag == -11
    lib.spldlt_solve(7, 1, x.ctypes.data_as(P), g["n"], an.akeep, f.fkeep, ctypes.byref(o),
                     ctypes.byref(inf))
    assert inf.flag == -11


@pytest.mark.parametrize("k,precision", [(20, 0), (24, 1), (40, 1)])
def test_spd_medium_grids(sylver, orc, gpu, k, precision):
    """Fronts large enough for the panel / tile-update kernels."""
    p = w.lognormal27(k, nrhs=3)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    assert an.inform.maxfront > 256
    f = sylver.Factor(an, True, p.a.val, precision=precision, ir_max_iter=10)
    assert f.flag == 0
    full = p.a.to_scipy_full()
    x = f.solve(p.rhs)
    be = w.backward_error(full, x, p.rhs).max()
    assert be <= 1e-14, (be, f.solve_stats())
    if k <= 24:
        o = orc.OracleFactor(True, an.symbolic(), p.a.val)
        xo = o.solve(p.rhs)
        xo = xo + o.solve(p.rhs - full @ xo)
        assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()


def test_many_rhs_and_ldx(sylver, gpu):
    """More right-hand sides than one solve launch takes (32), ldx > n."""
    p = w.laplace2d(30, nrhs=1)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    f = sylver.Factor(an, True, p.a.val)
    rng = np.random.default_rng(9)
    n = p.a.n
    b = np.asfortranarray(rng.standard_normal((n + 5, 37)))
    x = f.solve(b[:, :])  # ldx = n + 5
    full = p.a.to_scipy_full()
    be = w.backward_error(full, x[:n], b[:n]).max()
    assert be <= 1e-14


def test_refactorize_reuses_fkeep(sylver, gpu):
    p = w.laplace2d(25, nrhs=1)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    f = sylver.Factor(an, True, p.a.val)
    x1 = f.solve(p.rhs)
    assert f.refactor(2.0 * p.a.val) == 0
    x2 = f.solve(p.rhs)
    np.testing.assert_allclose(x2, 0.5 * x1, rtol=1e-12, atol=1e-14)


def test_trivial_sizes(sylver, gpu):
    # n = 1
    an = sylver.Analysis(1, np.array([1, 2]), np.array([1]))
    f = sylver.Factor(an, True, np.array([4.0]))
    assert f.flag == 0
    np.testing.assert_allclose(f.solve(np.array([[2.0]])), [[0.5]])
    # diagonal matrix
    n = 50
    an = sylver.Analysis(n, np.arange(1, n + 2), np.arange(1, n + 1))
    d = np.arange(1.0, n + 1)
    f = sylver.Factor(an, True, d)
    np.testing.assert_allclose(f.solve(np.ones((n, 1)))[:, 0], 1.0 / d, rtol=1e-15)


def _dense_spd(n, seed):
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, n))
    a = g @ g.T / n + np.eye(n)
    return w.SymMatrix.from_scipy(sp.csc_matrix(a)), a


@pytest.mark.parametrize("width,group", [(64, 2), (128, 2), (192, 2), (256, 2), (-1, 0),
                                         (128, 1), (128, 3), (64, 4), (192, 3)])
def test_fp32_panel_widths(sylver, orc, gpu, width, group):
    """Blocked FP32 large-front path: every outer panel width and number of
    panels per trailing update (and the 64-column SIMT path, width < 0)
    gives FP32-accurate factors, and FP64 refinement reaches the 1e-14
    backward error.  One dense 700 x 700 front (the last panel and the last
    group ragged) and a 3D grid whose separators exceed one panel."""
    sylver.set_schedule(fs_panel_cols=width, fs_panel_group=group)
    try:
        a, dense = _dense_spd(700, 3)
        rng = np.random.default_rng(4)
        b = rng.standard_normal((700, 2))
        an = sylver.Analysis(a.n, a.ptr, a.row)
        assert an.inform.maxfront >= 600
        f = sylver.Factor(an, True, a.val, precision=sylver.FP32, ir_max_iter=0)
        assert f.flag == 0
        x0 = f.solve(b)
        xt = np.linalg.solve(dense, b)
        assert np.abs(x0 - xt).max() <= 1e-4 * np.abs(xt).max()
        f2 = sylver.Factor(an, True, a.val, precision=sylver.FP32, ir_max_iter=10)
        x = f2.solve(b)
        assert np.abs(x - xt).max() <= 1e-12 * np.abs(xt).max()
        p = w.lognormal27(22, nrhs=2)
        an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
        assert an.inform.maxfront > 256
        f = sylver.Factor(an, True, p.a.val, precision=sylver.FP32, ir_max_iter=10)
        assert f.flag == 0
        x = f.solve(p.rhs)
        full = p.a.to_scipy_full()
        assert w.backward_error(full, x, p.rhs).max() <= 1e-14, f.solve_stats()
        o = orc.OracleFactor(True, an.symbolic(), p.a.val)
        xo = o.solve(p.rhs)
        xo = xo + o.solve(p.rhs - full @ xo)
        assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()
    finally:
        sylver.set_schedule()


def test_fp32_blocked_not_posdef(sylver, gpu):
    """A non-positive pivot inside a blocked diagonal block is reported."""
    a, dense = _dense_spd(400, 5)
    dense = dense.copy()
    dense[300, 300] = -50.0
    import scipy.sparse as sp
    m = w.SymMatrix.from_scipy(sp.csc_matrix(dense))
    an = sylver.Analysis(m.n, m.ptr, m.row)
    f = sylver.Factor(an, True, m.val, precision=sylver.FP32)
    assert f.flag == -6


def test_refinement_not_converged_is_reported(sylver, gpu):
    """Refinement that stops at ir_max_iter above ir_tol returns the warning
    SYLVER_GB300_WARNING_IR_NOT_CONVERGED (9) in inform.flag, with the error
    reached in the statistics; a converged refinement returns 0."""
    p = w.lognormal27(12, nrhs=2)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    f = sylver.Factor(an, True, p.a.val, precision=sylver.FP32, ir_tol=1e-30, ir_max_iter=2)
    x = f.solve(p.rhs)
    assert f.solve_inform.flag == sylver.WARNING_IR_NOT_CONVERGED
    it, be = f.solve_stats()
    assert it == 2 and 1e-30 < be
    assert len(f.solve_history()) == 3
    assert np.all(np.isfinite(x))
    g = sylver.Factor(an, True, p.a.val, precision=sylver.FP32, ir_tol=1e-14, ir_max_iter=10)
    g.solve(p.rhs)
    assert g.solve_inform.flag == 0
    assert g.solve_stats()[1] <= 1e-14


@pytest.mark.parametrize("nrhs", [1, 5, 16, 17, 33])
def test_solve_rhs_counts_match_oracle(sylver, orc, gpu, nrhs):
    """Right-hand-side counts that take every pass layout of the solve
    kernels (4, 8 and 16 per pass, several passes, more than one 32-column
    launch): the FP64 solve without refinement agrees with the oracle's, and
    the refined FP32 solve reaches the backward error, on a matrix with both
    small and blocked (large) fronts and contribution rows at every level."""
    p = w.lognormal27(20, nrhs=1)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    rhs = np.asfortranarray(np.random.default_rng(nrhs).standard_normal((p.a.n, nrhs)))
    o = orc.OracleFactor(True, an.symbolic(), p.a.val)
    xo = o.solve(rhs)
    f64 = sylver.Factor(an, True, p.a.val, precision=sylver.FP64)
    x = f64.solve(rhs)
    assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()
    f32 = sylver.Factor(an, True, p.a.val, precision=sylver.FP32, ir_max_iter=10)
    x32 = f32.solve(rhs)
    assert w.backward_error(p.a.to_scipy_full(), x32, rhs).max() <= 1e-14



@pytest.mark.parametrize("precision", [0, 1])
def test_factors_bitwise_reproducible(sylver, gpu, precision):
    """The assembly sums each front entry's original value and then its
    children in child order without atomics, so factorizing the same values
    twice into the same factor storage gives the same bits, FP64 and FP32 (the
    tensor-core updates included)."""
    import ctypes
    p = w.lognormal27(20, nrhs=1)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    f = sylver.Factor(an, True, p.a.val, precision=precision)
    assert f.flag == 0
    lib = sylver.load()
    nb = lib.sylver_gb300_fkeep_factor_bytes(f.fkeep, None, 0)
    assert nb > 0
    first = np.empty(nb, np.uint8)
    assert lib.sylver_gb300_fkeep_factor_bytes(f.fkeep, first.ctypes.data_as(ctypes.c_void_p),
                                               nb) == nb
    for _ in range(2):
        assert f.refactor(p.a.val, precision=precision) == 0
        again = np.empty(nb, np.uint8)
        assert lib.sylver_gb300_fkeep_factor_bytes(
            f.fkeep, again.ctypes.data_as(ctypes.c_void_p), nb) == nb
        assert np.array_equal(first, again)


def test_front_memory_economy_matches(sylver, orc, gpu):
    """Front storage economy forced on (schedule front_memory = 1: contribution
    blocks given back to later fronts once the parent's level has assembled
    them, every level assembled just before it, the mode large problems take
    automatically): the same solutions as the default layout, FP64 against the
    oracle and FP32 with refinement."""
    p = w.lognormal27(20, nrhs=2)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    ref = sylver.Factor(an, True, p.a.val).solve(p.rhs)
    o = orc.OracleFactor(True, an.symbolic(), p.a.val)
    xo = o.solve(p.rhs)
    try:
        sylver.set_schedule(front_memory=1)
        f = sylver.Factor(an, True, p.a.val)
        x = f.solve(p.rhs)
        f32 = sylver.Factor(an, True, p.a.val, precision=sylver.FP32, ir_max_iter=10)
        x32 = f32.solve(p.rhs)
    finally:
        sylver.set_schedule()
    assert np.abs(x - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()
    assert w.backward_error(p.a.to_scipy_full(), x32, p.rhs).max() <= 1e-14


def _comb(nch=40, length=40, nsep=5):
    """nch independent chains of `length` unknowns, each coupled through its
    last unknown to a dense separator of nsep: the root front has nch
    children with contribution blocks."""
    import scipy.sparse as sp
    n = nch * length + nsep
    rows, cols, vals = [], [], []
    for k in range(nch):
        b = k * length
        for i in range(length - 1):
            rows.append(b + i + 1); cols.append(b + i); vals.append(-1.0)
        for t in range(nsep):
            rows.append(nch * length + t); cols.append(b + length - 1); vals.append(-0.5)
    for t in range(nsep):
        for u in range(t):
            rows.append(nch * length + t); cols.append(nch * length + u); vals.append(-0.25)
    low = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    off = low + low.T
    d = np.asarray(abs(off).sum(axis=1)).ravel() + 1.0
    return w.SymMatrix.from_scipy(sp.csr_matrix(off + sp.diags(d)))


@pytest.mark.parametrize("case", ["grid", "comb40"])
def test_assembly_paths(sylver, orc, gpu, case):
    """Fronts are assembled in one pass per level (zero, original entries and
    children summed per column, stored once) unless a front has more than 32
    children with contribution blocks, when zeroing + original entries +
    extend-add run instead.  The per-kind profile shows which ran; both solve
    like the FP64 oracle and reach 1e-14 with FP32 factors and refinement."""
    if case == "grid":
        p = w.lognormal27(12, nrhs=2)
        a, order, rhs = p.a, p.order, p.rhs
    else:
        a = _comb()
        order = w.natural_order(a.n)
        rhs = np.asfortranarray(np.random.default_rng(9).standard_normal((a.n, 2)))
    an = sylver.Analysis(a.n, a.ptr, a.row, order=order)
    sy = an.symbolic()
    par = np.asarray(sy["sparent"]) - 1
    nrow, ncol = np.diff(sy["rptr"]), np.diff(sy["sptr"])
    kids = np.bincount(par[(par >= 0) & (par < sy["nnodes"]) & (nrow > ncol)],
                       minlength=sy["nnodes"])
    one_pass = kids.max() <= 32
    assert one_pass == (case == "grid")
    f = sylver.Factor(an, True, a.val)
    assert f.flag == 0
    prof = f.profile()
    if one_pass:
        assert prof["memset"]["launches"] == 0 and prof["init_a"]["launches"] == 0
    else:
        assert prof["memset"]["launches"] > 0 and prof["init_a"]["launches"] > 0
    assert prof["extend_add"]["launches"] > 0
    x = f.solve(rhs)
    o = orc.OracleFactor(True, sy, a.val)
    xo = o.solve(rhs)
    assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()
    f32 = sylver.Factor(an, True, a.val, precision=sylver.FP32, ir_max_iter=10)
    assert w.backward_error(a.to_scipy_full(), f32.solve(rhs), rhs).max() <= 1e-14
