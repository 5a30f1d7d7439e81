"""GPU threshold-pivoted LDL^T through the C-ABI against the CPU oracle.

Parity bar: inertia (negative / zero / positive pivot counts) equals the
oracle's and the eigenvalue count exactly; FP64 and FP32 factors reach a
scaled backward error <= 1e-14 after FP64 refinement; the refined solution
agrees with the oracle's to 1e-10 relative (scaled by conditioning)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from sylver_gb300 import workloads as w

pytestmark = pytest.mark.gpu

INDEF = [n for n in golden_names() if not load_golden(n)["posdef"]]


def inertia_from_d(d):
    neg = zero = two = 0
    k = 0
    ne = len(d) // 2
    while k < ne:
        if k + 1 < ne and np.isinf(d[2 * k + 2]):
            a, b, c = d[2 * k], d[2 * k + 1], d[2 * k + 3]
            det, tr = a * c - b * b, a + c
            neg += 1 if det < 0 else (2 if tr < 0 else 0)
            two += 1
            k += 2
        else:
            zero += d[2 * k] == 0
            neg += d[2 * k] < 0
            k += 1
    return neg, zero, two


@pytest.mark.parametrize("name", INDEF)
@pytest.mark.parametrize("precision", [0, 1])
def test_ldlt_golden(sylver, orc, gpu, name, precision):
    g = load_golden(name)
    an = sylver.Analysis(g["n"], g["ptr"], g["row"], order=g["order"])
    f = sylver.Factor(an, False, g["val"], precision=precision, ir_max_iter=10)
    assert f.flag == g["flag"], f.inform.as_dict()
    neg, zero, pos = g["inertia"]
    assert f.inform.num_neg == neg
    if "closed_inertia" in g:
        assert f.inform.num_neg == g["closed_inertia"][0]
    o = orc.OracleFactor(False, an.symbolic(), g["val"])
    assert o.stats["num_neg"] == f.inform.num_neg
    d, piv = f.diag(g["n"])
    assert inertia_from_d(d)[0] == neg
    assert sorted(piv.tolist()) == list(range(1, len(piv) + 1)) or len(piv) < g["n"]
    if g["flag"] == 7:
        assert f.inform.matrix_rank == g["n"] - 1
        return
    full = w.SymMatrix(g["n"], g["ptr"], g["row"], g["val"]).to_scipy_full()
    x = f.solve(g["rhs"])
    be = w.backward_error(full, x, g["rhs"]).max()
    assert be <= 1e-14, (be, f.solve_stats())
    scale = max(1.0, 1e-3 / g["mineig"])
    assert np.abs(x - g["x"]).max() <= 1e-10 * scale * np.abs(g["x"]).max()


def test_ldlt_partial_jobs(sylver, gpu):
    g = load_golden("shifted_laplace3d_9")
    an = sylver.Analysis(g["n"], g["ptr"], g["row"], order=g["order"])
    f = sylver.Factor(an, False, g["val"])
    x0 = f.solve(g["rhs"], job=0)
    y = f.solve(f.solve(f.solve(g["rhs"], job=1), job=2), job=3)
    np.testing.assert_allclose(y, x0, rtol=1e-10, atol=1e-12 * np.abs(x0).max())
    y2 = f.solve(f.solve(g["rhs"], job=1), job=4)
    np.testing.assert_allclose(y2, x0, rtol=1e-10, atol=1e-12 * np.abs(x0).max())


@pytest.mark.parametrize("k,precision", [(16, 0), (20, 1)])
def test_ldlt_shifted_laplacian(sylver, gpu, k, precision):
    """Known answer: inertia of the 7-point Laplacian minus sigma*I."""
    p = w.shifted_laplace3d(k, nrhs=2)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    f = sylver.Factor(an, False, p.a.val, precision=precision, ir_max_iter=10)
    assert f.flag == 0
    assert f.inform.num_neg == p.inertia[0]
    x = f.solve(p.rhs)
    assert w.backward_error(p.a.to_scipy_full(), x, p.rhs).max() <= 1e-14


def test_ldlt_kkt_haynsworth(sylver, orc, gpu):
    """Known answer: [[H, B^T], [B, -delta I]] has brows negative pivots."""
    p = w.kkt(8, nnz_per_row=4, seed=11, nrhs=1)
    opts = sylver.default_options()
    opts.ordering = 1
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, options=opts)
    f = sylver.Factor(an, False, p.a.val, ir_max_iter=10)
    assert f.flag == 0
    assert f.inform.num_neg == p.inertia[0]
    o = orc.OracleFactor(False, an.symbolic(), p.a.val)
    assert o.stats["num_neg"] == p.inertia[0]
    x = f.solve(p.rhs)
    assert w.backward_error(p.a.to_scipy_full(), x, p.rhs).max() <= 1e-14


def test_ldlt_delays_move_up(sylver, gpu):
    """Rows scaled by 1000 (the reference's cause_delays) in a multi-front
    matrix: columns are delayed to parents and the answer stays right."""
    rng = np.random.default_rng(3)
    p = w.shifted_laplace3d(10, nrhs=1)
    full = p.a.to_scipy_full().tolil()
    n = p.a.n
    for idx in rng.choice(n, size=n // 8, replace=False):
        full[idx, :] = full[idx, :] * 1000.0
        full[:, idx] = full[:, idx] * 1000.0
    full = full.tocsr()
    # keep the diagonal small so these pivots fail the threshold test
    for idx in range(n):
        if abs(full[idx, idx]) > 100:
            full[idx, idx] = full[idx, idx] * 1e-6
    a = w.SymMatrix.from_scipy(full)
    an = sylver.Analysis(a.n, a.ptr, a.row, order=p.order)
    f = sylver.Factor(an, False, a.val, ir_max_iter=10)
    assert f.flag == 0
    ev = np.linalg.eigvalsh(full.toarray())
    assert f.inform.num_neg == int(np.sum(ev < 0))
    assert f.inform.num_delay > 0 or f.inform.num_two > 0
    b = np.asfortranarray(rng.standard_normal((a.n, 1)))
    x = f.solve(b)
    assert w.backward_error(full, x, b).max() <= 1e-14


@pytest.mark.parametrize("scaling", [0, 1, 3, 4])
def test_kkt_matching_ordering_and_scalings(sylver, gpu, scaling):
    """Matching-based ordering (options.ordering = 2) on the saddle-point
    matrix with each scaling option: 0 none, 1 matching scaling of the
    values, 3 the scaling saved by the analysis, 4 equilibration.  Inertia by
    Haynsworth and a refined backward error <= 1e-14 in every case; the
    saved scaling leaves no warning, the others warn that it went unused
    (flag 8, src/spldlt_factorize_mod.F90:721-725)."""
    p = w.kkt(10, nrhs=1)
    o = sylver.default_options()
    o.ordering = 2
    o.scaling = scaling
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, options=o, val=p.a.val)
    assert an.flag >= 0
    f = sylver.Factor(an, False, p.a.val, ir_max_iter=10, options=o)
    assert f.flag == (0 if scaling == 3 else 8), f.inform.as_dict()
    assert f.inform.num_neg == p.inertia[0]
    x = f.solve(p.rhs)
    assert w.backward_error(p.a.to_scipy_full(), x, p.rhs).max() <= 1e-14
    print("kkt10 ordering=2 scaling", scaling, "delays", f.inform.num_delay,
          "two", f.inform.num_two)


def test_kkt_matching_ordering_fewer_delays(sylver, gpu):
    """The matched 2x2 pairs stay together: fewer delayed pivots than the
    plain nested dissection on the same saddle-point matrix."""
    p = w.kkt(12, nrhs=1)
    plain = sylver.Analysis(p.a.n, p.a.ptr, p.a.row)
    f0 = sylver.Factor(plain, False, p.a.val)
    o = sylver.default_options()
    o.ordering = 2
    o.scaling = 3
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, options=o, val=p.a.val)
    f1 = sylver.Factor(an, False, p.a.val, options=o)
    print("kkt12 delays: nested dissection", f0.inform.num_delay, "matching",
          f1.inform.num_delay)
    assert f0.inform.num_neg == f1.inform.num_neg == p.inertia[0]
    assert f1.inform.num_delay < f0.inform.num_delay
