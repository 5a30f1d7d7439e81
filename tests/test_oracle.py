"""The CPU oracle against the golden vectors and the reference tests' bounds.

Bounds: reference node tests require u * bwderr <= 5e-14 with full
elimination (tests/testing_factor_node_indef.hxx:426, :440); the Fortran
driver check uses a scaled residual < 5e-11 (tests/sylver_test_mod.F90:19).
Inertia must equal the eigenvalue count and, where one exists, the closed
form (shifted Laplacian spectrum, Haynsworth for KKT)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from sylver_gb300 import workloads as w

U = 0.01


def analyse(sylver, g, nemin=32):
    opts = sylver.default_options()
    opts.nemin = nemin
    an = sylver.Analysis(g["n"], g["ptr"], g["row"], order=g["order"], options=opts)
    assert an.flag >= 0
    return an


@pytest.mark.parametrize("name", golden_names())
def test_oracle_golden(sylver, orc, name):
    g = load_golden(name)
    an = analyse(sylver, g)
    sy = an.symbolic()
    o = orc.OracleFactor(g["posdef"], sy, g["val"], u=U)
    assert o.flag == g["flag"], o.stats
    if g["flag"] < 0:
        return
    full = w.SymMatrix(g["n"], g["ptr"], g["row"], g["val"]).to_scipy_full()
    if not g["posdef"]:
        neg, zero, pos = g["inertia"]
        assert o.stats["num_neg"] == neg
        assert o.stats["num_zero"] == zero
        if "closed_inertia" in g:
            assert (neg, zero, pos) == g["closed_inertia"]
    if g["flag"] == 7:
        assert o.stats["matrix_rank"] == g["n"] - 1
        return
    x = o.solve(g["rhs"])
    be = w.backward_error(full, x, g["rhs"]).max()
    assert U * be <= 5e-14
    # one FP64 refinement step reaches the 1e-14 target
    x2 = x + o.solve(g["rhs"] - full @ x)
    assert w.backward_error(full, x2, g["rhs"]).max() <= 1e-14
    rel = np.abs(x2 - g["x"]).max() / np.abs(g["x"]).max()
    assert rel <= 1e-10 * max(1.0, 1e-3 / max(g["mineig"], 1e-300))
    if "x_true" in g:
        assert np.abs(x2 - g["x_true"]).max() <= 1e-10


def test_oracle_delays_happen(sylver, orc):
    g = load_golden("dense_indef_delays_96")
    an = analyse(sylver, g)
    o = orc.OracleFactor(False, an.symbolic(), g["val"], u=0.5)
    # a strict threshold forces 2x2 pivots / pivot search on this matrix
    assert o.stats["num_two"] > 0


def test_oracle_partial_jobs(sylver, orc):
    """fwd then bwd equals job 0 (posdef); fwd, diag, bwd equals job 0 (indef)."""
    for name in ("laplace2d_12", "shifted_laplace3d_6"):
        g = load_golden(name)
        an = analyse(sylver, g)
        o = orc.OracleFactor(g["posdef"], an.symbolic(), g["val"], u=U)
        x_all = o.solve(g["rhs"], job=0)
        y = o.solve(g["rhs"], job=1)
        if not g["posdef"]:
            y = o.solve(y, job=2)
        y = o.solve(y, job=3)
        np.testing.assert_allclose(y, x_all, rtol=1e-12, atol=1e-12)


def test_oracle_inertia_closed_form_full_size_small(sylver, orc):
    """Known answer: the 7-point Laplacian on 16^3 minus sigma*I."""
    p = w.shifted_laplace3d(16, nrhs=1)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    o = orc.OracleFactor(False, an.symbolic(), p.a.val, u=U)
    assert o.stats["num_neg"] == p.inertia[0]
    assert o.stats["num_zero"] == 0


def _cause_delays_sparse(k=8, seed=3):
    """The reference's cause_delays idea (tests/common.hxx:753-790) on a
    sparse matrix: n/8 rows/columns scaled by 1000 with small diagonals."""
    rng = np.random.default_rng(seed)
    p = w.shifted_laplace3d(k, nrhs=1)
    full = p.a.to_scipy_full().tolil()
    n = p.a.n
    for idx in rng.choice(n, size=n // 8, replace=False):
        full[idx, :] = full[idx, :] * 1000.0
        full[:, idx] = full[:, idx] * 1000.0
    full = full.tocsr()
    for idx in range(n):
        if abs(full[idx, idx]) > 100:
            full[idx, idx] = full[idx, idx] * 1e-6
    return w.SymMatrix.from_scipy(full), p.order


@pytest.mark.parametrize("case", ["dense_indef_64", "dense_indef_delays_96", "kkt_4",
                                  "shifted_laplace3d_9", "cause_delays", "kkt6"])
@pytest.mark.parametrize("u", [0.01, 0.3])
def test_oracle_app_layout_matches_reference_layout(sylver, orc, case, u):
    """The oracle moves a block's failed columns behind the unprocessed ones
    at once; the reference leaves them in place, reaches them through the
    blocks to their left (ApplyT/UpdateT) and permutes them to the back at
    the end (src/factor_indef.hxx:885-1288).  Both restatements, same
    arithmetic, must give the same factors bit for bit."""
    if case == "cause_delays":
        a, order = _cause_delays_sparse()
    elif case == "kkt6":
        p = w.kkt(6, nrhs=1)
        a = p.a
        order = sylver.Analysis(a.n, a.ptr, a.row).symbolic()["perm"]
    else:
        g = load_golden(case)
        a, order = w.SymMatrix(g["n"], g["ptr"], g["row"], g["val"]), g["order"]
    an = sylver.Analysis(a.n, a.ptr, a.row, order=order)
    sy = an.symbolic()
    o1 = orc.OracleFactor(False, sy, a.val, u=u)
    o2 = orc.OracleFactor(False, sy, a.val, u=u, inplace=True)
    assert o1.stats == o2.stats
    for s in range(sy["nnodes"]):
        f1, f2 = o1.front(s), o2.front(s)
        assert (f1["m"], f1["n"], f1["nelim"]) == (f2["m"], f2["n"], f2["nelim"])
        np.testing.assert_array_equal(f1["var"], f2["var"])
        ne = f1["nelim"]
        assert np.array_equal(f1["d"][:2 * ne], f2["d"][:2 * ne])
        assert np.array_equal(np.tril(f1["a"]), np.tril(f2["a"]))


def test_oracle_app_fails_and_delays(sylver, orc):
    """The block steps leave columns to the threshold partial pivoting pass
    (not_first_pass) and some of those are delayed to parents."""
    a, order = _cause_delays_sparse()
    an = sylver.Analysis(a.n, a.ptr, a.row, order=order)
    o = orc.OracleFactor(False, an.symbolic(), a.val, u=0.01)
    assert o.stats["not_first_pass"] > 0
    assert o.stats["num_delay"] > 0
    full = a.to_scipy_full()
    ev = np.linalg.eigvalsh(full.toarray())
    assert o.stats["num_neg"] == int(np.sum(ev < 0))
    b = np.random.default_rng(5).standard_normal((a.n, 1))
    x = o.solve(b)
    x = x + o.solve(b - full @ x)
    assert w.backward_error(full, x, b).max() <= 1e-14
