"""The internal seam and the scaling contract, against the CPU oracle.

The reference's Fortran factor_core builds the numeric tree through
spldlt_create_numeric_tree[_posdef]_dbl(fkeep, symbolic_tree, aval, scaling,
child_contrib, options, inform) (src/spldlt_factorize_mod.F90:542-550,
src/NumericTree.cxx:27-45, src/NumericTreePosdef.cxx:19-27) and solves with
the tree solves on x in pivot order, applying the scaling around them
(src/spldlt_factorize_mod.F90:945-1050).  These tests drive exactly that
sequence through the C-ABI, with the symbolic arrays of our analysis in
SPRAL's layout, with and without a scaling vector, and compare with the
oracle's solution of the unscaled system.
"""
import numpy as np
import pytest

from sylver_gb300 import workloads as w

pytestmark = pytest.mark.gpu

CASES = [("laplace2d_20", True, lambda: w.laplace2d(20, nrhs=2)),
         ("lognormal27_9", True, lambda: w.lognormal27(9, nrhs=2)),
         ("shifted_laplace3d_8", False, lambda: w.shifted_laplace3d(8, nrhs=2)),
         ("kkt_5", False, lambda: w.kkt(5, nrhs=2))]


def _oracle_solution(orc, posdef, sym, p):
    o = orc.OracleFactor(posdef, sym, p.a.val)
    return o, o.solve(p.rhs)


@pytest.mark.parametrize("name,posdef,make", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("scaled", [False, True])
def test_seam_tree_matches_oracle(sylver, gpu, orc, name, posdef, make, scaled):
    p = make()
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    assert an.flag >= 0
    sym = an.symbolic()
    n = p.a.n
    invp = np.argsort(sym["perm"] - 1)  # invp[k] = variable at pivot position k
    o, xo = _oracle_solution(orc, posdef, sym, p)
    s_piv = None
    if scaled:
        s_user = np.random.default_rng(11).uniform(0.25, 4.0, n)
        s_piv = s_user[invp]
    tree = sylver.SeamTree(sym, posdef, p.a.val, scaling=s_piv)
    try:
        assert tree.tree, tree.inform.as_dict()
        assert tree.inform.flag >= 0, tree.inform.as_dict()
        if not posdef:
            # Sylvester's law: the same inertia whatever the scaling
            assert tree.inform.num_neg == o.stats["num_neg"]
        x = np.asfortranarray(p.rhs[invp])
        if scaled:
            x *= s_piv[:, None]
        assert tree.solve("fwd", x) == 0
        assert tree.solve("bwd" if posdef else "diag_bwd", x) == 0
        if scaled:
            x *= s_piv[:, None]
        xu = np.empty_like(x)
        xu[invp] = x
        scale = np.abs(xo).max()
        assert np.abs(xu - xo).max() <= 1e-10 * scale
        if not posdef:
            # fwd, diag, bwd one by one give what fwd + diag_bwd gave
            y = np.asfortranarray(p.rhs[invp])
            if scaled:
                y *= s_piv[:, None]
            for job in ("fwd", "diag", "bwd"):
                assert tree.solve(job, y) == 0
            if scaled:
                y *= s_piv[:, None]
            yu = np.empty_like(y)
            yu[invp] = y
            assert np.abs(yu - xo).max() <= 1e-10 * scale
    finally:
        tree.close()


@pytest.mark.parametrize("name,posdef,make", CASES, ids=[c[0] for c in CASES])
def test_public_scale_all_jobs(sylver, gpu, orc, name, posdef, make):
    """spldlt_factorize with a user `scale` (options.scaling = 0) factors
    S A S; job 0 solves A x = b, and the partial jobs compose to the same x:
    S enters with job 1 and leaves with jobs 3 / 4."""
    p = make()
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    sym = an.symbolic()
    n = p.a.n
    _, xo = _oracle_solution(orc, posdef, sym, p)
    s_user = np.random.default_rng(12).uniform(0.25, 4.0, n)
    f = sylver.Factor(an, posdef, p.a.val, scale=s_user)
    assert f.flag >= 0, f.inform.as_dict()
    scale = np.abs(xo).max()
    x = f.solve(p.rhs, job=0)
    assert np.abs(x - xo).max() <= 1e-10 * scale
    if posdef:
        y = f.solve(f.solve(p.rhs, job=1), job=3)
    else:
        y = f.solve(f.solve(p.rhs, job=1), job=4)
        z = f.solve(f.solve(f.solve(p.rhs, job=1), job=2), job=3)
        assert np.abs(z - xo).max() <= 1e-10 * scale
    assert np.abs(y - xo).max() <= 1e-10 * scale
    # FP32 factors of S A S with refinement on A reach the backward error
    f32 = sylver.Factor(an, posdef, p.a.val, precision=sylver.FP32, ir_max_iter=10,
                        scale=s_user)
    assert f32.flag >= 0
    x32 = f32.solve(p.rhs)
    assert w.backward_error(p.a.to_scipy_full(), x32, p.rhs).max() <= 1e-14
