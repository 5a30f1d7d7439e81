"""Host symbolic analysis: structure, A->front map, flags (CPU only)."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import golden_names, load_golden
from sylver_gb300 import workloads as w


def dense_fill(full, perm0):
    invp = np.argsort(perm0)
    a = full.toarray()[np.ix_(invp, invp)] != 0
    n = a.shape[0]
    cols = []
    for k in range(n):
        rows = np.nonzero(a[k + 1:, k])[0] + k + 1
        a[np.ix_(rows, rows)] = True
        cols.append(set([k]) | set(rows.tolist()))
    return cols


@pytest.mark.parametrize("name", golden_names())
def test_symbolic_covers_fill(sylver, name):
    g = load_golden(name)
    an = sylver.Analysis(g["n"], g["ptr"], g["row"], order=g["order"])
    assert an.flag >= 0
    sy = an.symbolic()
    full = w.SymMatrix(g["n"], g["ptr"], g["row"], g["val"]).to_scipy_full()
    cols = dense_fill(full, sy["perm"] - 1)
    sptr, rptr, rlist = sy["sptr"], sy["rptr"], sy["rlist"]
    for s in range(sy["nnodes"]):
        rl = rlist[rptr[s] - 1:rptr[s + 1] - 1] - 1
        assert list(rl[: sptr[s + 1] - sptr[s]]) == list(range(sptr[s] - 1, sptr[s + 1] - 1))
        assert np.all(np.diff(rl[sptr[s + 1] - sptr[s]:]) > 0)
        for j in range(sptr[s] - 1, sptr[s + 1] - 1):
            assert cols[j] <= set(rl.tolist())
        p = sy["sparent"][s] - 1
        if p < sy["nnodes"]:
            prl = set((rlist[rptr[p] - 1:rptr[p + 1] - 1] - 1).tolist())
            assert set(rl[sptr[s + 1] - sptr[s]:].tolist()) <= prl


@pytest.mark.parametrize("name", golden_names())
def test_amap_reassembles_A(sylver, name):
    """Scattering val through nlist into the fronts rebuilds P A P^T."""
    g = load_golden(name)
    an = sylver.Analysis(g["n"], g["ptr"], g["row"], order=g["order"])
    sy = an.symbolic()
    n = g["n"]
    perm0 = sy["perm"] - 1
    full = w.SymMatrix(n, g["ptr"], g["row"], g["val"]).to_scipy_full().toarray()
    invp = np.argsort(perm0)
    ap = np.tril(full[np.ix_(invp, invp)])
    rebuilt = np.zeros((n, n))
    for s in range(sy["nnodes"]):
        rl = sy["rlist"][sy["rptr"][s] - 1:sy["rptr"][s + 1] - 1] - 1
        nrow = len(rl)
        c0 = sy["sptr"][s] - 1
        for k in range(sy["nptr"][s] - 1, sy["nptr"][s + 1] - 1):
            src, dest = sy["nlist"][2 * k] - 1, sy["nlist"][2 * k + 1] - 1
            c, r = divmod(dest, nrow)
            rebuilt[rl[r], c0 + c] += g["val"][src]
    np.testing.assert_allclose(rebuilt, ap, rtol=0, atol=0)


def test_counts_match_flops_formula(sylver):
    p = w.laplace2d(30)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    sy = an.symbolic()
    assert an.inform.num_flops == w.factor_flops(sy["sptr"], sy["rptr"])
    assert an.inform.num_sup == sy["nnodes"]
    assert an.inform.maxfront == int(np.diff(sy["rptr"]).max())


def test_fundamental_supernodes_exact_counts(sylver):
    """With nemin=1 only fundamental supernodes merge, so num_factor equals
    the exact nnz(L) of the symbolic factorization."""
    p = w.laplace2d(14)
    opts = sylver.default_options()
    opts.nemin = 1
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order, options=opts)
    sy = an.symbolic()
    cols = dense_fill(p.a.to_scipy_full(), sy["perm"] - 1)
    assert an.inform.num_factor == sum(len(c) for c in cols)


def test_internal_ordering(sylver):
    """ordering=1 runs the library's nested dissection."""
    p = w.lognormal27(8, nrhs=1)
    opts = sylver.default_options()
    opts.ordering = 1
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, options=opts)
    assert an.flag == 0
    sy = an.symbolic()
    assert sorted(sy["perm"].tolist()) == list(range(1, p.a.n + 1))


def test_flags(sylver):
    o = sylver.default_options()
    # n < 0
    assert sylver.Analysis(-1, np.array([1]), np.array([1]), options=o).flag == -2
    # bad ptr
    an = sylver.Analysis(2, np.array([1, 3, 2]), np.array([1, 2]), options=o)
    assert an.flag == -3
    # all out of range
    an = sylver.Analysis(2, np.array([1, 2, 3]), np.array([5, 7]), options=o)
    assert an.flag == -4
    # some out of range -> warning 1
    an = sylver.Analysis(2, np.array([1, 3, 4]), np.array([1, 9, 2]), options=o)
    assert an.flag == 1
    # duplicate -> warning 2; missing diagonal -> 4
    an = sylver.Analysis(2, np.array([1, 4, 5]), np.array([1, 2, 2, 2]), options=o)
    assert an.flag == 2
    an = sylver.Analysis(3, np.array([1, 3, 4, 5]), np.array([1, 2, 2, 3]), options=o)
    assert an.flag == 0
    an = sylver.Analysis(3, np.array([1, 2, 3, 3]), np.array([2, 3]), options=o)
    assert an.flag in (4, 5)
    # user order that is not a permutation
    an = sylver.Analysis(3, np.array([1, 2, 3, 4]), np.array([1, 2, 3]),
                         order=np.array([1, 1, 2]), options=o)
    assert an.flag == -8
    # n = 0 is fine
    assert sylver.Analysis(0, np.array([1]), np.array([], dtype=np.int32), options=o).flag == 0
