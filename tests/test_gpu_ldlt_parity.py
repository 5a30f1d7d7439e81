"""FP64 LDL^T on the GPU against the oracle's restatement of the reference's
a-posteriori pivoting, pivot by pivot.

The oracle (oracle/oracle.cpp) restates the reference's indefinite path --
block-column APP with block size 32 (src/factor_indef.hxx:1338-1474,
src/kernels/ldlt_app.hxx:145-751, include/sylver/kernels/Column.hxx:41-125),
permute_failed (src/factor_indef.hxx:1190-1288), the failed-pivot TPP pass
and delays (src/factor_failed.hxx:29-157) -- with every multiply-add in a
fixed order that the GPU kernels repeat.  So on the same matrix the FP64
factorizations must agree exactly, not to a tolerance:
  * num_neg, num_zero, num_two, num_delay, not_first_pass, not_second_pass;
  * per front: rows, fully-summed columns (delays in) and columns eliminated;
  * the pivot order and every D^-1 entry, bit for bit.
The tree-level seam (spldlt_create_numeric_tree_dbl) is used because its
inform_c carries the pass counters; it runs the same factorization as
spldlt_factorize.  Solutions are compared to 1e-10 (the solves' own
summation orders differ)."""
import numpy as np
import pytest

from conftest import load_golden
from sylver_gb300 import workloads as w

pytestmark = pytest.mark.gpu

STATS = ("num_neg", "num_zero", "num_two", "num_delay", "not_first_pass", "not_second_pass")


def _oracle_fronts(o, nnodes):
    ms, ns, nes, ds, vs = [], [], [], [], []
    for s in range(nnodes):
        fr = o.front(s)
        ms.append(fr["m"]); ns.append(fr["n"]); nes.append(fr["nelim"])
        ds.append(fr["d"][:2 * fr["nelim"]])
        vs.append(fr["var"][:fr["nelim"]] + 1)
    return (np.array(ms), np.array(ns), np.array(nes),
            np.concatenate(ds) if ds else np.zeros(0), np.concatenate(vs) if vs else np.zeros(0))


def _gpu_fronts(sylver, tree, n, nnodes):
    import ctypes
    lib = sylver.load()
    P = ctypes.c_void_p
    m = np.zeros(nnodes, np.int32); nn = np.zeros_like(m); ne = np.zeros_like(m)
    assert lib.sylver_gb300_fkeep_fronts(tree, m.ctypes.data_as(P), nn.ctypes.data_as(P),
                                         ne.ctypes.data_as(P)) == nnodes
    d = np.zeros(2 * max(n, 1)); piv = np.zeros(max(n, 1), np.int32)
    k = lib.sylver_gb300_fkeep_diag(tree, d.ctypes.data_as(P), piv.ctypes.data_as(P))
    return m, nn, ne, d[:2 * k], piv[:k]


def check_exact(sylver, orc, a, order, u=0.01, rhs=None, oracle_stats=None):
    """Factor `a` (SymMatrix) on the GPU seam and with the oracle; assert the
    exact agreement above; return (seam tree, oracle factor, analysis)."""
    an = sylver.Analysis(a.n, a.ptr, a.row, order=order)
    assert an.flag >= 0
    sym = an.symbolic()
    o = orc.OracleFactor(False, sym, a.val, u=u)
    tree = sylver.SeamTree(sym, False, a.val, u=u)
    assert tree.tree, tree.inform.as_dict()
    gi = tree.inform.as_dict()
    for k in STATS:
        assert gi[k] == o.stats[k], (k, gi[k], o.stats[k], gi, o.stats)
    assert gi["flag"] == o.flag
    om, on, one, od, ov = _oracle_fronts(o, sym["nnodes"])
    gm, gn, gne, gd, gv = _gpu_fronts(sylver, tree.tree, a.n, sym["nnodes"])
    np.testing.assert_array_equal(gm, om)
    np.testing.assert_array_equal(gn, on)
    np.testing.assert_array_equal(gne, one)
    np.testing.assert_array_equal(gv, ov)
    assert np.array_equal(gd, od), np.abs(gd - od)[np.isfinite(od)].max()
    if rhs is not None:
        invp = np.argsort(sym["perm"] - 1)
        x = np.asfortranarray(rhs[invp])
        assert tree.solve("fwd", x) == 0 and tree.solve("diag_bwd", x) == 0
        xu = np.empty_like(x)
        xu[invp] = x
        xo = o.solve(rhs)
        assert np.abs(xu - xo).max() <= 1e-10 * np.abs(xo).max()
    return tree, o, an


@pytest.mark.parametrize("name,u", [("dense_indef_64", 0.01), ("dense_indef_delays_96", 0.01),
                                    ("dense_indef_delays_96", 0.1),
                                    ("dense_indef_delays_96", 0.5), ("dense_singular_40", 0.01),
                                    ("kkt_4", 0.01), ("shifted_laplace3d_6", 0.01),
                                    ("shifted_laplace3d_9", 0.01)])
def test_golden_exact(sylver, orc, gpu, name, u):
    g = load_golden(name)
    a = w.SymMatrix(g["n"], g["ptr"], g["row"], g["val"])
    tree, o, _ = check_exact(sylver, orc, a, g["order"], u=u,
                             rhs=None if g["flag"] == 7 else g["rhs"])
    tree.close()


@pytest.mark.parametrize("k", [12, 20])
def test_shifted_laplacian_exact(sylver, orc, gpu, k):
    p = w.shifted_laplace3d(k, nrhs=2)
    tree, o, _ = check_exact(sylver, orc, p.a, p.order, rhs=p.rhs)
    assert tree.inform.num_neg == p.inertia[0]
    tree.close()


@pytest.mark.parametrize("k", [6, 10])
def test_kkt_exact(sylver, orc, gpu, k):
    """delta = 1e-8 on the (2,2) block: the B rows fail the threshold test
    in their own fronts and are delayed."""
    p = w.kkt(k, nrhs=1)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row)  # library nested dissection
    order = an.symbolic()["perm"]
    tree, o, _ = check_exact(sylver, orc, p.a, order, rhs=p.rhs)
    assert tree.inform.num_neg == p.inertia[0]
    assert o.stats["not_first_pass"] > 0
    tree.close()


def _cause_delays(k=10, seed=3):
    """The reference's cause_delays (tests/common.hxx:753-790) on a sparse
    matrix: n/8 rows and columns scaled by 1000 with their diagonal kept
    small, so those pivots fail the threshold test where they first appear."""
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
    return w.SymMatrix.from_scipy(full), p.order, full


def test_delays_reach_parent_exact(sylver, orc, gpu):
    """Columns a child cannot eliminate are delayed into its parent, which
    eliminates them (same fronts, same pivots as the oracle)."""
    a, order, full = _cause_delays()
    rhs = np.asfortranarray(np.random.default_rng(4).standard_normal((a.n, 1)))
    tree, o, an = check_exact(sylver, orc, a, order, rhs=rhs)
    sym = an.symbolic()
    sptr = sym["sptr"]
    sparent = sym["sparent"] - 1
    gm, gn, gne, gd, gv = _gpu_fronts(sylver, tree.tree, a.n, sym["nnodes"])
    own = np.diff(sptr)
    assert tree.inform.num_delay > 0
    # a front whose fully-summed set grew by its children's delays and that
    # eliminated some of the delayed variables itself
    offs = np.concatenate([[0], np.cumsum(gne)])
    hit = False
    for s in range(sym["nnodes"]):
        if gn[s] <= own[s]:
            continue
        mine = set(range(sptr[s], sptr[s + 1]))  # own variables (1-based pivot positions)
        piv = set(gv[offs[s]:offs[s + 1]].tolist())
        below = set()
        for c in np.nonzero(sparent == s)[0]:
            below |= set(range(1, sptr[c + 1]))  # everything eliminable under s
        if (piv - mine) and (piv - mine) <= below:
            hit = True
            break
    assert hit
    ev = np.linalg.eigvalsh(full.toarray())
    assert tree.inform.num_neg == int(np.sum(ev < 0))
    tree.close()


def test_config2_shifted_laplacian_48(sylver, orc, gpu):
    """3D 7-point Laplacian on 48^3 minus sigma*I (n = 110,592), u = 0.01,
    4 right-hand sides from seed 1: exact agreement with the oracle, the
    closed-form inertia 5526 / 0 / 105066, and for FP64 and FP32 factors a
    scaled backward error <= 1e-14 after refinement with the solution
    within 1e-10 of the oracle's."""
    p = w.shifted_laplace3d(48, nrhs=4)
    assert p.inertia == (5526, 0, 105066)
    tree, o, an = check_exact(sylver, orc, p.a, p.order)
    assert tree.inform.num_neg == 5526 and tree.inform.num_zero == 0
    tree.close()
    full = p.a.to_scipy_full()
    xo = o.solve(p.rhs)
    xo = xo + o.solve(p.rhs - full @ xo)
    for prec in (sylver.FP64, sylver.FP32):
        f = sylver.Factor(an, False, p.a.val, precision=prec, ir_max_iter=10)
        assert f.flag == 0
        assert (f.inform.num_neg, f.inform.matrix_rank) == (5526, p.a.n)
        x = f.solve(p.rhs)
        assert w.backward_error(full, x, p.rhs).max() <= 1e-14
        assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()


def test_config5_kkt_largest_oracle_case(sylver, orc, gpu):
    """Saddle point [[H, B^T], [B, -1e-8 I]] with H the 7-point Laplacian on
    20^3 (n = 10,000; the 40^3 case is beyond the oracle): exact agreement,
    Haynsworth inertia, refined FP32 and FP64 solves to 1e-14."""
    p = w.kkt(20, nrhs=1)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row)
    order = an.symbolic()["perm"]
    tree, o, an = check_exact(sylver, orc, p.a, order)
    assert tree.inform.num_neg == p.inertia[0]
    tree.close()
    full = p.a.to_scipy_full()
    xo = o.solve(p.rhs)
    xo = xo + o.solve(p.rhs - full @ xo)
    for prec in (sylver.FP64, sylver.FP32):
        f = sylver.Factor(an, False, p.a.val, precision=prec, ir_max_iter=10)
        assert f.flag == 0
        assert f.inform.num_neg == p.inertia[0]
        x = f.solve(p.rhs)
        assert w.backward_error(full, x, p.rhs).max() <= 1e-14
        assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()


@pytest.mark.parametrize("precision", [0, 1])
def test_config1_laplace2d_100(sylver, orc, gpu, precision):
    """2D 5-point Laplacian on 100^2 (n = 10,000), x_true ~ U(-1,1) from
    seed 0, b = A x_true: forward error against x_true and the oracle."""
    p = w.laplace2d(100, nrhs=1)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    f = sylver.Factor(an, True, p.a.val, precision=precision, ir_max_iter=10)
    assert f.flag == 0
    x = f.solve(p.rhs)
    full = p.a.to_scipy_full()
    assert w.backward_error(full, x, p.rhs).max() <= 1e-14
    o = orc.OracleFactor(True, an.symbolic(), p.a.val)
    xo = o.solve(p.rhs)
    assert np.abs(x - xo).max() <= 1e-10 * np.abs(xo).max()
    assert np.abs(x - p.x_true.reshape(x.shape)).max() <= 1e-10


@pytest.mark.parametrize("name", ["dense_indef_delays_96", "kkt_4", "shifted_laplace3d_9"])
def test_factor_copyout_exact(sylver, orc, gpu, name):
    """The compact factor store (schedule front_memory = 1: each level's
    factor columns copied out of the front blocks, whole blocks given back
    after the parents' assembly, the mode large-contribution-block matrices
    take automatically) changes where L lives, not the arithmetic: the same
    exact agreement with the oracle, and the same solutions (to rounding)."""
    g = load_golden(name)
    a = w.SymMatrix(g["n"], g["ptr"], g["row"], g["val"])
    try:
        sylver.set_schedule(front_memory=1)
        tree, o, _ = check_exact(sylver, orc, a, g["order"],
                                 rhs=None if g["flag"] == 7 else g["rhs"])
        tree.close()
    finally:
        sylver.set_schedule()
    p = w.shifted_laplace3d(12, nrhs=2)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    ref = sylver.Factor(an, False, p.a.val).solve(p.rhs)
    try:
        sylver.set_schedule(front_memory=1)
        for prec in (sylver.FP64, sylver.FP32):
            f = sylver.Factor(an, False, p.a.val, precision=prec, ir_max_iter=10)
            x = f.solve(p.rhs)
            if prec == sylver.FP64:  # (the solves' atomic sums are not order-fixed)
                assert np.abs(x - ref).max() <= 1e-12 * np.abs(ref).max()
            assert w.backward_error(p.a.to_scipy_full(), x, p.rhs).max() <= 1e-14
    finally:
        sylver.set_schedule()


def test_config5_kkt_full_size(sylver, gpu):
    """Saddle point [[H, B^T], [B, -1e-8 I]] with H the 7-point Laplacian on
    40^3 (n = 80,000) under the matching-based ordering with its scaling:
    a ~1,000-deep chain of fronts with up to 35,061 rows and 30-50 pivots
    each, whose blocks would need 6.5 TB in place -- the factor columns go to
    the compact store and whole blocks are given back.  FP64 and FP32 with
    refinement: Haynsworth inertia, backward error <= 1e-14."""
    p = w.kkt(40, nrhs=1)
    o = sylver.default_options()
    o.ordering = 2
    o.scaling = 3
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, options=o, val=p.a.val)
    assert an.flag >= 0 and an.inform.maxfront > 30000
    full = p.a.to_scipy_full()
    xs = {}
    for prec in (sylver.FP32, sylver.FP64):
        f = sylver.Factor(an, False, p.a.val, precision=prec, ir_max_iter=10, options=o)
        assert f.flag == 0, f.inform.as_dict()
        assert f.inform.num_neg == p.inertia[0]
        assert f.inform.matrix_rank == p.a.n
        xs[prec] = f.solve(p.rhs)
        assert w.backward_error(full, xs[prec], p.rhs).max() <= 1e-14
