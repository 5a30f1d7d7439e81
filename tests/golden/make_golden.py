"""Generate the golden fixtures under tests/golden/ (run from the repo root).

Each fixture is a small sparse symmetric system in the reference's input
layout (1-based lower CSC) with
  * the exact solution of the dense FP64 system (numpy.linalg.solve),
  * the inertia from numpy.linalg.eigvalsh (and, where the matrix has one,
    the closed form: shifted 7-point Laplacian eigenvalues, Haynsworth for
    the KKT matrix),
  * the flag the reference returns for it.
The dense front cases mirror the reference's node tests
(tests/common.hxx:137-255, :753-790: random indefinite fronts, cause_delays
scaling n/8 rows by 1000, make_singular copying a scaled column).  The
random generators here are numpy's, not the reference's rand().
"""
from __future__ import annotations

import os
import sys

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from sylver_gb300 import workloads as w  # noqa: E402


def inertia_eig(full, tol=1e-10):
    ev = np.linalg.eigvalsh(full.toarray())
    scale = max(1.0, np.abs(ev).max())
    neg = int(np.sum(ev < -tol * scale))
    zero = int(np.sum(np.abs(ev) <= tol * scale))
    return (neg, zero, len(ev) - neg - zero), float(np.abs(ev).min())


def dense_indef(n, rng):
    a = rng.uniform(-1, 1, size=(n, n))
    return (a + a.T) / 2


def cause_delays(a, rng):
    n = a.shape[0]
    for _ in range(max(1, n // 8)):
        idx = int(rng.integers(0, n))
        a[idx, :] *= 1000
        a[:, idx] *= 1000
        a[idx, idx] /= 1000  # scaled once per row/col pass, as the lower-triangle loop does
        r, c = int(rng.integers(0, n)), int(rng.integers(0, n))
        a[r, c] *= 1000
        if r != c:
            a[c, r] *= 1000
    return a


def make_singular(a, c1, c2):
    scal = a[c1, c2] / a[c1, c1]
    col = scal * a[:, c1].copy()
    a[:, c2] = col
    a[c2, :] = col
    a[c2, c2] = scal * col[c1]
    return a


def save(name, full, posdef, order=None, rhs=None, closed_inertia=None, flag=0, extra=None,
         rng=None):
    full = sp.csr_matrix(full)
    m = w.SymMatrix.from_scipy(full)
    n = m.n
    rng = rng or np.random.default_rng(123)
    if rhs is None:
        rhs = np.asfortranarray(rng.standard_normal((n, 2)))
    inert, mineig = inertia_eig(full)
    if flag >= 0 and inert[1] == 0:
        x = np.linalg.solve(full.toarray(), rhs)
    else:
        x = np.zeros_like(rhs)
    if order is None:
        order = np.arange(1, n + 1, dtype=np.int32)
    d = dict(n=n, ptr=m.ptr, row=m.row, val=m.val, order=order.astype(np.int32), rhs=rhs,
             x=x, posdef=posdef, inertia=np.array(inert), flag=flag, mineig=mineig)
    if closed_inertia is not None:
        d["closed_inertia"] = np.array(closed_inertia)
    if extra:
        d.update(extra)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print(name, n, m.nnz, inert, "flag", flag)


def main():
    rng = np.random.default_rng(2024)
    p = w.laplace2d(12)
    save("laplace2d_12", p.a.to_scipy_full(), True, p.order, rhs=p.rhs,
         closed_inertia=p.inertia, extra=dict(x_true=p.x_true))
    p = w.laplace2d(20, 13)
    save("laplace2d_20x13", p.a.to_scipy_full(), True, p.order, rhs=p.rhs,
         closed_inertia=p.inertia, extra=dict(x_true=p.x_true))
    p = w.shifted_laplace3d(6, nrhs=2)
    save("shifted_laplace3d_6", p.a.to_scipy_full(), False, p.order, rhs=p.rhs,
         closed_inertia=p.inertia, extra=dict(sigma=p.sigma))
    p = w.shifted_laplace3d(9, nrhs=2)
    save("shifted_laplace3d_9", p.a.to_scipy_full(), False, p.order, rhs=p.rhs,
         closed_inertia=p.inertia, extra=dict(sigma=p.sigma))
    p = w.lognormal27(7, nrhs=2)
    save("lognormal27_7", p.a.to_scipy_full(), True, p.order, rhs=p.rhs,
         closed_inertia=p.inertia)
    p = w.kkt(4, nnz_per_row=3, seed=7, nrhs=2)
    save("kkt_4", p.a.to_scipy_full(), False, None, rhs=p.rhs, closed_inertia=p.inertia)
    # dense fronts (one supernode) as in the reference's factor_node tests
    a = dense_indef(64, rng)
    save("dense_indef_64", a, False)
    a = cause_delays(dense_indef(96, rng), rng)
    save("dense_indef_delays_96", a, False)
    b = rng.uniform(-1, 1, size=(48, 48))
    save("dense_posdef_48", b @ b.T + 48 * np.eye(48), True)
    # exactly singular: an empty row/column gives an exact zero pivot
    # (a column merely proportional to another leaves a round-off pivot above
    # `small`, which neither this library nor the reference flags)
    a = dense_indef(40, rng)
    a[17, :] = 0.0
    a[:, 17] = 0.0
    save("dense_singular_40", a + 0.0, False, flag=7)
    # a symmetric indefinite matrix given to the Cholesky path: -6
    p = w.shifted_laplace3d(5, nrhs=1)
    save("not_posdef_5", p.a.to_scipy_full(), True, p.order, rhs=p.rhs, flag=-6)
    # random sparse SPD with a natural order (internal analysis quality varies)
    r = sp.random(150, 150, density=0.03, random_state=5)
    spd = r @ r.T + sp.identity(150) * 5.0
    save("random_spd_150", spd, True)


if __name__ == "__main__":
    main()
