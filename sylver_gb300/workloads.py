"""Synthetic sparse symmetric matrices and orderings for the factor/solve path.

Every generator returns the lower triangle in the reference's input format
(``spldlt_analyse``/``spldlt_factorize`` in include/sylver/sylver.h:73-92):
compressed sparse column, 1-based, ``ptr`` int64 of length n+1 and ``row``
int32, values float64.  Orderings follow SPRAL's convention for ``order``:
``order[i]`` is the 1-based pivot position of variable ``i``.

Workloads (seeded, no external data):
  * 2D 5-point Laplacian, Dirichlet boundary (SPD).
  * 3D 7-point Laplacian minus sigma*I with sigma between two distinct
    eigenvalues near a spectrum quantile (indefinite, closed-form inertia).
  * 3D 27-point weighted Laplacian with log-normal edge weights, Dirichlet
    ghost edges of weight 1 and a small diagonal shift (SPD).
  * batches of small 2D Laplacians with random shifts (SPD).
  * saddle-point KKT [[H, B^T], [B, -delta I]] (indefinite, Haynsworth
    inertia).
"""
from __future__ import annotations

import dataclasses
import numpy as np
import scipy.sparse as sp


@dataclasses.dataclass
class SymMatrix:
    """Lower triangle of a symmetric matrix in 1-based CSC form."""
    n: int
    ptr: np.ndarray   # int64, n+1, 1-based
    row: np.ndarray   # int32, nnz, 1-based
    val: np.ndarray   # float64, nnz

    @classmethod
    def from_scipy(cls, a: sp.spmatrix) -> "SymMatrix":
        low = sp.tril(sp.csc_matrix(a), format="csc")
        low.sort_indices()
        low.sum_duplicates()
        return cls(n=low.shape[0],
                   ptr=(low.indptr.astype(np.int64) + 1),
                   row=(low.indices.astype(np.int32) + 1),
                   val=low.data.astype(np.float64))

    def to_scipy_full(self) -> sp.csr_matrix:
        """Full symmetric matrix (both triangles) as scipy CSR (0-based)."""
        low = sp.csc_matrix((self.val, self.row - 1, self.ptr - 1),
                            shape=(self.n, self.n))
        full = low + sp.tril(low, -1).T
        return sp.csr_matrix(full)

    @property
    def nnz(self) -> int:
        return int(self.ptr[-1] - 1)


# ---------------------------------------------------------------------------
# grid helpers

def _grid_index(dims):
    return np.arange(int(np.prod(dims))).reshape(dims, order="F")


def _stencil_offsets(ndim: int, kind: str):
    if kind == "star":
        offs = []
        for d in range(ndim):
            e = [0] * ndim
            e[d] = 1
            offs.append(tuple(e))
        return offs
    # box stencil: all offsets in {-1,0,1}^ndim that are lexicographically positive
    offs = []
    for o in np.ndindex(*([3] * ndim)):
        o = tuple(int(v) - 1 for v in o)
        if all(v == 0 for v in o):
            continue
        # keep one of each +-pair
        first = next(v for v in o if v != 0)
        if first > 0:
            offs.append(o)
    return offs


def _grid_edges(dims, kind):
    """Undirected edges (i<j) of a grid graph, sorted lexicographically."""
    idx = _grid_index(dims)
    ndim = len(dims)
    ii, jj = [], []
    for o in _stencil_offsets(ndim, kind):
        src = [slice(max(0, -v), dims[d] - max(0, v)) for d, v in enumerate(o)]
        dst = [slice(s.start + v, s.stop + v) for s, v in zip(src, o)]
        a = idx[tuple(src)].ravel(order="F")
        b = idx[tuple(dst)].ravel(order="F")
        ii.append(np.minimum(a, b))
        jj.append(np.maximum(a, b))
    ii = np.concatenate(ii)
    jj = np.concatenate(jj)
    order = np.lexsort((jj, ii))
    return ii[order], jj[order]


def _nbr_count_full(ndim, kind):
    return 2 * ndim if kind == "star" else 3 ** ndim - 1


def grid_laplacian(dims, kind="star", weights=None, ghost_weight=1.0):
    """Weighted graph Laplacian of a grid with Dirichlet ghost neighbours.

    Diagonal = sum of incident edge weights + ghost_weight per missing
    neighbour (so the unweighted star stencil gives 4 / 6 on the diagonal).
    Returns (scipy CSR full matrix, edges i, edges j, weights)."""
    dims = tuple(int(d) for d in dims)
    n = int(np.prod(dims))
    ii, jj = _grid_edges(dims, kind)
    w = np.ones(ii.shape[0]) if weights is None else np.asarray(weights, dtype=np.float64)
    deg = np.zeros(n)
    np.add.at(deg, ii, w)
    np.add.at(deg, jj, w)
    cnt = np.zeros(n, dtype=np.int64)
    np.add.at(cnt, ii, 1)
    np.add.at(cnt, jj, 1)
    missing = _nbr_count_full(len(dims), kind) - cnt
    diag = deg + ghost_weight * missing
    a = sp.coo_matrix((np.concatenate([-w, -w, diag]),
                       (np.concatenate([ii, jj, np.arange(n)]),
                        np.concatenate([jj, ii, np.arange(n)]))), shape=(n, n))
    return sp.csr_matrix(a), ii, jj, w


# ---------------------------------------------------------------------------
# orderings

def grid_nested_dissection(dims, leaf=2):
    """Geometric nested dissection of a box grid (stand-in for METIS ND).

    Recursively splits the longest axis by a one-plane separator (valid for
    both the star and box stencils), numbering part 1, part 2, then the
    separator.  Returns ``order`` (1-based pivot position per variable)."""
    dims = tuple(int(d) for d in dims)
    idx = _grid_index(dims)
    seq = []

    def rec(lo, hi):
        ext = [h - l for l, h in zip(lo, hi)]
        if min(ext) <= 0:
            return
        if int(np.prod(ext)) <= leaf ** len(dims) or max(ext) <= 2:
            sl = tuple(slice(l, h) for l, h in zip(lo, hi))
            seq.append(idx[sl].ravel(order="F"))
            return
        d = int(np.argmax(ext))
        mid = lo[d] + ext[d] // 2
        hi1 = list(hi); hi1[d] = mid
        lo2 = list(lo); lo2[d] = mid + 1
        rec(list(lo), hi1)
        rec(lo2, list(hi))
        los = list(lo); his = list(hi)
        los[d] = mid; his[d] = mid + 1
        sl = tuple(slice(l, h) for l, h in zip(los, his))
        seq.append(idx[sl].ravel(order="F"))

    rec([0] * len(dims), list(dims))
    piv = np.concatenate(seq)
    n = int(np.prod(dims))
    assert piv.shape[0] == n
    order = np.empty(n, dtype=np.int32)
    order[piv] = np.arange(1, n + 1, dtype=np.int32)
    return order


def natural_order(n):
    return np.arange(1, n + 1, dtype=np.int32)


# ---------------------------------------------------------------------------
# the five workloads

@dataclasses.dataclass
class Problem:
    name: str
    a: SymMatrix
    order: np.ndarray           # 1-based pivot positions
    posdef: bool
    rhs: np.ndarray             # n x nrhs, Fortran order
    x_true: np.ndarray | None = None
    inertia: tuple | None = None  # (num_neg, num_zero, num_pos) when known


def laplace2d(nx=100, ny=None, seed=0, nrhs=1):
    """2D 5-point Laplacian, Dirichlet; b = A x_true, x_true ~ U(-1,1)."""
    ny = nx if ny is None else ny
    full, *_ = grid_laplacian((nx, ny), "star")
    a = SymMatrix.from_scipy(full)
    rng = np.random.default_rng(seed)
    x = np.asfortranarray(rng.uniform(-1.0, 1.0, size=(a.n, nrhs)))
    b = np.asfortranarray(full @ x)
    return Problem(f"laplace2d_{nx}x{ny}", a, grid_nested_dissection((nx, ny)),
                   True, b, x_true=x, inertia=(0, 0, a.n))


def laplace1d_eigs(k):
    return 2.0 - 2.0 * np.cos(np.arange(1, k + 1) * np.pi / (k + 1))


def shifted_laplace3d(k=48, quantile=0.05, seed=1, nrhs=4):
    """3D 7-point Laplacian on k^3 minus sigma*I; sigma is the midpoint of
    the nearest pair of distinct adjacent eigenvalues around the quantile
    index.  The inertia is known in closed form."""
    e1 = laplace1d_eigs(k)
    lam = (e1[:, None, None] + e1[None, :, None] + e1[None, None, :]).ravel()
    lam.sort()
    q = int(quantile * lam.size)
    uniq = np.unique(np.round(lam, 12))
    pos = np.searchsorted(uniq, lam[q])
    lo = uniq[max(pos - 1, 0)] if uniq[min(pos, uniq.size - 1)] > lam[q] else uniq[pos]
    hi = uniq[np.searchsorted(uniq, lo, side="right")]
    sigma = 0.5 * (lo + hi)
    num_neg = int(np.sum(lam < sigma))
    full, *_ = grid_laplacian((k, k, k), "star")
    full = sp.csr_matrix(full - sigma * sp.identity(full.shape[0]))
    a = SymMatrix.from_scipy(full)
    rng = np.random.default_rng(seed)
    b = np.asfortranarray(rng.standard_normal((a.n, nrhs)))
    p = Problem(f"shifted_laplace3d_{k}", a, grid_nested_dissection((k, k, k)),
                False, b, inertia=(num_neg, 0, a.n - num_neg))
    p.sigma = sigma
    return p


def lognormal27(k=80, seed=2, rhs_seed=3, nrhs=16, shift_frac=1e-3):
    """3D 27-point weighted Laplacian on k^3; weights exp(N(0,1)) per edge
    (edges in lexicographic (i,j) order), Dirichlet ghost edges weight 1,
    plus shift_frac * min(diag) on the diagonal (SPD)."""
    dims = (k, k, k)
    ii, jj = _grid_edges(dims, "box")
    rng = np.random.default_rng(seed)
    w = np.exp(rng.standard_normal(ii.shape[0]))
    full, *_ = grid_laplacian(dims, "box", weights=w)
    d = full.diagonal()
    full = sp.csr_matrix(full + shift_frac * d.min() * sp.identity(full.shape[0]))
    a = SymMatrix.from_scipy(full)
    rng2 = np.random.default_rng(rhs_seed)
    b = np.asfortranarray(rng2.standard_normal((a.n, nrhs)))
    return Problem(f"lognormal27_{k}", a, grid_nested_dissection(dims), True, b,
                   inertia=(0, 0, a.n))


def batched_laplace2d(count=2000, smin=8, smax=64, seed=4):
    """Independent SPD instances: s x s 5-point Laplacians, s ~ U{smin..smax},
    diagonal shift ~ U(0.1, 1), one N(0,1) right-hand side each."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        s = int(rng.integers(smin, smax + 1))
        shift = float(rng.uniform(0.1, 1.0))
        full, *_ = grid_laplacian((s, s), "star")
        full = sp.csr_matrix(full + shift * sp.identity(full.shape[0]))
        a = SymMatrix.from_scipy(full)
        b = np.asfortranarray(rng.standard_normal((a.n, 1)))
        out.append(Problem(f"batch{i}_s{s}", a, grid_nested_dissection((s, s)),
                           True, b, inertia=(0, 0, a.n)))
    return out


def kkt(k=40, brows=None, nnz_per_row=4, delta=1e-8, seed=5, nrhs=1):
    """Saddle point [[H, B^T], [B, -delta I]]; H = 7-point Laplacian on k^3,
    B random with nnz_per_row distinct columns per row, values N(0,1).
    Inertia by Haynsworth: (brows negative, 0 zero, n_H positive) when B has
    full row rank."""
    nh = k ** 3
    brows = nh // 4 if brows is None else brows
    rng = np.random.default_rng(seed)
    h, *_ = grid_laplacian((k, k, k), "star")
    cols = np.empty((brows, nnz_per_row), dtype=np.int64)
    for r in range(brows):
        cols[r] = rng.choice(nh, size=nnz_per_row, replace=False)
    vals = rng.standard_normal((brows, nnz_per_row))
    b = sp.csr_matrix((vals.ravel(), (np.repeat(np.arange(brows), nnz_per_row),
                                      cols.ravel())), shape=(brows, nh))
    full = sp.bmat([[h, b.T], [b, -delta * sp.identity(brows)]], format="csr")
    a = SymMatrix.from_scipy(full)
    rhs = np.asfortranarray(rng.standard_normal((a.n, nrhs)))
    p = Problem(f"kkt_{k}_{brows}", a, natural_order(a.n), False, rhs,
                inertia=(brows, 0, nh))
    p.grid_dims = (k, k, k)
    p.nh = nh
    return p


# ---------------------------------------------------------------------------
# measurement helpers (host side)

def factor_flops(sptr, rptr):
    """Factor flop count of the reference's compute_flops
    (src/spldlt_analyse_mod.F90:1744-1764): sum over fronts of sum_{j=m-n+1}^{m} j^2."""
    sptr = np.asarray(sptr, dtype=np.int64)
    rptr = np.asarray(rptr, dtype=np.int64)
    n = np.diff(sptr)
    m = np.diff(rptr)
    def s2(k):
        return k * (k + 1) * (2 * k + 1) // 6
    return int(np.sum(s2(m) - s2(m - n)))


def backward_error(full: sp.spmatrix, x: np.ndarray, b: np.ndarray):
    """Per-RHS scaled backward error max_i|b-Ax|_i / (||A||inf ||x||inf + ||b||inf)
    (tests/common.hxx:1003-1050; drivers/spldlt_test.F90:216-267)."""
    x = x.reshape(b.shape)
    r = b - full @ x
    anorm = abs(full).sum(axis=1).max()
    out = []
    for j in range(b.shape[1]):
        den = anorm * np.abs(x[:, j]).max() + np.abs(b[:, j]).max()
        out.append(np.abs(r[:, j]).max() / den if den > 0 else 0.0)
    return np.array(out)


def block_diagonal(problems):
    """Stack independent instances into one block-diagonal system (their
    assembly trees form a forest, so one analysis / factorization / solve
    processes every instance level by level in shared launches).  Returns
    (Problem, offsets) with offsets[k] the first row of instance k."""
    ptrs, rows, vals, orders, rhs = [], [], [], [], []
    offs = [0]
    nz = 0
    for p in problems:
        n0 = offs[-1]
        a = p.a
        ptrs.append(a.ptr[:-1] - 1 + nz)
        rows.append(a.row + n0)
        vals.append(a.val)
        orders.append(p.order + n0)
        rhs.append(p.rhs[:, 0])
        nz += a.nnz
        offs.append(n0 + a.n)
    n = offs[-1]
    ptr = np.concatenate(ptrs + [np.array([nz], dtype=np.int64)]) + 1
    big = SymMatrix(n, ptr.astype(np.int64), np.concatenate(rows).astype(np.int32),
                    np.concatenate(vals))
    b = np.asfortranarray(np.concatenate(rhs).reshape(-1, 1))
    inert = (0, 0, n) if all(p.posdef for p in problems) else None
    return Problem(f"batch{len(problems)}", big, np.concatenate(orders).astype(np.int32),
                   all(p.posdef for p in problems), b, inertia=inert), np.array(offs)


def instance_backward_errors(problems, offs, x):
    """Scaled backward error of each instance of a block-diagonal solve."""
    out = []
    for k, p in enumerate(problems):
        xs = x[offs[k]:offs[k + 1]]
        out.append(backward_error(p.a.to_scipy_full(), xs, p.rhs).max())
    return np.array(out)
