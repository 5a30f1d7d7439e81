"""Matching-based scaling and ordering (options.ordering = 2) on the host.

The reference gets them from SPRAL's match_order_metis / hungarian_scale_sym
(src/spldlt_analyse_mod.F90:787-816, src/spldlt_factorize_mod.F90:735-760);
here they are restated from the published method (maximum-product matching
with dual variables, Duff & Pralet symmetric scaling, cycles split into 2x2
pairs).  Properties checked against a dense reference computation:
  * |s_i a_ij s_j| <= 1 everywhere and = 1 on a perfect matching, whose
    product of |a_ij| equals the optimum found by scipy's assignment solver;
  * each 2x2 pair of the matching gets consecutive pivot positions;
  * option errors: ordering outside 0..2 -> -8, ordering 2 without values -> -9.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp
from scipy.optimize import linear_sum_assignment

from sylver_gb300 import workloads as w


def _analyse(sylver, a, ordering=2, with_val=True):
    o = sylver.default_options()
    o.ordering = ordering
    return sylver.Analysis(a.n, a.ptr, a.row, options=o, val=a.val if with_val else None)


def _dense(a):
    return a.to_scipy_full().toarray()


@pytest.mark.parametrize("make", [lambda: w.kkt(4, nrhs=1).a,
                                  lambda: w.shifted_laplace3d(6, nrhs=1).a,
                                  lambda: w.laplace2d(9, nrhs=1).a])
def test_matching_scaling_properties(sylver, make):
    a = make()
    an = _analyse(sylver, a)
    assert an.flag >= 0
    s = an.scaling()
    assert s is not None and np.all(s > 0)
    A = _dense(a)
    S = np.abs(s[:, None] * A * s[None, :])
    assert S.max() <= 1 + 1e-12
    # an optimal maximum-product matching exists among the entries equal to 1
    cost = np.where(A != 0, -np.log(np.abs(A) + (A == 0)), 1e30)
    r, c = linear_sum_assignment(cost)
    best = -cost[r, c].sum()
    ones = np.isclose(S, 1.0, rtol=1e-10) & (A != 0)
    r1, c1 = linear_sum_assignment(np.where(ones, 0.0, 1.0))
    assert np.all(ones[r1, c1])
    ours = np.log(np.abs(A[r1, c1])).sum()
    assert abs(ours - best) <= 1e-8 * max(1.0, abs(best))


def test_matching_order_keeps_pairs_adjacent(sylver):
    """KKT matrix: B rows have a tiny diagonal, so the matching pairs them
    with H variables; every such pair sits in consecutive pivot positions."""
    p = w.kkt(5, nrhs=1)
    a = p.a
    an = _analyse(sylver, a)
    s = an.scaling()
    A = _dense(a)
    S = np.abs(s[:, None] * A * s[None, :])
    pos = an.symbolic()["perm"] - 1  # variable -> pivot position
    nh = p.nh
    # rows of B: diagonal -1e-8 is never a unit entry after scaling
    paired = 0
    for b in range(nh, a.n):
        partners = [j for j in np.nonzero(np.isclose(S[b], 1.0, rtol=1e-10))[0] if j != b]
        assert partners, b
        if any(abs(pos[b] - pos[j]) == 1 for j in partners):
            paired += 1
    assert paired >= 0.9 * (a.n - nh)


def test_ordering_option_errors(sylver):
    a = w.laplace2d(5, nrhs=1).a
    assert _analyse(sylver, a, ordering=3).flag == -8
    assert _analyse(sylver, a, ordering=2, with_val=False).flag == -9
