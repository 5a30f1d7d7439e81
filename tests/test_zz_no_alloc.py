"""The allocation-free forward tree solve against the allocating one.

spldlt_tree_solve_fwd_noalloc_dbl exists for callers that cannot let the
library call cudaMalloc (an application-owned memory pool, or code that must
not risk cudaMalloc's device-wide synchronisation).  It must give the same
answer as spldlt_tree_solve_fwd_dbl, the allocating entry point, on the same
factorization -- here twice in a row, so the second call also shows that
what the shared static scratch kept from the first call does not leak in.
This file is collected last so that a stop-at-first-failure run has already
run every other test."""
import ctypes

import numpy as np
import pytest

from sylver_gb300 import workloads as w

pytestmark = pytest.mark.gpu


def _rhs(n, nrhs, seed):
    return np.asfortranarray(np.random.default_rng(seed).standard_normal((n, nrhs)))


@pytest.mark.parametrize("posdef", [True, False])
def test_noalloc_forward_solve_matches(sylver, gpu, posdef):
    import torch
    lib = sylver.load()
    p = w.lognormal27(14, nrhs=1) if posdef else w.shifted_laplace3d(12, nrhs=1)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    f = sylver.Factor(an, posdef, p.a.val)
    assert f.flag == 0
    n = p.a.n
    P = ctypes.c_void_p
    # 40 right-hand sides run as two chunks (32 + 8): the second chunk reuses
    # the scratch slabs the first one left behind
    for call, nrhs in enumerate((3, 5, 40)):
        b = _rhs(n, nrhs, 100 + call)
        ldx = n + 7
        # existing entry point: host memory, allocates its own device buffers
        x_ref = np.zeros((ldx, nrhs), order="F")
        x_ref[:n] = b
        rc = lib.spldlt_tree_solve_fwd_dbl(posdef, f.fkeep, nrhs, x_ref.ctypes.data_as(P), ldx)
        assert rc == 0
        # allocation-free entry point: device memory supplied by the caller
        x_dev = torch.zeros((nrhs, ldx), dtype=torch.float64, device="cuda")
        x_dev[:, :n] = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
        torch.cuda.synchronize()
        rc = lib.spldlt_tree_solve_fwd_noalloc_dbl(posdef, f.fkeep, nrhs, P(x_dev.data_ptr()),
                                                   ldx, None)
        assert rc == 0
        x_na = x_dev.cpu().numpy().T
        scale = np.abs(x_ref[:n]).max()
        assert np.abs(x_na[:n] - x_ref[:n]).max() <= 1e-12 * scale
        # rows past n are untouched
        assert np.all(x_na[n:] == 0.0)


def test_noalloc_rejects_bad_sizes(sylver, gpu):
    import torch
    lib = sylver.load()
    p = w.laplace2d(10, nrhs=1)
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    f = sylver.Factor(an, True, p.a.val)
    x = torch.zeros(p.a.n, dtype=torch.float64, device="cuda")
    P = ctypes.c_void_p
    assert lib.spldlt_tree_solve_fwd_noalloc_dbl(True, f.fkeep, 1, P(x.data_ptr()), p.a.n - 1,
                                                 None) == -10
    assert lib.spldlt_tree_solve_fwd_noalloc_dbl(True, f.fkeep, 0, P(x.data_ptr()), p.a.n,
                                                 None) == -10
    # FP32 factors are not served by this entry point
    f32 = sylver.Factor(an, True, p.a.val, precision=sylver.FP32)
    assert lib.spldlt_tree_solve_fwd_noalloc_dbl(True, f32.fkeep, 1, P(x.data_ptr()), p.a.n,
                                                 None) == -98


def test_noalloc_rejects_level_beyond_scratch(sylver, gpu):
    """A level whose slabs (sum of its front rows x min(nrhs, 32) doubles)
    exceed the 2,097,152-double static array is refused before any launch,
    and x is left as it was."""
    import torch
    lib = sylver.load()
    p = w.laplace2d(400, nrhs=1)  # widest level about 175,000 rows
    an = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
    f = sylver.Factor(an, True, p.a.val)
    assert f.flag == 0
    n, nrhs = p.a.n, 32
    b = _rhs(n, nrhs, 7)
    x_dev = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    torch.cuda.synchronize()
    P = ctypes.c_void_p
    rc = lib.spldlt_tree_solve_fwd_noalloc_dbl(True, f.fkeep, nrhs, P(x_dev.data_ptr()), n, None)
    assert rc == -10
    assert np.array_equal(x_dev.cpu().numpy().T, b)
    # one right-hand side fits (about 175,000 doubles) and matches the
    # allocating entry point
    x1 = np.asfortranarray(b[:, :1].copy())
    rc = lib.spldlt_tree_solve_fwd_dbl(True, f.fkeep, 1, x1.ctypes.data_as(P), n)
    assert rc == 0
    x1_dev = torch.from_numpy(b[:, 0].copy()).cuda()
    torch.cuda.synchronize()
    rc = lib.spldlt_tree_solve_fwd_noalloc_dbl(True, f.fkeep, 1, P(x1_dev.data_ptr()), n, None)
    assert rc == 0
    got = x1_dev.cpu().numpy()
    assert np.abs(got - x1[:, 0]).max() <= 1e-12 * np.abs(x1).max()
