"""Tensor-core (tcgen05, 3xBF16) Schur-complement update.

The self-check runs the same transposed split + TMA + tcgen05 path as the
factorization on a synthetic panel and compares with an FP64 host product;
3xBF16 with six products and FP32 accumulation of 64-wide k chunks must be
close to FP32 accuracy: the bound 1e-5 is two orders of magnitude below what
a single BF16 product (unit roundoff ~4e-3) gives and about what FP32
accumulation over K <= 257 terms gives.  The larger cases have more tiles
than the GPU has SMs, so persistent CTAs walk several tiles and reuse every
accumulator and pipeline stage."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rows,k", [(128, 32), (200, 70), (300, 257), (1000, 96),
                                    (2500, 160), (4000, 64)])
def test_tc_update_selfcheck(sylver, gpu, rows, k):
    lib = sylver.load()
    err = ctypes.c_double(-1.0)
    rc = lib.sylver_gb300_tc_selfcheck(rows, k, ctypes.byref(err))
    assert rc == 0
    assert 0.0 <= err.value <= 1e-5, err.value
