"""Configuration 4: 2,000 independent SPD instances (5-point Laplacians on
s x s grids, s ~ U{8..64}, random shifts) factorized and solved together.

The instances are stacked into one block-diagonal system; their assembly
trees form a forest, so every level of every tree shares the same launches
and the whole factorization is one captured launch sequence.  FP32 factors,
FP64 refinement; each instance must reach a scaled backward error <= 1e-14."""
import numpy as np
import pytest

from sylver_gb300 import workloads as w

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    probs = w.batched_laplace2d(2000)
    big, offs = w.block_diagonal(probs)
    return probs, big, offs


def test_batched_instances_one_launch_sequence(sylver, orc, gpu, batch):
    probs, big, offs = batch
    an = sylver.Analysis(big.a.n, big.a.ptr, big.a.row, order=big.order)
    assert an.flag == 0
    f = sylver.Factor(an, True, big.a.val, precision=sylver.FP32, ir_tol=1e-15, ir_max_iter=10)
    assert f.flag == 0
    c = f.counters()
    # one launch sequence for all 2,000 trees: launches scale with tree
    # height, not with the number of instances
    assert c["kernel_launches"] < 200, c
    x = f.solve(big.rhs)
    be = w.instance_backward_errors(probs, offs, x)
    assert be.max() <= 1e-14, be.max()
    # spot-check instances against the FP64 oracle
    for k in (0, 777, 1999):
        p = probs[k]
        an_k = sylver.Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)
        o = orc.OracleFactor(True, an_k.symbolic(), p.a.val)
        xo = o.solve(p.rhs)
        xk = x[offs[k]:offs[k + 1]]
        assert np.abs(xk - xo).max() <= 1e-10 * np.abs(xo).max()
