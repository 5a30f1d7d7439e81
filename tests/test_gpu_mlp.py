"""The schedule MLP's GPU kernels against the FP64 NumPy oracle, and what the
trained network gains over the schedule search without it.

Tolerances: forward outputs and gradients are FP32 kernels checked against an
FP64 restatement -- relative error <= 1e-4 in the 2-norm (FP32 rounding of
sums of ~100 terms is ~1e-6; the margin covers reordered accumulation)."""
import os
import time

import numpy as np
import pytest

from oracle import mlp as omlp

pytestmark = pytest.mark.gpu

D0, H = 23, 32


def _data(seed, B=61):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((B, D0)).astype(np.float32)
    wt = rng.standard_normal(D0)
    y = (np.tanh(x @ wt / 4.0) + 0.1 * np.sin(3 * x[:, 0])).astype(np.float32)
    return x, y


def test_mlp_forward_and_gradient_match_oracle(sylver, gpu):
    from sylver_gb300.scheduler import Mlp
    m = Mlp(D0, H, seed=7)
    p = m.params()
    assert p.size == H * D0 + H + H * H + H + H + 1
    x, y = _data(1)
    yg = m.forward(x)
    yo, _ = omlp.forward(p, x, D0, H)
    assert np.linalg.norm(yg - yo) <= 1e-4 * np.linalg.norm(yo)
    lg, gg = m.loss_grad(x, y)
    lo, go = omlp.loss_grad(p, x, y, D0, H)
    assert abs(lg - lo) <= 1e-4 * lo
    assert np.linalg.norm(gg - go) <= 1e-4 * np.linalg.norm(go)
    # per block too: every layer's gradient, not just the dominant one
    o = 0
    for k in (H * D0, H, H * H, H, H, 1):
        a, b = gg[o:o + k], go[o:o + k]
        assert np.linalg.norm(a - b) <= 1e-4 * max(np.linalg.norm(b), 1e-6), o
        o += k


def test_mlp_gradient_matches_finite_differences_of_oracle(sylver, gpu):
    """Independent of the oracle's backward pass: central differences of the
    oracle's FP64 loss at the GPU's parameters."""
    from sylver_gb300.scheduler import Mlp
    m = Mlp(D0, H, seed=3)
    p = m.params().astype(np.float64)
    x, y = _data(2)
    _, gg = m.loss_grad(x, y)
    rng = np.random.default_rng(0)
    for i in rng.choice(p.size, 40, replace=False):
        e = np.zeros_like(p); e[i] = 1e-6
        fd = (omlp.loss_grad(p + e, x, y, D0, H)[0] - omlp.loss_grad(p - e, x, y, D0, H)[0]) / 2e-6
        assert abs(gg[i] - fd) <= 2e-4 * max(1.0, np.abs(gg).max()), i


def test_mlp_training_follows_oracle_adam(sylver, gpu):
    from sylver_gb300.scheduler import Mlp
    m = Mlp(D0, H, seed=11)
    p0 = m.params()
    x, y = _data(3, B=200)
    l0, _ = m.loss_grad(x, y)
    lg = m.train(x, y, epochs=300, lr=3e-3)
    po, lo = omlp.adam_train(p0, x, y, D0, H, epochs=300, lr=3e-3)
    assert lg < 0.2 * l0 and lo < 0.2 * l0
    # FP32 and FP64 Adam trajectories agree to well within the loss drop
    assert abs(lg - lo) <= 0.05 * l0
    assert np.linalg.norm(m.params() - po) <= 0.05 * np.linalg.norm(po)


WEIGHTS = os.path.join(os.path.dirname(__file__), "..", "sylver_gb300", "data", "sched_mlp.npz")


def test_learned_schedule_gains_over_search_without_it(sylver, gpu):
    """Held-out saddle-point instances (seeds never used in training).  The
    method without the network is the measured sweep over every candidate
    schedule.  The network proposes from one factorization, and its choice is
    judged by measured time: within 10% (+0.5 ms) of the sweep's best in total,
    never slower in total than the default schedule, at a fraction of the
    sweep's tuning cost."""
    from sylver_gb300 import scheduler as sc
    assert os.path.exists(WEIGHTS), "trained schedule weights missing"
    ls = sc.LearnedScheduler(WEIGHTS)
    assert ls.model is not None
    tot = dict(default=0.0, best=0.0, mlp=0.0, sweep_s=0.0, mlp_s=0.0)
    for s in (400, 401, 402, 403):
        p = sc.kkt_instance(s)
        an = sc.analyse(p)
        sc.measure(an, p, False, sylver.FP64, {"ldlt_tpp_cols": 0}, repeats=1)  # warm-up
        t0 = time.perf_counter()
        best, times = ls.autotuner.tune(an, p)
        tot["sweep_s"] += time.perf_counter() - t0
        t0 = time.perf_counter()
        choice, how, used = ls.propose(an, p)
        tot["mlp_s"] += time.perf_counter() - t0
        assert how == "mlp" and used == 1
        ms, _, flag = sc.measure(an, p, False, sylver.FP64, {"ldlt_tpp_cols": choice})
        assert flag >= 0
        tot["default"] += times[0]
        tot["best"] += times[best]
        tot["mlp"] += ms
        print(f"seed {s}: default {times[0]:.2f} best {times[best]:.2f} (tpp {best}) "
              f"mlp {ms:.2f} (tpp {choice})")
    print(tot)
    assert tot["mlp"] <= 1.10 * tot["best"] + 0.5
    assert tot["mlp"] <= 1.02 * tot["default"] + 0.5
    assert tot["mlp_s"] < 0.5 * tot["sweep_s"]


CHOL_WEIGHTS = os.path.join(os.path.dirname(__file__), "..", "sylver_gb300", "data",
                            "sched_chol_mlp.npz")


def test_learned_cholesky_schedule_against_sweep(sylver, gpu):
    """Cholesky schedule (panel width and group, small-front cutoff, tensor-core
    threshold) from the per-level MLP, on held-out log-normal matrices (seeds
    outside the training range 500-523): proposed from the analysis alone (no
    factorization), within 5 % (+0.2 ms) of the measured sweep's best and not
    slower than the default schedule by more than 2 % (+0.2 ms), judged by
    measured factor time."""
    from sylver_gb300 import scheduler as sc
    assert os.path.exists(CHOL_WEIGHTS), "trained Cholesky schedule weights missing"
    ls = sc.CholLearnedScheduler(CHOL_WEIGHTS)
    assert ls.model is not None
    tot = dict(default=0.0, best=0.0, mlp=0.0)
    for s in (900, 901):
        p = sc.spd_instance(s)
        an = sc.spd_analyse(p)
        choice, how, used = ls.propose(an, p)
        assert how == "mlp" and used == 0
        best, times = ls.autotuner.tune(an, p)
        ci = ls.autotuner.candidates.index(choice)
        di = ls.autotuner.candidates.index(sc.CHOL_DEFAULT)
        tot["default"] += times[di]
        tot["best"] += min(times)
        tot["mlp"] += times[ci]
        print(f"seed {s} n={p.a.n}: default {times[di]:.3f} best {min(times):.3f} "
              f"mlp {times[ci]:.3f} {choice}")
    print(tot)
    assert tot["mlp"] <= 1.05 * tot["best"] + 0.2
    assert tot["mlp"] <= 1.02 * tot["default"] + 0.2
