"""Autotuners and learned schedulers for the factorization's kernel paths.

A *schedule* (``sylver_gb300_schedule_t``) chooses which kernels process
which fronts -- for LDL^T, the column count below which a front skips the
a-posteriori block steps and goes straight to threshold partial pivoting;
for Cholesky, the small-front cutoff and the tensor-core threshold.  It never
changes the arithmetic of a pivot decision or an update.

* ``Autotuner`` measures every candidate schedule on the matrix (CUDA-event
  factor time reported by the library) and keeps the fastest: exact, but it
  costs one factorization per candidate.
* ``LearnedScheduler`` predicts the log factor time of each candidate with a
  small MLP (``sylver_gb300_mlp_*``: forward, backward and Adam kernels on the
  GPU) from features of the assembly tree -- front-size histograms, flop
  distribution and the delayed-pivot count the solver recorded on a first
  factorization -- and proposes the argmin after a single measurement; it
  falls back to the autotuner when it has no trained weights or the matrix is
  outside the range it was trained on.  Measured time is the judge of its
  error.

Cholesky (FP32 factors): the schedule is the blocked path's outer panel width
and group (fs_panel_cols, fs_panel_group), the small-front cutoff
(small_front_rows) and the tensor-core contribution-block threshold
(tc_min_cb_rows).  ``CholAutotuner`` sweeps the candidate grid with measured
factor times; ``CholLearnedScheduler`` predicts, for every candidate, the
time of each level of the assembly tree from features of that level (front
counts, sizes, flops) with the same GPU MLP, trained on the per-level
CUDA-event timings the library records (``sylver_gb300_profile_levels``) on
generated log-normal 27-point matrices; the predicted factor time is the sum
over levels, and the argmin is proposed from the analysis alone (no
factorization).  It falls back to the autotuner without weights or outside
its training range.

    python -m sylver_gb300.scheduler record OUT.npz [count] [seed0]
    python -m sylver_gb300.scheduler train DATA.npz OUT_WEIGHTS.npz [epochs]
    python -m sylver_gb300.scheduler evaluate WEIGHTS.npz [count] [seed0]
    python -m sylver_gb300.scheduler chol-record OUT.npz [count] [seed0]
    python -m sylver_gb300.scheduler chol-train DATA.npz OUT_WEIGHTS.npz [epochs]
    python -m sylver_gb300.scheduler chol-evaluate WEIGHTS.npz [k ...]
"""
from __future__ import annotations

import ctypes
import os
import sys
import time

import numpy as np

from . import FP32, FP64, Analysis, Factor, default_options, load, set_schedule
from . import workloads as w

HERE = os.path.dirname(os.path.abspath(__file__))
DATA = os.path.join(HERE, "data")

# LDL^T candidates: fronts with <= this many fully-summed columns use TPP only
LDLT_TPP_CANDIDATES = (0, 16, 32, 64, 96, 128, 192, 256, 512)
HIDDEN = 64


def kkt_instance(seed):
    """Training / evaluation instance of the saddle-point family: H a 7-point
    Laplacian on k^3 with k ~ U{8..16}, B with n_H/4 rows of 4 N(0,1)
    entries, delta = 1e-8 (the 40^3 configuration at small scale)."""
    rng = np.random.default_rng(seed)
    k = int(rng.integers(8, 17))
    return w.kkt(k, nnz_per_row=4, delta=1e-8, seed=seed, nrhs=1)


def analyse(p):
    opts = default_options()
    opts.ordering = 1
    return Analysis(p.a.n, p.a.ptr, p.a.row, options=opts)


def tree_features(an, posdef, precision, num_delay):
    """Features of one analysed matrix (independent of the schedule)."""
    sy = an.symbolic()
    m = np.diff(sy["rptr"]).astype(np.float64)
    n = np.diff(sy["sptr"]).astype(np.float64)
    fl = np.array([((mm) * (mm + 1) * (2 * mm + 1) - (mm - nn) * (mm - nn + 1) *
                    (2 * (mm - nn) + 1)) / 6.0 for mm, nn in zip(m, n)])
    F = max(fl.sum(), 1.0)
    f = [np.log2(max(an.n, 1)) / 24.0, np.log2(F) / 48.0, np.log2(max(m.max(), 1)) / 16.0,
         np.log2(len(m)) / 20.0, np.log2(max((m * m).sum(), 1)) / 40.0]
    for t in (8, 16, 32, 64, 128, 256, 512):
        f.append(float(np.mean(n <= t)))
    for t in (32, 128, 512):
        f.append(float(fl[n <= t].sum() / F))
    f += [float(posdef), float(precision), np.log2(1.0 + num_delay) / 16.0]
    return np.array(f, dtype=np.float32)


def schedule_features(tpp_cols):
    return np.array([tpp_cols / 512.0, float(tpp_cols > 0)], dtype=np.float32)


def measure(an, p, posdef, precision, schedule, repeats=2):
    """Factor time (ms, CUDA events, best of `repeats`) under a schedule."""
    set_schedule(**schedule)
    try:
        f = Factor(an, posdef, p.a.val, precision=precision)
        best = f.counters()["factor_ms"]
        for _ in range(repeats - 1):
            f.refactor(p.a.val, precision=precision)
            best = min(best, f.counters()["factor_ms"])
        return best, f.inform.num_delay, f.flag
    finally:
        set_schedule()


class Autotuner:
    """Exhaustive measured sweep over the candidate schedules."""

    def __init__(self, candidates=LDLT_TPP_CANDIDATES):
        self.candidates = candidates

    def tune(self, an, p, posdef=False, precision=FP64):
        times = {}
        for c in self.candidates:
            ms, _, flag = measure(an, p, posdef, precision, {"ldlt_tpp_cols": c})
            if flag >= 0:
                times[c] = ms
        best = min(times, key=times.get)
        return best, times


class Mlp:
    """GPU MLP (library kernels); parameters are a flat FP32 vector."""

    def __init__(self, nin, nhidden=HIDDEN, seed=0):
        self.lib = load()
        self.h = self.lib.sylver_gb300_mlp_create(int(nin), int(nhidden), int(seed))
        if not self.h:
            raise RuntimeError("sylver_gb300_mlp_create failed (no GPU?)")
        self.nin, self.nhidden = nin, nhidden
        self.np = int(self.lib.sylver_gb300_mlp_num_params(self.h))

    def params(self):
        p = np.zeros(self.np, np.float32)
        self.lib.sylver_gb300_mlp_get_params(self.h, p.ctypes.data_as(ctypes.c_void_p))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.np
        self.lib.sylver_gb300_mlp_set_params(self.h, p.ctypes.data_as(ctypes.c_void_p))

    def forward(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros(x.shape[0], np.float32)
        rc = self.lib.sylver_gb300_mlp_forward(self.h, x.ctypes.data_as(ctypes.c_void_p),
                                               x.shape[0], y.ctypes.data_as(ctypes.c_void_p))
        assert rc == 0
        return y

    def loss_grad(self, x, y):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        loss = np.zeros(1, np.float32)
        g = np.zeros(self.np, np.float32)
        rc = self.lib.sylver_gb300_mlp_loss_grad(self.h, x.ctypes.data_as(ctypes.c_void_p),
                                                 y.ctypes.data_as(ctypes.c_void_p), x.shape[0],
                                                 loss.ctypes.data_as(ctypes.c_void_p),
                                                 g.ctypes.data_as(ctypes.c_void_p))
        assert rc == 0
        return float(loss[0]), g

    def train(self, x, y, epochs=3000, lr=3e-3):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        loss = np.zeros(1, np.float32)
        rc = self.lib.sylver_gb300_mlp_train(self.h, x.ctypes.data_as(ctypes.c_void_p),
                                             y.ctypes.data_as(ctypes.c_void_p), x.shape[0],
                                             int(epochs), float(lr),
                                             loss.ctypes.data_as(ctypes.c_void_p))
        assert rc == 0
        return float(loss[0])

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.sylver_gb300_mlp_free(self.h)
            self.h = None


class LearnedScheduler:
    """Propose a schedule from the MLP's predicted factor times; fall back to
    the autotuner without weights or outside the training range."""

    def __init__(self, weights=None, autotuner=None):
        self.autotuner = autotuner or Autotuner()
        self.model = None
        if weights and os.path.exists(weights):
            z = np.load(weights)
            self.mu, self.sd = z["mu"], z["sd"]
            self.ymu, self.ysd = float(z["ymu"]), float(z["ysd"])
            self.fmin, self.fmax = z["fmin"], z["fmax"]
            self.model = Mlp(int(z["nin"]), int(z["nhidden"]))
            self.model.set_params(z["params"])

    def predict_ms(self, tf, candidates):
        x = np.stack([np.concatenate([tf, schedule_features(c)]) for c in candidates])
        y = self.model.forward((x - self.mu) / self.sd)
        return np.exp(y * self.ysd + self.ymu)

    def in_range(self, tf):
        span = self.fmax - self.fmin
        return bool(np.all(tf >= self.fmin - 0.25 * span) and np.all(tf <= self.fmax + 0.25 * span))

    def propose(self, an, p, posdef=False, precision=FP64):
        """Returns (tpp_cols, how, factorizations_used)."""
        if self.model is None:
            best, times = self.autotuner.tune(an, p, posdef, precision)
            return best, "autotuner", len(times)
        # one factorization under the default schedule records the delay history
        _, delays, _ = measure(an, p, posdef, precision, {"ldlt_tpp_cols": 0}, repeats=1)
        tf = tree_features(an, posdef, precision, delays)
        if not self.in_range(tf):
            best, times = self.autotuner.tune(an, p, posdef, precision)
            return best, "autotuner", 1 + len(times)
        cands = self.autotuner.candidates
        pred = self.predict_ms(tf, cands)
        return cands[int(np.argmin(pred))], "mlp", 1


# ---------------------------------------------------------------------------

def record(out, count=200, seed0=100):
    rows_x, rows_y, meta = [], [], []
    t0 = time.time()
    for s in range(seed0, seed0 + count):
        p = kkt_instance(s)
        an = analyse(p)
        base_ms, delays, flag = measure(an, p, False, FP64, {"ldlt_tpp_cols": 0})
        tf = tree_features(an, False, FP64, delays)
        for c in LDLT_TPP_CANDIDATES:
            ms, _, fl = measure(an, p, False, FP64, {"ldlt_tpp_cols": c})
            if fl < 0:
                continue
            rows_x.append(np.concatenate([tf, schedule_features(c)]))
            rows_y.append(np.log(ms))
            meta.append((s, c, ms))
        print(f"seed {s} n={p.a.n} base {base_ms:.2f} ms delays {delays} "
              f"({time.time() - t0:.0f}s)", flush=True)
        if (s - seed0) % 20 == 19:  # keep what was recorded so far
            np.savez_compressed(out, x=np.array(rows_x, np.float32),
                                y=np.array(rows_y, np.float32), meta=np.array(meta))
    np.savez_compressed(out, x=np.array(rows_x, np.float32), y=np.array(rows_y, np.float32),
                        meta=np.array(meta))


def train(data, out, epochs=4000, seed=0):
    z = np.load(data)
    x, y = z["x"], z["y"]
    ntf = x.shape[1] - 2
    mu, sd = x.mean(0), x.std(0) + 1e-6
    ymu, ysd = float(y.mean()), float(y.std() + 1e-6)
    xn, yn = (x - mu) / sd, (y - ymu) / ysd
    m = Mlp(x.shape[1], HIDDEN, seed)
    loss0, _ = m.loss_grad(xn, yn)
    loss = m.train(xn, yn, epochs=epochs)
    print(f"train {x.shape[0]} samples: loss {loss0:.4f} -> {loss:.4f}")
    np.savez_compressed(out, params=m.params(), mu=mu, sd=sd, ymu=ymu, ysd=ysd, nin=x.shape[1],
                        nhidden=HIDDEN, fmin=x[:, :ntf].min(0), fmax=x[:, :ntf].max(0),
                        loss0=loss0, loss=loss)
    return loss0, loss


def evaluate(weights, count=10, seed0=300):
    ls = LearnedScheduler(weights)
    at = ls.autotuner
    res = []
    for s in range(seed0, seed0 + count):
        p = kkt_instance(s)
        an = analyse(p)
        best, times = at.tune(an, p)
        choice, how, used = ls.propose(an, p)
        ms_choice, _, _ = measure(an, p, False, FP64, {"ldlt_tpp_cols": choice})
        res.append(dict(seed=s, n=p.a.n, default_ms=times[0], best=best, best_ms=times[best],
                        choice=choice, how=how, choice_ms=ms_choice, sweep=len(times), used=used))
        print(res[-1], flush=True)
    return res


# ---------------------------------------------------------------------------
# Cholesky schedules (FP32 factors), learned from per-level timings

CHOL_CANDIDATES = tuple(
    dict(fs_panel_cols=pc, fs_panel_group=g, small_front_rows=sm, tc_min_cb_rows=tc)
    for pc in (64, 128, 256) for g in (1, 2, 4) if pc * g <= 512
    for sm in (96, 128) for tc in (64, 256))
CHOL_DEFAULT = dict(fs_panel_cols=64, fs_panel_group=4, small_front_rows=96, tc_min_cb_rows=64)
CHOL_LEVEL_FEATURES = 10


def spd_instance(seed):
    """Training / evaluation instance of the SPD family: 27-point log-normal
    Laplacian on k^3, k ~ U{16..44} (the 80^3 configuration at small scale)."""
    rng = np.random.default_rng(seed)
    k = int(rng.integers(16, 45))
    return w.lognormal27(k, seed=seed, rhs_seed=seed + 1, nrhs=1)


def spd_analyse(p):
    return Analysis(p.a.n, p.a.ptr, p.a.row, order=p.order)


def level_features(an):
    """One row per level of the assembly tree (leaves first): fronts, sizes,
    flops and the fractions of fronts each kernel path would take."""
    sy = an.symbolic()
    m = np.diff(sy["rptr"]).astype(np.float64)
    n = np.diff(sy["sptr"]).astype(np.float64)
    par = np.asarray(sy["sparent"]) - 1
    nn = len(m)
    h = np.zeros(nn, np.int64)
    for i in range(nn):  # postorder: children first
        if 0 <= par[i] < nn:
            h[par[i]] = max(h[par[i]], h[i] + 1)
    fl = (m * (m + 1) * (2 * m + 1) - (m - n) * (m - n + 1) * (2 * (m - n) + 1)) / 6.0
    rows = []
    for lv in range(int(h.max()) + 1 if nn else 0):
        idx = np.nonzero(h == lv)[0]
        mm, nv, ff = m[idx], n[idx], fl[idx]
        rows.append([np.log2(1 + len(idx)) / 16, np.log2(1 + (mm * mm).sum()) / 40,
                     np.log2(1 + mm.max()) / 16, np.log2(1 + nv.max()) / 16,
                     np.log2(1 + ff.sum()) / 48, np.log2(1 + ff.max()) / 48,
                     float(np.mean(nv >= 96)), float(np.mean(mm - nv >= 64)),
                     float(np.mean(mm <= 128)), lv / 32.0])
    return np.array(rows, dtype=np.float32)


def chol_schedule_features(c):
    return np.array([c["fs_panel_cols"] / 256.0, c["fs_panel_group"] / 8.0,
                     c["small_front_rows"] / 128.0, np.log2(c["tc_min_cb_rows"]) / 8.0],
                    dtype=np.float32)


def chol_measure(an, p, sched, repeats=2, levels=False):
    """Measured FP32 factor time (ms, CUDA events, best of `repeats`) under a
    schedule, and optionally the per-level times of one more factorization."""
    set_schedule(**sched)
    try:
        f = Factor(an, True, p.a.val, precision=FP32)
        best = f.counters()["factor_ms"]
        for _ in range(repeats - 1):
            f.refactor(p.a.val, precision=FP32)
            best = min(best, f.counters()["factor_ms"])
        lv = f.profile_levels() if levels else None
        return best, lv, f.flag
    finally:
        set_schedule()


class CholAutotuner:
    """Measured sweep over the Cholesky candidate schedules."""

    def __init__(self, candidates=CHOL_CANDIDATES):
        self.candidates = candidates

    def tune(self, an, p):
        times = []
        for c in self.candidates:
            ms, _, flag = chol_measure(an, p, c)
            times.append(ms if flag >= 0 else np.inf)
        best = int(np.argmin(times))
        return self.candidates[best], times


class CholLearnedScheduler:
    """Per-level MLP over (level features, schedule); predicted factor time =
    sum over levels; proposes the argmin from the analysis alone."""

    def __init__(self, weights=None, autotuner=None):
        self.autotuner = autotuner or CholAutotuner()
        self.model = None
        if weights and os.path.exists(weights):
            z = np.load(weights)
            self.mu, self.sd = z["mu"], z["sd"]
            self.ymu, self.ysd = float(z["ymu"]), float(z["ysd"])
            self.fmin, self.fmax = z["fmin"], z["fmax"]
            self.model = Mlp(int(z["nin"]), int(z["nhidden"]))
            self.model.set_params(z["params"])

    def predict_ms(self, lf, candidates):
        out = []
        for c in candidates:
            sf = np.repeat(chol_schedule_features(c)[None, :], len(lf), 0)
            x = np.concatenate([lf, sf], 1)
            y = self.model.forward((x - self.mu) / self.sd)
            out.append(float(np.exp(y * self.ysd + self.ymu).sum()))
        return np.array(out)

    def in_range(self, lf):
        span = self.fmax - self.fmin
        return bool(np.all(lf >= self.fmin - 0.25 * span) and np.all(lf <= self.fmax + 0.25 * span))

    def propose(self, an, p):
        """Returns (schedule, how, factorizations_used)."""
        lf = level_features(an)
        if self.model is None or not self.in_range(lf):
            best, times = self.autotuner.tune(an, p)
            return best, "autotuner", 2 * len(times)
        cands = self.autotuner.candidates
        return cands[int(np.argmin(self.predict_ms(lf, cands)))], "mlp", 0


def chol_record(out, count=24, seed0=500):
    rows_x, rows_y, meta = [], [], []
    t0 = time.time()
    for s in range(seed0, seed0 + count):
        p = spd_instance(s)
        an = spd_analyse(p)
        lf = level_features(an)
        for ci, c in enumerate(CHOL_CANDIDATES):
            ms, lv, flag = chol_measure(an, p, c, repeats=1, levels=True)
            if flag < 0:
                continue
            for l in range(min(len(lv), len(lf))):
                rows_x.append(np.concatenate([lf[l], chol_schedule_features(c)]))
                rows_y.append(np.log(lv[l] + 1e-3))
                meta.append((s, ci, l, lv[l], ms))
        print(f"seed {s} n={p.a.n} levels {len(lf)} ({time.time() - t0:.0f}s)", flush=True)
    np.savez_compressed(out, x=np.array(rows_x, np.float32), y=np.array(rows_y, np.float32),
                        meta=np.array(meta))


def chol_train(data, out, epochs=6000, seed=0):
    z = np.load(data)
    x, y = z["x"], z["y"]
    mu, sd = x.mean(0), x.std(0) + 1e-6
    ymu, ysd = float(y.mean()), float(y.std() + 1e-6)
    m = Mlp(x.shape[1], HIDDEN, seed)
    xn, yn = (x - mu) / sd, (y - ymu) / ysd
    loss0, _ = m.loss_grad(xn, yn)
    loss = m.train(xn, yn, epochs=epochs, lr=2e-3)
    print(f"train {x.shape[0]} level samples: loss {loss0:.4f} -> {loss:.4f}")
    nlf = CHOL_LEVEL_FEATURES
    np.savez_compressed(out, params=m.params(), mu=mu, sd=sd, ymu=ymu, ysd=ysd, nin=x.shape[1],
                        nhidden=HIDDEN, fmin=x[:, :nlf].min(0), fmax=x[:, :nlf].max(0),
                        loss0=loss0, loss=loss)
    return loss0, loss


def chol_evaluate(weights, ks=(40, 56, 80)):
    """Default vs learned vs measured sweep (factor ms) on k^3 log-normal
    27-point matrices (seed 2, the benchmark's matrix at k = 80)."""
    ls = CholLearnedScheduler(weights)
    res = []
    for k in ks:
        p = w.lognormal27(k, nrhs=1)
        an = spd_analyse(p)
        t0 = time.perf_counter()
        choice, how, used = ls.propose(an, p)
        t_prop = time.perf_counter() - t0
        t0 = time.perf_counter()
        best, times = ls.autotuner.tune(an, p)
        t_sweep = time.perf_counter() - t0
        ci = ls.autotuner.candidates.index(choice)
        di = ls.autotuner.candidates.index(CHOL_DEFAULT)
        res.append(dict(k=k, n=p.a.n, default_ms=times[di], best=best, best_ms=min(times),
                        choice=choice, how=how, choice_ms=times[ci], propose_s=t_prop,
                        sweep_s=t_sweep, factorizations_used=used))
        print(res[-1], flush=True)
    return res


def main(argv):
    cmd = argv[0]
    if cmd == "chol-record":
        chol_record(argv[1], *(int(a) for a in argv[2:4]))
        return
    if cmd == "chol-train":
        chol_train(argv[1], argv[2], *(int(a) for a in argv[3:4]))
        return
    if cmd == "chol-evaluate":
        chol_evaluate(argv[1], tuple(int(a) for a in argv[2:]) or (40, 56, 80))
        return
    if cmd == "record":
        record(argv[1], *(int(a) for a in argv[2:4]))
    elif cmd == "train":
        train(argv[1], argv[2], *(int(a) for a in argv[3:4]))
    elif cmd == "evaluate":
        evaluate(argv[1], *(int(a) for a in argv[2:4]))
    else:
        raise SystemExit(__doc__)


if __name__ == "__main__":
    main(sys.argv[1:])
