"""Benchmark: sparse SPD factor + solve to backward error 1e-14 on one GB300.

Workload: 3D 27-point weighted Laplacian on 80^3 (n = 512,000), log-normal
edge weights exp(N(0,1)), 16 right-hand sides N(0,1); FP32 factors with FP64
iterative refinement to a scaled backward error <= 1e-14 (the plain FP64 GPU
path is reported beside it).  A "step" is one numeric factorization plus
one refined solve of all right-hand sides.  The metric is the reference's
factor flop count (src/spldlt_analyse_mod.F90:1744-1764) divided by the
step time, in GFLOP/s.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Our arm prints `value` (inputs already in HBM: device-resident values and
right-hand sides through spldlt_factorize_device / spldlt_solve_device) and
`e2e` (the reference C-ABI with host buffers: spldlt_factorize_mixed +
spldlt_solve, host<->device copies inside the timed region).  The reference
arm times the CPU oracle (FP64 multifrontal over OpenBLAS, all host threads)
on the same workload.  Multi-GPU: the path does not shard, so N ranks run N
independent replicas (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "factor+solve s to backward err 1e-14: FP32+IR vs FP64, 1 GB300; GFLOP/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--k", type=int, default=80, help="grid edge (80 -> n=512,000)")
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--tol", type=float, default=1e-14)
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--no-ldlt", action="store_true",
                    help="skip the indefinite (shifted 7-point 48^3) factor + solve leg")
    ap.add_argument("--ldlt-k", type=int, default=48)
    ap.add_argument("--cpu-sample-k", type=int, default=0,
                    help="grid edge of the CPU baseline sample (0: auto)")
    ap.add_argument("--cpu-1core-k", type=int, default=40,
                    help="grid edge of the one-core sequential-BLAS CPU sample (0: skip)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed helpers (replicas only)

def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if _cuda_ok() else "gloo"
        dist.init_process_group(backend)
    return rank, ws


def _cuda_ok():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(v, ws):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if _cuda_ok() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks during the timed region

class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                     "--format=csv,noheader,nounits"], capture_output=True, text=True,
                    timeout=5).stdout.strip()
                if out:
                    self.samples.append([s.strip() for s in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for nm, v in zip(names, s[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


# ---------------------------------------------------------------------------

def workload(k, nrhs):
    from sylver_gb300 import workloads as w
    return w.lognormal27(k, nrhs=nrhs)


def traffic_record(kernel):
    """DRAM bytes per launch of `kernel` from the committed one-pass ncu record
    (profiles/traffic_lognormal27_80.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic_lognormal27_80.json")) as f:
            d = json.load(f)
        return d if d.get("kernel") == kernel else None
    except Exception:
        return None


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d["hbm_gbs"], d["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


def run_ours(args, rank, ws):
    import torch
    import sylver_gb300 as sg
    from sylver_gb300 import workloads as w

    lib = sg.load()
    torch.cuda.set_device(0)
    prob = workload(args.k, args.nrhs)
    a = prob.a
    an = sg.Analysis(a.n, a.ptr, a.row, order=prob.order)
    assert an.flag >= 0, an.flag
    flops = float(an.inform.num_flops)
    n, nrhs = a.n, args.nrhs
    prec = sg.FP32 if args.precision == "fp32" else sg.FP64
    maxit = 20

    stream = torch.cuda.ExternalStream(lib.sylver_gb300_stream())
    val_d = torch.from_numpy(a.val).cuda()
    b_d = torch.from_numpy(np.ascontiguousarray(prob.rhs.T)).cuda()  # nrhs x n == col-major n x nrhs
    x_d = torch.empty_like(b_d)
    torch.cuda.synchronize()

    opts = sg.default_options()
    fkeep = ctypes.c_void_p()
    inf = sg.Inform()
    P = ctypes.c_void_p

    def step_device():
        lib.spldlt_factorize_device(True, P(val_d.data_ptr()), an.akeep, ctypes.byref(fkeep),
                                    ctypes.byref(opts), ctypes.byref(inf), prec, args.tol, maxit)
        if inf.flag < 0:
            raise RuntimeError(f"factorize failed {inf.flag}")
        with torch.cuda.stream(stream):
            x_d.copy_(b_d)
        sinf = sg.Inform()
        lib.spldlt_solve_device(0, nrhs, P(x_d.data_ptr()), n, an.akeep, fkeep,
                                ctypes.byref(opts), ctypes.byref(sinf))
        if sinf.flag != 0:
            raise RuntimeError(f"solve flag {sinf.flag} (not converged or failed)")

    def timed(fn, steps, warm):
        for _ in range(warm):
            fn()
        barrier(ws)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        t0 = time.perf_counter()
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        barrier(ws)
        return e0.elapsed_time(e1) / 1e3, wall

    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        t_dev, wall_dev = timed(step_device, args.steps, args.warmup)
    it, be = ctypes.c_int(), ctypes.c_double()
    lib.sylver_gb300_solve_stats(fkeep, ctypes.byref(it), ctypes.byref(be))
    nl, lv, fms = ctypes.c_long(), ctypes.c_int(), ctypes.c_double()
    lib.sylver_gb300_fkeep_counters(fkeep, ctypes.byref(nl), ctypes.byref(lv), ctypes.byref(fms))
    # independent check of the final solution in FP64 on the host
    x_h = x_d.cpu().numpy().T
    full = a.to_scipy_full()
    be_host = float(w.backward_error(full, np.asfortranarray(x_h), prob.rhs).max())

    # e2e through the reference C-ABI with host buffers in pinned memory: the
    # values and the right-hand sides go host -> device and the solution
    # device -> host inside every step
    val_host = torch.empty(a.val.shape, dtype=torch.float64, pin_memory=True).numpy()
    val_host[:] = a.val
    rhs_t = torch.empty((nrhs, n), dtype=torch.float64, pin_memory=True)
    rhs_t.numpy().T[:] = prob.rhs
    x_t = torch.empty((nrhs, n), dtype=torch.float64, pin_memory=True)
    x_host = x_t.numpy().T  # n x nrhs, column-major, ldx = n
    f2 = ctypes.c_void_p()

    def step_e2e():
        lib.spldlt_factorize_mixed(True, None, None, val_host.ctypes.data_as(P), None, an.akeep,
                                   ctypes.byref(f2), ctypes.byref(opts), ctypes.byref(inf),
                                   prec, args.tol, maxit)
        x_t.copy_(rhs_t)  # the in-place solve overwrites x: restore the right-hand sides
        sinf = sg.Inform()
        lib.spldlt_solve(0, nrhs, x_host.ctypes.data_as(P), n, an.akeep, f2, ctypes.byref(opts),
                         ctypes.byref(sinf))
        if sinf.flag != 0:
            raise RuntimeError(f"solve flag {sinf.flag}")

    e2e_steps = args.steps
    t_e2e, wall_e2e = timed(step_e2e, e2e_steps, args.warmup)
    be_e2e = float(w.backward_error(full, x_host, prob.rhs).max())
    lib.spldlt_free_fkeep(ctypes.byref(f2))

    # per-kernel profile (extra factorization, outside the timed regions)
    ms = np.zeros(12); cnt = np.zeros(12, dtype=np.int64); fl = np.zeros(12)
    lib.sylver_gb300_profile_factor(fkeep, None, ms.ctypes.data_as(P), cnt.ctypes.data_as(P),
                                    fl.ctypes.data_as(P))
    kinds = sg.Factor.KINDS
    prof = {k: {"ms": round(float(ms[i]), 3), "launches": int(cnt[i])} for i, k in enumerate(kinds)
            if cnt[i]}
    hbm, bf16, src = peaks()

    def rate(k):
        return fl[k] / (ms[k] * 1e-3) / 1e12 if cnt[k] and ms[k] > 0 else 0.0
    # dominant update kernel: tensor-core (3xBF16, six BF16 MMAs per useful
    # flop) or SIMT tile update
    dom = 9 if ms[9] >= ms[5] else 5
    achieved = rate(dom)
    mma_rate = 6.0 * achieved if dom == 9 else achieved
    trec = traffic_record("k_update_tc") if dom == 9 and args.k == 80 else None

    # plain FP64 GPU path on the same workload (comparison)
    fp64 = None
    if prec == sg.FP32 and not args.no_fp64_compare:
        f3 = ctypes.c_void_p()

        def step64():
            lib.spldlt_factorize_device(True, P(val_d.data_ptr()), an.akeep, ctypes.byref(f3),
                                        ctypes.byref(opts), ctypes.byref(inf), sg.FP64, args.tol,
                                        maxit)
            with torch.cuda.stream(stream):
                x_d.copy_(b_d)
            sinf = sg.Inform()
            lib.spldlt_solve_device(0, nrhs, P(x_d.data_ptr()), n, an.akeep, f3,
                                    ctypes.byref(opts), ctypes.byref(sinf))
        t64, _ = timed(step64, 1, 1)
        it64, be64 = ctypes.c_int(), ctypes.c_double()
        lib.sylver_gb300_solve_stats(f3, ctypes.byref(it64), ctypes.byref(be64))
        fp64 = {"s_per_step": round(t64, 4), "gflops": round(flops / t64 / 1e9, 1),
                "ir_iters": it64.value, "bwd_err": be64.value,
                "fp32_speedup": round(t64 / (t_dev / args.steps), 2)}
        # roofline of the FP64 path's dominant kernel against the measured
        # FP64 FMA rate of this GPU (fma chains timed with CUDA events)
        ms64 = np.zeros(12); cnt64 = np.zeros(12, dtype=np.int64); fl64 = np.zeros(12)
        lib.sylver_gb300_profile_factor(f3, None, ms64.ctypes.data_as(P), cnt64.ctypes.data_as(P),
                                        fl64.ctypes.data_as(P))
        peak64 = ctypes.c_double()
        lib.sylver_gb300_fp64_fma_rate(ctypes.byref(peak64))
        d64 = int(np.argmax(ms64))
        ach64 = fl64[d64] / (ms64[d64] * 1e-3) / 1e12 if ms64[d64] > 0 else 0.0
        fp64["roofline"] = {
            "kernel": sg.Factor.KINDS[d64], "bound": "fp64 pipe",
            "achieved": round(ach64, 4), "peak": round(peak64.value, 4), "unit": "TFLOP/s",
            "frac": round(ach64 / peak64.value, 3) if peak64.value > 0 else None,
            "peak_source": "measured: independent fma chains on every SM, CUDA events",
            "share_of_profiled_factorization": round(float(ms64[d64] / max(ms64.sum(), 1e-9)), 3),
            "factor_rate_tflops": round(float(fl64.sum() / (ms64.sum() * 1e-3) / 1e12), 4)}
        lib.spldlt_free_fkeep(ctypes.byref(f3))

    ldlt = ldlt_leg(args, lib, stream) if (rank == 0 and not args.no_ldlt) else None

    t_step = allmax(t_dev / args.steps, ws)
    t_e2e_step = allmax(t_e2e / e2e_steps, ws)
    launches_step = int(nl.value) + 0
    cpu = cpu_baseline(args, flops) if rank == 0 else None
    h2d = a.val.nbytes + prob.rhs.nbytes
    d2h = prob.rhs.nbytes
    out = {
        "metric": METRIC, "value": round(ws * flops / t_step / 1e9, 2), "unit": "GFLOP/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(t_step * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if prec == sg.FP32 else "f64",
        "data": "synthetic (seeded 27-point log-normal Laplacian; no dataset)",
        "config": {"workload": f"lognormal27 {args.k}^3 SPD, n={n}, nrhs={nrhs}, "
                               f"{'FP32 factor + FP64 IR' if prec == sg.FP32 else 'FP64'} "
                               f"to bwd err {args.tol:g}",
                   "n": n, "nnz_lower": int(a.nnz), "nrhs": nrhs,
                   "factor_flops": flops, "fronts": int(an.inform.num_sup),
                   "maxfront": int(an.inform.maxfront),
                   "parallelism": f"replicas x{ws}",
                   "l2": "inputs larger than L2 (front arena of several GB per step)"},
        "e2e": {"value": round(ws * flops / t_e2e_step / 1e9, 2), "unit": "GFLOP/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": round(t_e2e_step * 1e3, 3), "bwd_err": be_e2e},
        "roofline": {"kernel": ("k_update_tc (tcgen05 3xBF16 Schur-complement update)"
                                if dom == 9 else "k_update (SIMT tile update)"),
                     "bound": "tensor", "achieved": round(achieved, 3), "peak": bf16,
                     "unit": "TFLOP/s", "frac": round(achieved / bf16, 4),
                     "peak_source": f"{src} dense bf16 (MEASURED_PEAKS.json)",
                     "achieved_counts": "useful (algorithmic) flops; 3xBF16 issues 6 BF16 "
                                        "MMA flops per useful flop",
                     "frac_note": "of measured dense bf16 peak; tensor_pipe_frac is the BF16 "
                                  "MMA rate (6x useful) against the same peak",
                     "tensor_pipe_tflops": round(mma_rate, 3),
                     "tensor_pipe_frac": round(mma_rate / bf16, 4),
                     "simt_update_tflops": round(rate(5), 3),
                     "launches": int(cnt[dom]),
                     "traffic": trec["per_launch_bytes"] if trec else None,
                     "traffic_unit": "bytes per launch (dram read + write)",
                     "traffic_source": ("one-pass ncu capture of every launch at this size, "
                                        "profiles/traffic_lognormal27_80.json") if trec else None,
                     "share_of_profiled_factorization": round(float(ms[dom] / max(ms.sum(), 1e-9)), 3),
                     "share_of_step": round(float(ms[dom]) / (t_dev / args.steps * 1e3), 3)},
        "kernel_profile_ms": prof,
        "accuracy": {"ir_iters": it.value, "bwd_err_device": be.value,
                     "bwd_err_host_check": be_host},
        "fp64_gpu_path": fp64,
        "ldlt_config2": ldlt,
        "clocks": clk.summary(),
        "gpu_launches": int(launches_step * args.steps),
        "cpu_baseline": cpu,
    }
    lib.spldlt_free_fkeep(ctypes.byref(fkeep))
    return out


def ldlt_leg(args, lib, stream):
    """Indefinite LDL^T on the shifted 7-point Laplacian (k^3 minus sigma*I,
    4 right-hand sides, APP threshold u = 0.01): factor + refined solve per
    step, device-resident values and right-hand sides, CUDA events on the
    library stream; FP32 factors + FP64 refinement and plain FP64 factors.
    Reported beside the headline; not part of its timed region."""
    import torch
    import sylver_gb300 as sg
    from sylver_gb300 import workloads as w
    p = w.shifted_laplace3d(args.ldlt_k, nrhs=4)
    a = p.a
    an = sg.Analysis(a.n, a.ptr, a.row, order=p.order)
    flops = float(an.inform.num_flops)
    n, nrhs = a.n, 4
    val_d = torch.from_numpy(a.val).cuda()
    b_d = torch.from_numpy(np.ascontiguousarray(p.rhs.T)).cuda()
    x_d = torch.empty_like(b_d)
    opts = sg.default_options()
    P = ctypes.c_void_p
    full = a.to_scipy_full()
    out = {"workload": f"shifted 7-point Laplacian {args.ldlt_k}^3 minus sigma*I, n={n}, "
                       f"nrhs={nrhs}, APP u=0.01", "factor_flops": flops}
    for name, prec in (("fp32_ir", sg.FP32), ("fp64", sg.FP64)):
        fk = ctypes.c_void_p()
        inf = sg.Inform()
        tf = ts = 0.0
        steps = 3
        for it in range(steps + 1):
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            torch.cuda.synchronize()
            e[0].record(stream)
            lib.spldlt_factorize_device(False, P(val_d.data_ptr()), an.akeep, ctypes.byref(fk),
                                        ctypes.byref(opts), ctypes.byref(inf), prec, 1e-14, 20)
            e[1].record(stream)
            with torch.cuda.stream(stream):
                x_d.copy_(b_d)
            sinf = sg.Inform()
            lib.spldlt_solve_device(0, nrhs, P(x_d.data_ptr()), n, an.akeep, fk,
                                    ctypes.byref(opts), ctypes.byref(sinf))
            e[2].record(stream)
            torch.cuda.synchronize()
            if it > 0:
                tf += e[0].elapsed_time(e[1]) / steps
                ts += e[1].elapsed_time(e[2]) / steps
        it_, be = ctypes.c_int(), ctypes.c_double()
        lib.sylver_gb300_solve_stats(fk, ctypes.byref(it_), ctypes.byref(be))
        x = x_d.cpu().numpy().T
        out[name] = {"factor_ms": round(tf, 3), "solve_ms": round(ts, 3),
                     "gflops": round(flops / ((tf + ts) * 1e-3) / 1e9, 1),
                     "ir_iters": it_.value,
                     "bwd_err_host_check": float(w.backward_error(full, np.asfortranarray(x),
                                                                  p.rhs).max()),
                     "inertia": [inf.num_neg, n - inf.matrix_rank, inf.matrix_rank - inf.num_neg],
                     "num_delay": inf.num_delay, "num_two": inf.num_two}
        lib.spldlt_free_fkeep(ctypes.byref(fk))
    out["inertia_closed_form"] = list(p.inertia)
    out["fp32_speedup_vs_fp64"] = round((out["fp64"]["factor_ms"] + out["fp64"]["solve_ms"]) /
                                        (out["fp32_ir"]["factor_ms"] + out["fp32_ir"]["solve_ms"]), 2)
    return out


def cpu_baseline(args, gpu_flops):
    """Oracle (CPU FP64 multifrontal over OpenBLAS, all host threads) on a
    bounded sample of the same workload: factor + solve + one refinement."""
    import oracle
    import sylver_gb300 as sg
    from sylver_gb300 import workloads as w
    oracle.build()
    oracle.load()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    k = args.cpu_sample_k or reference_sample_k(args)
    prob = workload(k, args.nrhs)
    an = sg.Analysis(prob.a.n, prob.a.ptr, prob.a.row, order=prob.order)
    full = prob.a.to_scipy_full()
    t0 = time.perf_counter()
    o = oracle.OracleFactor(True, an.symbolic(), prob.a.val)
    x = o.solve(prob.rhs)
    x = x + o.solve(prob.rhs - full @ x)
    t = time.perf_counter() - t0
    be = float(w.backward_error(full, x, prob.rhs).max())
    out = {"value": round(an.inform.num_flops / t / 1e9, 2), "unit": "GFLOP/s", "cores": cores,
           "kind": "port", "seconds": round(t, 3), "bwd_err": be,
           "sample": f"one factor+solve+1 IR of lognormal27 {k}^3 (n={prob.a.n}, "
                     f"nrhs={args.nrhs}), FP64, OpenBLAS {cores} threads",
           "host": host_cpu()}
    # one core, sequential BLAS, on a smaller grid of the same family (the
    # full grid would take minutes on one core)
    if args.cpu_1core_k > 0:
        oracle.set_threads(1)
        p1 = workload(args.cpu_1core_k, args.nrhs)
        an1 = sg.Analysis(p1.a.n, p1.a.ptr, p1.a.row, order=p1.order)
        full1 = p1.a.to_scipy_full()
        t0 = time.perf_counter()
        o1 = oracle.OracleFactor(True, an1.symbolic(), p1.a.val)
        x1 = o1.solve(p1.rhs)
        x1 = x1 + o1.solve(p1.rhs - full1 @ x1)
        t1 = time.perf_counter() - t0
        oracle.set_threads(cores)
        out["one_core"] = {
            "value": round(an1.inform.num_flops / t1 / 1e9, 2), "unit": "GFLOP/s", "cores": 1,
            "seconds": round(t1, 3), "bwd_err": float(w.backward_error(full1, x1, p1.rhs).max()),
            "sample": f"one factor+solve+1 IR of lognormal27 {args.cpu_1core_k}^3 "
                      f"(n={p1.a.n}, nrhs={args.nrhs}), FP64, OpenBLAS 1 thread (sequential)"}
    return out


def host_cpu():
    """Model, architecture and logical CPU count of the host (lscpu when
    present, else /proc/cpuinfo)."""
    import subprocess
    info = {"logical_cpus": os.cpu_count()}
    try:
        txt = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in txt.splitlines():
            key, _, val = line.partition(":")
            if key.strip() in ("Architecture", "Model name", "Thread(s) per core",
                               "Core(s) per socket", "Socket(s)", "CPU max MHz"):
                info[key.strip()] = val.strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return info


def reference_sample_k(args):
    """Grid edge of the reference arm's per-step sample: the largest edge <= args.k
    (a multiple of 4) whose steps and warm-ups together fit in about five minutes.
    One full 80^3 step of the FP64 oracle port takes about 23 s on the 16 Neoverse-V2
    cores of a GB300 host, and the factor work grows like k^6 on these grids."""
    budget_s, t80 = 300.0, 23.0
    per_step = budget_s / max(1, args.steps + args.warmup)
    k = int(80.0 * (per_step / t80) ** (1.0 / 6.0))
    return max(16, min(args.k, k // 4 * 4))


def run_reference(args, rank, ws):
    """CPU reference arm: the oracle port (FP64, all host threads)."""
    import oracle
    import sylver_gb300 as sg
    from sylver_gb300 import workloads as w
    oracle.build()
    oracle.load()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    k = args.cpu_sample_k or reference_sample_k(args)
    prob = workload(k, args.nrhs)
    an = sg.Analysis(prob.a.n, prob.a.ptr, prob.a.row, order=prob.order)
    sy = an.symbolic()
    full = prob.a.to_scipy_full()
    flops = float(an.inform.num_flops)

    def step():
        o = oracle.OracleFactor(True, sy, prob.a.val)
        x = o.solve(prob.rhs)
        return x + o.solve(prob.rhs - full @ x)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        x = step()
    t = (time.perf_counter() - t0) / args.steps
    be = float(w.backward_error(full, x, prob.rhs).max())
    v = round(flops / t / 1e9, 2)
    return {"metric": METRIC, "value": v, "unit": "GFLOP/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded 27-point log-normal Laplacian; no dataset)",
            "config": {"workload": f"lognormal27 {k}^3 SPD, n={prob.a.n}, nrhs={args.nrhs}, "
                                   "FP64 factor + 1 FP64 IR (CPU)",
                       "parallelism": "host threads"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "GFLOP/s", "cores": cores, "kind": "port",
                             "sample": f"one factor+solve+1 IR of lognormal27 {k}^3 (n={prob.a.n}, "
                                       f"nrhs={args.nrhs}) per step, sized so that {args.steps} "
                                       f"steps + {args.warmup} warm-ups fit in about 5 minutes; "
                                       f"FP64, OpenBLAS {cores} threads"},
            "e2e": {"value": v, "unit": "GFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "accuracy": {"bwd_err": be}}


def main():
    args = parse()
    rank, ws = dist_init()
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args, rank, ws)))
        return
    out = run_ours(args, rank, ws)
    if rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
