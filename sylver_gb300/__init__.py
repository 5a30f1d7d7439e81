"""sylver_gb300 -- GB300-native numeric factorize + solve behind SyLVER's C-ABI.

The product is the shared library ``_build/libsylver_gb300.so`` (host C++ and
sm_103a CUDA).  This module is a thin ctypes mirror of the reference C
interface (include/sylver/sylver.h:73-123): the same entry points, argument
meaning and flag values, so tests read like the reference's own drivers.
There is no CPU fallback: loading fails loudly when the library is missing,
and factorize returns SYLVER_ERROR_CUDA_UNKNOWN (-51) without a GPU.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsylver_gb300.so")

FP64 = 0
FP32 = 1

FLAGS = {
    0: "SUCCESS", -1: "ERROR_CALL_SEQUENCE", -2: "ERROR_A_N_OOR", -3: "ERROR_A_PTR",
    -4: "ERROR_A_ALL_OOR", -5: "ERROR_SINGULAR", -6: "ERROR_NOT_POS_DEF",
    -7: "ERROR_PTR_ROW", -8: "ERROR_ORDER", -9: "ERROR_VAL", -10: "ERROR_X_SIZE",
    -11: "ERROR_JOB_OOR", -50: "ERROR_ALLOCATION", -51: "ERROR_CUDA_UNKNOWN",
    -98: "ERROR_UNIMPLEMENTED", -99: "ERROR_UNKNOWN", 1: "WARNING_IDX_OOR",
    2: "WARNING_DUP_IDX", 3: "WARNING_DUP_AND_OOR", 4: "WARNING_MISSING_DIAGONAL",
    5: "WARNING_MISS_DIAG_OORDUP", 6: "WARNING_ANAL_SINGULAR", 7: "WARNING_FACT_SINGULAR",
    8: "WARNING_MATCH_ORD_NO_SCALE", 9: "GB300_WARNING_IR_NOT_CONVERGED",
    -13: "ERROR_NOT_LLT", -14: "ERROR_NOT_LDLT", -15: "ERROR_NO_SAVED_SCALING",
    -52: "ERROR_CUBLAS_UNKNOWN",
}
WARNING_IR_NOT_CONVERGED = 9


class Inform(ctypes.Structure):
    """sylver_inform_t (include/sylver/sylver.h:19-37)."""
    _fields_ = [("flag", ctypes.c_int), ("matrix_dup", ctypes.c_int),
                ("matrix_missing_diag", ctypes.c_int), ("matrix_outrange", ctypes.c_int),
                ("matrix_rank", ctypes.c_int), ("maxdepth", ctypes.c_int),
                ("maxfront", ctypes.c_int), ("num_delay", ctypes.c_int),
                ("num_factor", ctypes.c_long), ("num_flops", ctypes.c_long),
                ("num_neg", ctypes.c_int), ("num_sup", ctypes.c_int),
                ("num_two", ctypes.c_int), ("stat", ctypes.c_int),
                ("cuda_error", ctypes.c_int), ("cublas_error", ctypes.c_int),
                ("unused", ctypes.c_char * 80)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "unused"}


class Options(ctypes.Structure):
    """sylver_options_t (include/sylver/sylver.h:39-71)."""
    _fields_ = [("array_base", ctypes.c_int), ("print_level", ctypes.c_int),
                ("unit_diagnostics", ctypes.c_int), ("unit_error", ctypes.c_int),
                ("unit_warning", ctypes.c_int), ("ordering", ctypes.c_int),
                ("nemin", ctypes.c_int), ("prune_tree", ctypes.c_bool),
                ("min_gpu_work", ctypes.c_long), ("scaling", ctypes.c_int),
                ("pivot_method", ctypes.c_int), ("small", ctypes.c_double),
                ("u", ctypes.c_double), ("small_subtree_threshold", ctypes.c_long),
                ("nb", ctypes.c_int), ("cpu_topology", ctypes.c_int),
                ("action", ctypes.c_bool), ("use_gpu", ctypes.c_bool),
                ("gpu_perf_coeff", ctypes.c_double), ("failed_pivot_method", ctypes.c_int),
                ("scheduler", ctypes.c_int)]


class OptionsC(ctypes.Structure):
    """sylver_options_c, the seam's options_c (src/sylver_ciface.hxx:39-51)."""
    _fields_ = [("print_level", ctypes.c_int), ("action", ctypes.c_bool),
                ("small", ctypes.c_double), ("u", ctypes.c_double),
                ("multiplier", ctypes.c_double), ("small_subtree_threshold", ctypes.c_long),
                ("nb", ctypes.c_int), ("pivot_method", ctypes.c_int),
                ("failed_pivot_method", ctypes.c_int), ("cpu_topology", ctypes.c_int)]


class InformC(ctypes.Structure):
    """sylver_inform_c, the seam's inform_c (src/sylver_ciface.hxx:74-87)."""
    _fields_ = [("flag", ctypes.c_int), ("num_delay", ctypes.c_int),
                ("num_neg", ctypes.c_int), ("num_two", ctypes.c_int),
                ("num_zero", ctypes.c_int), ("maxfront", ctypes.c_int),
                ("not_first_pass", ctypes.c_int), ("not_second_pass", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Schedule(ctypes.Structure):
    """sylver_gb300_schedule_t: kernel-path choices (0 = default)."""
    _fields_ = [("small_front_rows", ctypes.c_int), ("tc_min_cb_rows", ctypes.c_int),
                ("solve_large_cols", ctypes.c_int), ("ldlt_tpp_cols", ctypes.c_int),
                ("fs_panel_cols", ctypes.c_int), ("fs_panel_group", ctypes.c_int),
                ("front_memory", ctypes.c_int), ("solve_dataflow", ctypes.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def set_schedule(**kw):
    """Schedule for factorizations planned afterwards; no arguments = defaults."""
    if not kw:
        load().sylver_gb300_set_schedule(None)
        return
    s = Schedule(**{k: int(v) for k, v in kw.items()})
    load().sylver_gb300_set_schedule(ctypes.byref(s))


def get_schedule():
    s = Schedule()
    load().sylver_gb300_get_schedule(ctypes.byref(s))
    return s.as_dict()


_lib = None

# every extern "C" entry point declared in include/sylver_gb300.h
EXPORTS = (
    "sylver_init", "sylver_finalize", "sylver_default_options", "spldlt_analyse",
    "spldlt_factorize", "spldlt_solve", "spldlt_free_akeep", "spldlt_free_fkeep",
    "spldlt_create_symbolic_tree", "spldlt_destroy_symbolic_tree",
    "spldlt_create_numeric_tree_dbl", "spldlt_create_numeric_tree_posdef_dbl",
    "spldlt_destroy_numeric_tree_dbl", "spldlt_destroy_numeric_tree_posdef_dbl",
    "spldlt_tree_solve_fwd_dbl", "spldlt_tree_solve_bwd_dbl", "spldlt_tree_solve_diag_dbl",
    "spldlt_tree_solve_diag_bwd_dbl", "spldlt_tree_solve_fwd_posdef_dbl",
    "spldlt_tree_solve_bwd_posdef_dbl", "spldlt_factorize_mixed", "spldlt_factorize_device",
    "spldlt_solve_device", "sylver_gb300_solve_stats", "sylver_gb300_akeep_sizes",
    "sylver_gb300_akeep_arrays", "sylver_gb300_fkeep_diag", "sylver_gb300_fkeep_counters",
    "sylver_gb300_fkeep_fronts", "sylver_gb300_akeep_scaling", "sylver_gb300_profile_levels",
    "sylver_gb300_stream", "sylver_gb300_profile_factor", "spldlt_tree_solve_fwd_noalloc_dbl",
    "sylver_gb300_tc_selfcheck", "sylver_gb300_fp64_fma_rate", "sylver_gb300_fkeep_factor_bytes",
    "sylver_gb300_dataflow_selftest",
    "sylver_gb300_solve_history", "sylver_gb300_set_schedule",
    "sylver_gb300_get_schedule", "sylver_gb300_profile_solve", "sylver_gb300_mlp_create", "sylver_gb300_mlp_free",
    "sylver_gb300_mlp_num_params", "sylver_gb300_mlp_set_params", "sylver_gb300_mlp_get_params",
    "sylver_gb300_mlp_forward", "sylver_gb300_mlp_loss_grad", "sylver_gb300_mlp_train",
)


def build(force=False):
    from . import native_build
    return native_build.build(force=force)


def load(path: str | None = None):
    """Load the native library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"sylver_gb300 native library missing: {path} (run build())")
    lib = ctypes.CDLL(path)
    P, I, L, D, B = ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_double, ctypes.c_bool
    PP = ctypes.POINTER(ctypes.c_void_p)
    PO, PI = ctypes.POINTER(Options), ctypes.POINTER(Inform)
    sig = {
        "sylver_init": (None, [I, I]),
        "sylver_finalize": (None, []),
        "sylver_default_options": (None, [PO]),
        "spldlt_analyse": (None, [I, P, P, P, P, PP, B, PO, PI]),
        "spldlt_factorize": (None, [B, P, P, P, P, P, PP, PO, PI]),
        "spldlt_factorize_mixed": (None, [B, P, P, P, P, P, PP, PO, PI, I, D, I]),
        "spldlt_factorize_device": (None, [B, P, P, PP, PO, PI, I, D, I]),
        "spldlt_solve": (None, [I, I, P, I, P, P, PO, PI]),
        "spldlt_solve_device": (None, [I, I, P, I, P, P, PO, PI]),
        "spldlt_free_akeep": (None, [PP]),
        "spldlt_free_fkeep": (None, [PP]),
        "sylver_gb300_solve_stats": (I, [P, ctypes.POINTER(I), ctypes.POINTER(D)]),
        "sylver_gb300_akeep_sizes": (I, [P, ctypes.POINTER(I), ctypes.POINTER(I),
                                         ctypes.POINTER(L), ctypes.POINTER(L)]),
        "sylver_gb300_akeep_arrays": (I, [P, P, P, P, P, P, P, P]),
        "sylver_gb300_fkeep_diag": (I, [P, P, P]),
        "sylver_gb300_fkeep_fronts": (I, [P, P, P, P]),
        "sylver_gb300_akeep_scaling": (I, [P, P]),
        "sylver_gb300_profile_levels": (I, [P, P, P, I]),
        "sylver_gb300_fkeep_counters": (I, [P, ctypes.POINTER(L), ctypes.POINTER(I),
                                            ctypes.POINTER(D)]),
        "sylver_gb300_stream": (P, []),
        "sylver_gb300_profile_factor": (I, [P, P, P, P, P]),
        "sylver_gb300_profile_solve": (I, [P, I, P, P]),
        "sylver_gb300_tc_selfcheck": (I, [I, I, ctypes.POINTER(D)]),
        "sylver_gb300_dataflow_selftest": (I, [I, ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(D)]),
        "sylver_gb300_fp64_fma_rate": (I, [ctypes.POINTER(D)]),
        "sylver_gb300_fkeep_factor_bytes": (L, [P, P, L]),
        "sylver_gb300_solve_history": (I, [P, P, I]),
        "sylver_gb300_set_schedule": (None, [ctypes.POINTER(Schedule)]),
        "sylver_gb300_get_schedule": (None, [ctypes.POINTER(Schedule)]),
        "sylver_gb300_mlp_create": (P, [I, I, ctypes.c_uint]),
        "sylver_gb300_mlp_free": (None, [P]),
        "sylver_gb300_mlp_num_params": (L, [P]),
        "sylver_gb300_mlp_set_params": (I, [P, P]),
        "sylver_gb300_mlp_get_params": (I, [P, P]),
        "sylver_gb300_mlp_forward": (I, [P, P, I, P]),
        "sylver_gb300_mlp_loss_grad": (I, [P, P, P, I, P, P]),
        "sylver_gb300_mlp_train": (I, [P, P, P, I, I, ctypes.c_float, P]),
        "spldlt_create_symbolic_tree": (P, [P, I, I, P, P, P, P, P, P, I, P, P, P, P]),
        "spldlt_destroy_symbolic_tree": (None, [P]),
        "spldlt_create_numeric_tree_dbl": (P, [B, P, P, P, P, P, ctypes.POINTER(OptionsC),
                                               ctypes.POINTER(InformC)]),
        "spldlt_create_numeric_tree_posdef_dbl": (P, [P, P, P, P, P, ctypes.POINTER(OptionsC),
                                                      ctypes.POINTER(InformC)]),
        "spldlt_destroy_numeric_tree_dbl": (None, [B, P]),
        "spldlt_destroy_numeric_tree_posdef_dbl": (None, [P]),
        "spldlt_tree_solve_fwd_posdef_dbl": (I, [P, I, P, I]),
        "spldlt_tree_solve_bwd_posdef_dbl": (I, [P, I, P, I]),
        "spldlt_tree_solve_fwd_dbl": (I, [B, P, I, P, I]),
        "spldlt_tree_solve_bwd_dbl": (I, [B, P, I, P, I]),
        "spldlt_tree_solve_diag_dbl": (I, [B, P, I, P, I]),
        "spldlt_tree_solve_diag_bwd_dbl": (I, [B, P, I, P, I]),
        "spldlt_tree_solve_fwd_noalloc_dbl": (I, [B, P, I, P, I, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def default_options() -> Options:
    o = Options()
    load().sylver_default_options(ctypes.byref(o))
    return o


class Analysis:
    """Result of spldlt_analyse (owns akeep)."""

    def __init__(self, n, ptr, row, order=None, options=None, check=True, val=None):
        lib = load()
        self.options = options or default_options()
        if order is not None:
            self.options.ordering = 0
            self._order = np.ascontiguousarray(order, dtype=np.int32)
        else:
            self._order = None
        self._ptr = np.ascontiguousarray(ptr, dtype=np.int64)
        self._row = np.ascontiguousarray(row, dtype=np.int32)
        self.n = int(n)
        self.akeep = ctypes.c_void_p()
        self.inform = Inform()
        self._val = None if val is None else np.ascontiguousarray(val, dtype=np.float64)
        lib.spldlt_analyse(self.n, _p(self._order) if self._order is not None else None,
                           _p(self._ptr), _p(self._row),
                           _p(self._val) if self._val is not None else None,
                           ctypes.byref(self.akeep),
                           bool(check), ctypes.byref(self.options), ctypes.byref(self.inform))
        self.flag = self.inform.flag

    def scaling(self):
        """Scaling saved by a matching-based analysis (user order) or None."""
        s = np.zeros(max(self.n, 1))
        k = load().sylver_gb300_akeep_scaling(self.akeep, _p(s))
        return s[:k] if k > 0 else None

    def symbolic(self):
        """SymbolicTree arrays (1-based, reference layout) + perm."""
        lib = load()
        n, nn = ctypes.c_int(), ctypes.c_int()
        rl, nl = ctypes.c_long(), ctypes.c_long()
        lib.sylver_gb300_akeep_sizes(self.akeep, ctypes.byref(n), ctypes.byref(nn),
                                     ctypes.byref(rl), ctypes.byref(nl))
        nn = nn.value
        out = dict(n=n.value, nnodes=nn,
                   sptr=np.zeros(nn + 1, np.int32), sparent=np.zeros(max(nn, 1), np.int32),
                   rptr=np.zeros(nn + 1, np.int64), rlist=np.zeros(max(rl.value, 1), np.int32),
                   nptr=np.zeros(nn + 1, np.int64), nlist=np.zeros(max(nl.value, 1), np.int64),
                   perm=np.zeros(max(n.value, 1), np.int32))
        lib.sylver_gb300_akeep_arrays(self.akeep, _p(out["sptr"]), _p(out["sparent"]),
                                      _p(out["rptr"]), _p(out["rlist"]), _p(out["nptr"]),
                                      _p(out["nlist"]), _p(out["perm"]))
        out["sparent"] = out["sparent"][:nn]
        out["rlist"] = out["rlist"][:rl.value]
        out["nlist"] = out["nlist"][:nl.value]
        out["perm"] = out["perm"][:n.value]
        return out

    def __del__(self):
        if getattr(self, "akeep", None) and _lib is not None and self.akeep:
            _lib.spldlt_free_akeep(ctypes.byref(self.akeep))


class Factor:
    """Result of spldlt_factorize / spldlt_factorize_mixed (owns fkeep)."""

    def __init__(self, analysis: Analysis, posdef: bool, val, precision=FP64,
                 ir_tol=1e-14, ir_max_iter=0, options=None, scale=None, ptr=None, row=None):
        lib = load()
        self.analysis = analysis
        self.options = options or analysis.options
        self.posdef = bool(posdef)
        self.fkeep = ctypes.c_void_p()
        self.inform = Inform()
        self.refactor(val, precision=precision, ir_tol=ir_tol, ir_max_iter=ir_max_iter,
                      scale=scale)

    def refactor(self, val, precision=FP64, ir_tol=1e-14, ir_max_iter=0, scale=None):
        lib = load()
        self._val = np.ascontiguousarray(val, dtype=np.float64)
        self._scale = None if scale is None else np.ascontiguousarray(scale, dtype=np.float64)
        lib.spldlt_factorize_mixed(self.posdef, None, None, _p(self._val),
                                   _p(self._scale) if self._scale is not None else None,
                                   self.analysis.akeep, ctypes.byref(self.fkeep),
                                   ctypes.byref(self.options), ctypes.byref(self.inform),
                                   int(precision), float(ir_tol), int(ir_max_iter))
        self.flag = self.inform.flag
        return self.flag

    def solve(self, b, job=0):
        x = np.array(b, dtype=np.float64, order="F", copy=True)
        if x.ndim == 1:
            x = x.reshape(-1, 1, order="F")
        inf = Inform()
        load().spldlt_solve(int(job), x.shape[1], _p(x), x.shape[0], self.analysis.akeep,
                            self.fkeep, ctypes.byref(self.options), ctypes.byref(inf))
        self.solve_inform = inf
        if inf.flag < 0:
            raise RuntimeError(f"spldlt_solve failed: {inf.flag} {FLAGS.get(inf.flag)}")
        return x

    def solve_stats(self):
        it, be = ctypes.c_int(), ctypes.c_double()
        load().sylver_gb300_solve_stats(self.fkeep, ctypes.byref(it), ctypes.byref(be))
        return it.value, be.value

    def solve_history(self):
        h = np.zeros(64)
        k = load().sylver_gb300_solve_history(self.fkeep, _p(h), 64)
        return h[:max(k, 0)].tolist()

    def counters(self):
        nl, lv, ms = ctypes.c_long(), ctypes.c_int(), ctypes.c_double()
        load().sylver_gb300_fkeep_counters(self.fkeep, ctypes.byref(nl), ctypes.byref(lv),
                                           ctypes.byref(ms))
        return dict(kernel_launches=nl.value, nlevels=lv.value, factor_ms=ms.value)

    # "extend_add" also holds the one-pass assembly (zeroing, original entries and
    # extend-add in one launch per level; "memset" and "init_a" are then empty)
    KINDS = ("memset", "init_a", "extend_add", "small_fronts", "panel_trsm", "update",
             "diag_chol", "diag_inverse", "panel_split", "update_tc", "blk_diag", "blk_panel")

    def profile(self, val_dev_ptr=None):
        """Per-kernel-kind timing of one extra factorization (no graph)."""
        ms = np.zeros(16); nl = np.zeros(16, dtype=np.int64); fl = np.zeros(12)
        rc = load().sylver_gb300_profile_factor(self.fkeep, val_dev_ptr, _p(ms), _p(nl), _p(fl))
        if rc != 0:
            raise RuntimeError(f"profile failed: {rc}")
        return {k: dict(ms=float(ms[i]), launches=int(nl[i]), flops=float(fl[i]))
                for i, k in enumerate(self.KINDS)}

    def profile_levels(self, val_dev_ptr=None):
        """Per-level factorization time (ms) of one extra, launch-by-launch
        factorization (Cholesky), leaves first."""
        ml = np.zeros(256)
        k = load().sylver_gb300_profile_levels(self.fkeep, val_dev_ptr, _p(ml), 256)
        if k < 0:
            raise RuntimeError(f"profile_levels failed: {k}")
        return ml[:k]

    SOLVE_KINDS = ("small_fwd", "small_bwd", "gather_fwd", "gather_bwd", "scatter_fwd",
                   "scatter_bwd", "diag_fwd", "rows_fwd", "rows_bwd", "diag_bwd", "cb_bwd",
                   "cb_fwd", "unused", "chain_fwd", "chain_bwd")

    def profile_solve(self, nrhs=16):
        """Per-kernel-kind timing of one forward + backward sweep (no graph)."""
        ms = np.zeros(16); nl = np.zeros(16, dtype=np.int64)
        rc = load().sylver_gb300_profile_solve(self.fkeep, int(nrhs), _p(ms), _p(nl))
        if rc != 0:
            raise RuntimeError(f"profile_solve failed: {rc}")
        return {k: dict(ms=float(ms[i]), launches=int(nl[i])) for i, k in enumerate(self.SOLVE_KINDS)}

    def fronts(self):
        """Per-front (m, n, nelim) of an LDL^T factor, postorder."""
        nn = self.analysis.symbolic()["nnodes"]
        m = np.zeros(max(nn, 1), np.int32); n = np.zeros_like(m); ne = np.zeros_like(m)
        k = load().sylver_gb300_fkeep_fronts(self.fkeep, _p(m), _p(n), _p(ne))
        return m[:max(k, 0)], n[:max(k, 0)], ne[:max(k, 0)]

    def diag(self, n):
        d = np.zeros(2 * max(n, 1), dtype=np.float64)
        piv = np.zeros(max(n, 1), dtype=np.int32)
        k = load().sylver_gb300_fkeep_diag(self.fkeep, _p(d), _p(piv))
        return d[:2 * max(k, 0)], piv[:max(k, 0)]

    def __del__(self):
        if getattr(self, "fkeep", None) and _lib is not None and self.fkeep:
            _lib.spldlt_free_fkeep(ctypes.byref(self.fkeep))


class SeamTree:
    """The reference's internal C++ seam, driven as the Fortran factor_core
    and solve drive it (src/spldlt_factorize_mod.F90:542-550, :901-1060):
    spldlt_create_symbolic_tree from SPRAL-layout arrays (1-based, pivot
    order), spldlt_create_numeric_tree[_posdef]_dbl with an optional scaling
    vector indexed by the tree's variables, and spldlt_tree_solve_*_dbl on x in
    pivot order."""

    def __init__(self, sym, posdef, aval, scaling=None, u=0.01, small=1e-20, action=True):
        lib = load()
        self.posdef = bool(posdef)
        self._arr = {k: np.ascontiguousarray(sym[k]) for k in
                     ("sptr", "sparent", "rptr", "rlist", "nptr", "nlist")}
        a = self._arr
        self.n, nn = int(sym["n"]), int(sym["nnodes"])
        self.st = lib.spldlt_create_symbolic_tree(
            None, self.n, nn, _p(a["sptr"].astype(np.int32)), _p(a["sparent"].astype(np.int32)),
            _p(a["rptr"].astype(np.int64)), _p(a["rlist"].astype(np.int32)),
            _p(a["nptr"].astype(np.int64)), _p(a["nlist"].astype(np.int64)), 0, None, None,
            None, None)
        self._aval = np.ascontiguousarray(aval, dtype=np.float64)
        self._scaling = None if scaling is None else np.ascontiguousarray(scaling, np.float64)
        o = OptionsC(print_level=0, action=bool(action), small=float(small), u=float(u),
                     multiplier=1.1, small_subtree_threshold=4000000, nb=256, pivot_method=2,
                     failed_pivot_method=1, cpu_topology=1)
        self.inform = InformC()
        sc = _p(self._scaling) if self._scaling is not None else None
        if self.posdef:
            self.tree = lib.spldlt_create_numeric_tree_posdef_dbl(
                None, self.st, _p(self._aval), sc, None, ctypes.byref(o),
                ctypes.byref(self.inform))
        else:
            self.tree = lib.spldlt_create_numeric_tree_dbl(
                False, None, self.st, _p(self._aval), sc, None, ctypes.byref(o),
                ctypes.byref(self.inform))

    def solve(self, job, x):
        """Tree solve `job` ("fwd", "diag", "bwd", "diag_bwd") in place on x
        (n x nrhs, pivot order); returns the reference flag."""
        lib = load()
        assert x.flags.f_contiguous and x.dtype == np.float64
        nrhs = x.shape[1] if x.ndim == 2 else 1
        if self.posdef and job in ("fwd", "bwd"):
            fn = getattr(lib, f"spldlt_tree_solve_{job}_posdef_dbl")
            return fn(self.tree, nrhs, _p(x), x.shape[0])
        fn = getattr(lib, f"spldlt_tree_solve_{job}_dbl")
        return fn(self.posdef, self.tree, nrhs, _p(x), x.shape[0])

    def close(self):
        lib = load()
        if getattr(self, "tree", None):
            if self.posdef:
                lib.spldlt_destroy_numeric_tree_posdef_dbl(self.tree)
            else:
                lib.spldlt_destroy_numeric_tree_dbl(False, self.tree)
            self.tree = None
        if getattr(self, "st", None):
            lib.spldlt_destroy_symbolic_tree(self.st)
            self.st = None
