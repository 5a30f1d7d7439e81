"""CPU FP64 oracle for the factorize/solve path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the checker.  The product library never imports it.

``oracle.cpp`` restates the reference's multifrontal numeric phase in plain
C++ over BLAS (see its header for the file:line citations).  BLAS comes from
scipy's bundled OpenBLAS through the function pointers scipy exports in
``scipy.linalg.cython_blas`` / ``cython_lapack``, so the same code runs on x86
and aarch64 hosts.
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile oracle.cpp into oracle/_build/liboracle.so (g++, -O3)."""
    src = os.path.join(_HERE, "oracle.cpp")
    if (not force and os.path.exists(_SO)
            and os.path.getmtime(_SO) >= os.path.getmtime(src)):
        return _SO
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _SO + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                           src, "-o", tmp])
    os.replace(tmp, _SO)
    return _SO


def _capsule_ptr(cap) -> int:
    get_name = ctypes.pythonapi.PyCapsule_GetName
    get_name.restype = ctypes.c_char_p
    get_name.argtypes = [ctypes.py_object]
    get_ptr = ctypes.pythonapi.PyCapsule_GetPointer
    get_ptr.restype = ctypes.c_void_p
    get_ptr.argtypes = [ctypes.py_object, ctypes.c_char_p]
    return get_ptr(cap, get_name(cap))


def _blas_lib():
    import scipy
    d = os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs")
    cands = glob.glob(os.path.join(d, "*openblas*"))
    return ctypes.CDLL(cands[0]) if cands else None


def set_threads(k: int) -> bool:
    """Set the OpenBLAS thread count used by the oracle; False if unknown."""
    lib = _blas_lib()
    if lib is None:
        return False
    for name in ("scipy_openblas_set_num_threads", "openblas_set_num_threads",
                 "scipy_openblas_set_num_threads64_"):
        if hasattr(lib, name):
            getattr(lib, name)(ctypes.c_int(int(k)))
            return True
    return False


def load():
    global _lib
    if _lib is not None:
        return _lib
    lib = ctypes.CDLL(build())
    import scipy.linalg.cython_blas as cb
    import scipy.linalg.cython_lapack as cl
    lib.oracle_set_blas.argtypes = [ctypes.c_void_p] * 4
    lib.oracle_set_blas(_capsule_ptr(cb.__pyx_capi__["dgemm"]),
                        _capsule_ptr(cb.__pyx_capi__["dtrsm"]),
                        _capsule_ptr(cb.__pyx_capi__["dsyrk"]),
                        _capsule_ptr(cl.__pyx_capi__["dpotrf"]))
    P = ctypes.c_void_p
    lib.oracle_factor.restype = P
    lib.oracle_factor.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P,
                                  P, P, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                  ctypes.c_int, P]
    lib.oracle_solve.restype = ctypes.c_int
    lib.oracle_solve.argtypes = [P, ctypes.c_int, ctypes.c_int, P, ctypes.c_int]
    lib.oracle_free.argtypes = [P]
    lib.oracle_set_inplace.argtypes = [ctypes.c_int]
    lib.oracle_front.restype = ctypes.c_int
    lib.oracle_front.argtypes = [P, ctypes.c_int, P, P, P, P]
    _lib = lib
    return lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class OracleFactor:
    """FP64 multifrontal factorization of one matrix on the CPU."""

    STAT_NAMES = ("flag", "num_neg", "num_zero", "num_two", "num_delay", "maxfront",
                  "not_first_pass", "not_second_pass", "matrix_rank")

    def __init__(self, posdef, symb, val, u=0.01, small=1e-20, action=True, tpp_cols=0,
                 inplace=False):
        """symb: dict with n, nnodes, sptr, sparent, rptr, rlist, nptr, nlist,
        perm (all 1-based, reference layout).  LDL^T: a-posteriori pivoting in
        blocks of 32 then threshold partial pivoting on the failed columns;
        fronts with at most tpp_cols fully-summed columns use threshold
        partial pivoting only.  inplace=True runs the block steps in the
        reference's own layout (failed columns left in place until
        permute_failed), a check of the default layout."""
        lib = load()
        self._keep = {k: np.ascontiguousarray(v) for k, v in symb.items()
                      if isinstance(v, np.ndarray)}
        k = self._keep
        self.n = int(symb["n"])
        self.posdef = bool(posdef)
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        st = np.zeros(9, dtype=np.int32)
        lib.oracle_set_inplace(int(bool(inplace)))
        self.h = lib.oracle_factor(
            int(posdef), self.n, int(symb["nnodes"]),
            _p(k["sptr"].astype(np.int32)) if k["sptr"].dtype != np.int32 else _p(k["sptr"]),
            _p(k["sparent"]), _p(k["rptr"]), _p(k["rlist"]), _p(k["nptr"]),
            _p(k["nlist"]), _p(k["perm"]), _p(self.val), float(u), float(small),
            int(action), int(tpp_cols), _p(st))
        lib.oracle_set_inplace(0)
        self.stats = dict(zip(self.STAT_NAMES, (int(v) for v in st)))
        self.flag = self.stats["flag"]

    def solve(self, b, job=0):
        x = np.array(b, dtype=np.float64, order="F", copy=True)
        if x.ndim == 1:
            x = x.reshape(-1, 1, order="F")
        rc = load().oracle_solve(self.h, int(job), x.shape[1], _p(x), x.shape[0])
        if rc != 0:
            raise RuntimeError("oracle solve failed")
        return x

    def front(self, s):
        mn = np.zeros(3, dtype=np.int32)
        load().oracle_front(self.h, int(s), _p(mn), None, None, None)
        m, n, ne = (int(v) for v in mn)
        a = np.zeros((m, m), dtype=np.float64, order="F")
        d = np.zeros(max(2 * n, 1), dtype=np.float64)
        var = np.zeros(m, dtype=np.int32)
        load().oracle_front(self.h, int(s), _p(mn), _p(a), _p(d), _p(var))
        return dict(m=m, n=n, nelim=ne, a=a, d=d[:2 * n], var=var)

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _lib is not None:
            _lib.oracle_free(h)
            self.h = None
