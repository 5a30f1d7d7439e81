"""Build libsylver_gb300.so in-tree with nvcc for sm_103a.

Every translation unit under csrc/ is compiled in parallel into
sylver_gb300/_build/, then linked into sylver_gb300/_build/libsylver_gb300.so
with the CUDA runtime linked statically (no torch, no other dependency).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libsylver_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]
# LDL^T kernels: no multiply-add contraction (every fused multiply-add there
# is written out, in an order a CPU restatement can repeat bit for bit)
FILE_FLAGS = {"kernels_ldlt.cu": ["-fmad=false"]}


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src, os.path.abspath(__file__)] + glob.glob(os.path.join(CSRC, "*.hpp")) + \
        glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(HERE, "..", "include", "*.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    srcs = sources()
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, s):
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, *FILE_FLAGS.get(os.path.basename(s), []),
                   *(extra or []), "-c", s, "-o", o]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            errs = []
            for j, f in zip(jobs, futs):
                r = f.result()
                if verbose and (r.stdout or r.stderr):
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    errs.append(" ".join(j) + "\n" + r.stdout + r.stderr)
            if errs:
                raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    if jobs or not os.path.exists(LIB) or force:
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
