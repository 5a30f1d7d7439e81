// Allocation-free forward tree solve.
//
// Some callers cannot let a library call cudaMalloc: applications whose own
// pool allocator owns the whole device-memory budget, and latency-sensitive
// code that must not risk the device-wide synchronisation cudaMalloc/cudaFree
// may cause while other streams are busy.  For them this file exports one
// entry point that performs the forward solve of an existing factorization
// (the same operation as spldlt_tree_solve_fwd_dbl, on device data) with its
// only scratch space -- the per-front right-hand-side slabs of the level
// sweep -- in a file-scope __device__ array instead of allocated memory.
//
//  * Limit: one level needs (sum of the level's front rows) x min(nrhs, 32)
//    doubles of slab space; more than NOALLOC_SCRATCH_DOUBLES (2,097,152
//    doubles = 16 MiB) is rejected with SYLVER_ERROR_X_SIZE.  The array is
//    part of the library image: every GPU that loads the library holds it
//    until the process exits.
//  * Set-up: the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current and caches it.  Every
//    call waits for its stream before returning, so the entry point is not
//    for use while that stream is being captured.
//  * Device: the factorization lives on the library's device.  The call is
//    refused (SYLVER_ERROR_CALL_SEQUENCE) when another device is current or
//    the caller's stream belongs to another device, before anything runs.
//  * Sharing: every call uses the same array.  The kernel fully rewrites the
//    slab rows it reads (zeroing the rows it accumulates into), so stale
//    contents from an earlier call never leak into a result, but two calls
//    whose work overlaps on the GPU (different streams, or different host
//    threads) race on the array and give wrong answers.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "../../include/sylver_gb300.h"
#include "ldlt.hpp"
#include "numeric.hpp"

namespace sylver_gb300 {

constexpr size_t NOALLOC_SCRATCH_DOUBLES = size_t(1) << 21;
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

namespace {
constexpr int kMaxDevices = 64;
// per-device address cache; two host threads may race on the first lookup,
// both store the same address
std::atomic<double*> g_scratch_addr[kMaxDevices];
}  // namespace

// Device address of the static scratch on the current device (set-up on the
// first call per device).
static double* noalloc_scratch_ptr(int* err) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    *err = SYLVER_ERROR_CUDA_UNKNOWN;
    return nullptr;
  }
  double* cached = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!cached) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      *err = SYLVER_ERROR_CUDA_UNKNOWN;
      return nullptr;
    }
    cached = static_cast<double*>(p);
    g_scratch_addr[dev].store(cached, std::memory_order_release);
  }
  return cached;
}

}  // namespace sylver_gb300

using namespace sylver_gb300;

extern "C" int spldlt_tree_solve_fwd_noalloc_dbl(bool posdef, void const* tree, int nrhs,
                                                 double* x_dev, int ldx, void* stream) {
  const FKeep* fk = static_cast<const FKeep*>(tree);
  if (!fk || !fk->ak) return SYLVER_ERROR_CALL_SEQUENCE;
  if (fk->flag < 0) return SYLVER_ERROR_CALL_SEQUENCE;
  if (fk->posdef != posdef) return SYLVER_ERROR_CALL_SEQUENCE;
  if (fk->precision != SYLVER_GB300_FP64) return SYLVER_ERROR_UNIMPLEMENTED;
  const int n = fk->ak->n;
  if (nrhs < 1 || ldx < n || !x_dev) return SYLVER_ERROR_X_SIZE;
  if (n == 0) return SYLVER_SUCCESS;
  // descriptors of the factorization (device memory owned by the tree)
  const FrontDesc* fr;
  const int64_t* scr;
  const int* rows;
  int64_t scratch_rows;
  if (fk->ldlt) {
    if (!ldlt_solve_tables(*fk, &fr, &scr, &rows, &scratch_rows)) return SYLVER_ERROR_CALL_SEQUENCE;
  } else {
    fr = fk->dfr.as<FrontDesc>();
    scr = fk->dscr.as<int64_t>();
    rows = fk->rlist0.as<int>();
    scratch_rows = fk->scratch_rows;
  }
  const int chunk = nrhs < 32 ? nrhs : 32;
  if ((size_t)scratch_rows * (size_t)chunk > NOALLOC_SCRATCH_DOUBLES) return SYLVER_ERROR_X_SIZE;
  // the factorization's device memory belongs to the library's device: the
  // current device and the caller's stream must be that device's
  const int lib_dev = Runtime::get().device;
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess || cur != lib_dev) return SYLVER_ERROR_CALL_SEQUENCE;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : Runtime::get().stream;
  if (stream) {
    int sdev = -1;
    if (cudaStreamGetDevice(s, &sdev) != cudaSuccess || sdev != lib_dev)
      return SYLVER_ERROR_CALL_SEQUENCE;
  }
  int err = 0;
  double* scratch = noalloc_scratch_ptr(&err);
  if (!scratch) return err;
  // clear an error left by earlier work so that the check after the launches
  // sees only this call's
  cudaGetLastError();
  try {
    const double* arena = fk->arena.as<double>();
    for (int r0 = 0; r0 < nrhs; r0 += 32) {
      const int nr = nrhs - r0 < 32 ? nrhs - r0 : 32;
      double* xr = x_dev + (int64_t)r0 * ldx;
      // one CTA per front and level; ldx is the column stride of x
      for (const Level& L : fk->levels)
        launch_solve_fwd<double, double>(arena, fr + L.f0, L.f1 - L.f0, rows, xr, ldx, nr,
                                         scratch, scr + L.f0, !posdef, s);
    }
    if (cudaGetLastError() != cudaSuccess) return SYLVER_ERROR_CUDA_UNKNOWN;
    if (cudaStreamSynchronize(s) != cudaSuccess) return SYLVER_ERROR_CUDA_UNKNOWN;
  } catch (const std::exception&) {
    return SYLVER_ERROR_CUDA_UNKNOWN;
  }
  return SYLVER_SUCCESS;
}
