// Level-batched triangular solves, permutation, FP64 residual and norms for
// iterative refinement.
//
// Reference behaviour replaced:
//   NumericTreePosdef::solve_fwd / solve_bwd   src/NumericTreePosdef.hxx:357-450
//   NumericTree::solve_fwd / solve_diag_bwd     src/NumericTree.hxx:408-520
//   permute + scale wrapper                     src/spldlt_factorize_mod.F90:901-1060
//   backward error (driver)                     drivers/spldlt_test.F90:216-267
//
// One CTA handles one front of a level.  The front's right-hand-side rows are
// gathered into a per-front scratch slab (m x nrhs), processed in 32-column
// blocks (warp 0 solves the diagonal block with shuffles, all warps apply the
// off-diagonal block), and scattered back; rows below the pivots go to
// ancestors with atomics because sibling fronts of a level share them.
#include "device.hpp"

namespace sylver_gb300 {

namespace {

constexpr int SB = 32;      // column block
constexpr int MAXR = 32;    // right-hand sides per launch
constexpr int RC = 8;       // right-hand sides per register chunk
constexpr int GB = 8;       // gather/scatter elements in flight per thread
// dynamic shared memory of the small-front triangle kernel (pivot rows of the
// right-hand sides and their destinations)
constexpr size_t TRI_SMEM = 96 * 1024;
// right-hand sides per pass of the contribution-row kernels: 4 for a few,
// else 16 (FP32) / 8 (FP64), more in several passes
template <typename ACC> constexpr int RQ_MID = sizeof(ACC) == 8 ? 8 : 16;

template <typename T> __device__ __forceinline__ void aadd(T* p, T v) { atomicAdd(p, v); }

// The large fronts' pivot rows are solved in 256-column block steps.  FP32:
// one dataflow launch per level and direction (k_chain, below) whose tasks
// hand each step to the next through counters.  FP64: one launch per step
// with programmatic dependent launch (pdl_trigger / pdl_wait): a step lets
// the next one launch at once, and its CTAs stage the factor data they need
// (which no step writes) before they wait for the previous step's grid.

template <typename T, typename ACC>
__global__ void __launch_bounds__(256) k_solve_fwd(const T* __restrict__ arena,
                                                   const FrontDesc* __restrict__ fr,
                                                   const int* __restrict__ rlist,
                                                   ACC* __restrict__ x, int n, int nrhs,
                                                   ACC* __restrict__ scratch,
                                                   const int64_t* __restrict__ scr_off,
                                                   bool unit) {
  __shared__ ACC y[SB][MAXR];
  for (int e = threadIdx.x; e < SB * MAXR; e += blockDim.x) (&y[0][0])[e] = ACC(0);
  const FrontDesc f = fr[blockIdx.x];
  const T* L = arena + f.off;
  const int ld = f.ld, m = f.m, nc = f.n;
  const int* rl = rlist + f.rl;
  ACC* xs = scratch + scr_off[blockIdx.x] * nrhs;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // gather in batches of GB elements per thread, all loads in flight
  for (int base = 0; base < m * nrhs; base += GB * 256) {
    ACC v[GB];
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u, i = idx % m, r = idx / m;
      v[u] = (idx < m * nrhs && i < nc) ? x[(int64_t)r * n + rl[i]] : ACC(0);
    }
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u;
      if (idx < m * nrhs) xs[idx] = v[u];
    }
  }
  __shared__ ACC Ld[SB][SB + 1];  // Ld[k][i] = L(c0 + i, c0 + k)
  __shared__ ACC rdg[SB];         // 1 / L(c0 + k, c0 + k)
  const int nwarps = blockDim.x >> 5;
  __syncthreads();
  for (int c0 = 0; c0 < nc; c0 += SB) {
    const int bw = min(SB, nc - c0);
    {
      ACC lv[SB * SB / 256];
#pragma unroll
      for (int u = 0; u < SB * SB / 256; ++u) {
        const int e = tid + 256 * u, i = e % SB, k = e / SB;
        lv[u] = (i < bw && k < bw) ? (ACC)L[(int64_t)(c0 + k) * ld + c0 + i] : ACC(0);
      }
#pragma unroll
      for (int u = 0; u < SB * SB / 256; ++u) {
        const int e = tid + 256 * u;
        Ld[e / SB][e % SB] = lv[u];
        if (e % SB == e / SB) rdg[e % SB] = (e % SB < bw && !unit) ? ACC(1) / lv[u] : ACC(1);
      }
    }
    __syncthreads();
    // diagonal block: one right-hand side per warp at a time
    for (int r = warp; r < nrhs; r += nwarps) {
      ACC v = (lane < bw) ? xs[(int64_t)r * m + c0 + lane] : ACC(0);
      __syncwarp();  // converged before the shuffle chain
      for (int kk = 0; kk < bw; ++kk) {
        const ACC vk = __shfl_sync(0xffffffffu, v, kk) * rdg[kk];
        if (lane == kk) v = vk;
        if (lane > kk && lane < bw) v -= Ld[kk][lane] * vk;
      }
      if (lane < bw) {
        xs[(int64_t)r * m + c0 + lane] = v;
        y[lane][r] = v;
      }
    }
    __syncthreads();
    const int c1 = c0 + bw;
    for (int i = c1 + tid; i < m; i += blockDim.x) {
      ACC lv[SB];
#pragma unroll
      for (int kk = 0; kk < SB; ++kk) lv[kk] = (kk < bw) ? (ACC)L[(int64_t)(c0 + kk) * ld + i] : ACC(0);
      for (int r0 = 0; r0 < nrhs; r0 += RC) {
        ACC acc[RC], xo[RC];
#pragma unroll
        for (int q = 0; q < RC; ++q) {
          acc[q] = ACC(0);
          xo[q] = (r0 + q < nrhs) ? xs[(int64_t)(r0 + q) * m + i] : ACC(0);
        }
#pragma unroll
        for (int kk = 0; kk < SB; ++kk) {
#pragma unroll
          for (int q = 0; q < RC; ++q) acc[q] += lv[kk] * y[kk][min(r0 + q, MAXR - 1)];
        }
#pragma unroll
        for (int q = 0; q < RC; ++q)
          if (r0 + q < nrhs) xs[(int64_t)(r0 + q) * m + i] = xo[q] - acc[q];
      }
    }
    __syncthreads();
  }
  for (int base = 0; base < m * nrhs; base += GB * 256) {
    ACC v[GB];
    int dsti[GB];
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u, i = idx % m;
      v[u] = idx < m * nrhs ? xs[idx] : ACC(0);
      dsti[u] = idx < m * nrhs ? rl[i] : 0;
    }
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u, i = idx % m, r = idx / m;
      if (idx >= m * nrhs) break;
      ACC* dst = x + (int64_t)r * n + dsti[u];
      if (i < nc) *dst = v[u];
      else aadd(dst, v[u]);
    }
  }
}

// Small fronts, pivot rows only.  The front's n fully-summed rows of the
// right-hand sides (ys[r*n + i], r < nrhs) and its row list stay in shared
// memory from the gather to the write-back.
//   forward   y = L11^-1 x(pivots), written back to x; the contribution rows
//             receive -L21 y afterwards from k_rect_fwd, which reads y there;
//   backward  z = L11^-T (x(pivots) - t), where t = L21^T x(contribution
//             rows) was accumulated beforehand by k_rect_bwd into tacc (laid
//             out like x); the gather takes t and clears it.
// Column blocks of 32: the warps solve the diagonal block with shuffles, two
// right-hand sides interleaved per warp; the rest of the triangle is updated
// (forward) or reduced (backward) from 32-row tiles of L staged in shared
// memory, thread (row or column = lane, right-hand sides warp + 8j).
template <typename T, typename ACC, bool BWD>
__global__ void __launch_bounds__(256) k_tri(const T* __restrict__ arena,
                                             const FrontDesc* __restrict__ fr,
                                             const int* __restrict__ rlist, ACC* __restrict__ x,
                                             ACC* __restrict__ tacc, int n, int nrhs,
                                             bool unit) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ ACC Ld[SB][SB + 1];  // Ld[k][i] = L(c0 + i, c0 + k)
  __shared__ ACC Lr[SB][SB + 1];  // backward: Lr[ii][k] = L(r0 + ii, c0 + k)
  __shared__ ACC tt[SB][MAXR + 1];  // backward: the block's reduction over rows [c1, nc)
  __shared__ ACC rdg[SB];         // 1 / L(c0 + k, c0 + k)
  const FrontDesc f = fr[blockIdx.x];
  const T* L = arena + f.off;
  const int ld = f.ld, nc = f.n, mr = nc * nrhs;
  ACC* ys = reinterpret_cast<ACC*>(dsm);
  int* rls = reinterpret_cast<int*>(ys + mr);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < nc; i += 256) rls[i] = rlist[f.rl + i];
  __syncthreads();
  for (int base = 0; base < mr; base += GB * 256) {
    // every load of the batch issued before the first store
    ACC v[GB], tv[GB];
    int64_t gi[GB];
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u;
      gi[u] = idx < mr ? (int64_t)(idx / nc) * n + rls[idx % nc] : -1;
      v[u] = gi[u] >= 0 ? x[gi[u]] : ACC(0);
      tv[u] = (BWD && gi[u] >= 0) ? tacc[gi[u]] : ACC(0);
    }
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u;
      if (idx < mr) ys[idx] = v[u] - tv[u];
      if (BWD && gi[u] >= 0) tacc[gi[u]] = ACC(0);
    }
  }
  __syncthreads();
  const int nblk = (nc + SB - 1) / SB;
  for (int bi = 0; bi < nblk; ++bi) {
    const int b = BWD ? nblk - 1 - bi : bi;
    const int c0 = b * SB, bw = min(SB, nc - c0), c1 = c0 + bw;
    if (BWD) {
      // tt[k][r] = sum_{i in [c1, nc)} L(i, c0 + k) z(i, r): thread (k =
      // lane, right-hand sides warp + 8j)
      ACC acc[MAXR / 8];
#pragma unroll
      for (int j = 0; j < MAXR / 8; ++j) acc[j] = ACC(0);
      for (int r0 = c1; r0 < nc; r0 += SB) {
        const int nrow = min(SB, nc - r0);
#pragma unroll
        for (int u = 0; u < SB * SB / 256; ++u) {
          const int e = tid + 256 * u, ii = e % SB, k = e / SB;
          Lr[ii][k] = (ii < nrow && k < bw) ? (ACC)L[(int64_t)(c0 + k) * ld + r0 + ii] : ACC(0);
        }
        __syncthreads();
        for (int ii = 0; ii < nrow; ++ii) {
          const ACC l = Lr[ii][lane];
#pragma unroll
          for (int j = 0; j < MAXR / 8; ++j) {
            const int r = warp + 8 * j;
            if (r < nrhs) acc[j] += l * ys[r * nc + r0 + ii];
          }
        }
        __syncthreads();
      }
#pragma unroll
      for (int j = 0; j < MAXR / 8; ++j) tt[lane][warp + 8 * j] = acc[j];
    }
    {
      ACC lv[SB * SB / 256];
#pragma unroll
      for (int u = 0; u < SB * SB / 256; ++u) {
        const int e = tid + 256 * u, i = e % SB, k = e / SB;
        lv[u] = (i < bw && k < bw) ? (ACC)L[(int64_t)(c0 + k) * ld + c0 + i] : ACC(0);
      }
#pragma unroll
      for (int u = 0; u < SB * SB / 256; ++u) {
        const int e = tid + 256 * u;
        Ld[e / SB][e % SB] = lv[u];
        if (e % SB == e / SB) rdg[e % SB] = (e % SB < bw && !unit) ? ACC(1) / lv[u] : ACC(1);
      }
    }
    __syncthreads();
    // diagonal block: right-hand sides r and r + 8 per warp, interleaved
    for (int r = warp; r < nrhs; r += 16) {
      const int r2 = r + 8;
      const bool two = r2 < nrhs;
      ACC v = ACC(0), w = ACC(0);
      if (lane < bw) {
        v = ys[r * nc + c0 + lane];
        if (two) w = ys[r2 * nc + c0 + lane];
        if (BWD) {
          v -= tt[lane][r];
          if (two) w -= tt[lane][r2];
        }
      }
      __syncwarp();  // converged before the shuffle chain
      if (!BWD) {
        for (int kk = 0; kk < bw; ++kk) {
          const ACC vk = __shfl_sync(0xffffffffu, v, kk) * rdg[kk];
          const ACC wk = __shfl_sync(0xffffffffu, w, kk) * rdg[kk];
          if (lane == kk) {
            v = vk;
            w = wk;
          }
          if (lane > kk && lane < bw) {
            const ACC l = Ld[kk][lane];
            v -= l * vk;
            w -= l * wk;
          }
        }
      } else {
        for (int kk = bw - 1; kk >= 0; --kk) {
          if (lane == kk) {
            v = v * rdg[kk];
            w = w * rdg[kk];
          }
          const ACC zk = __shfl_sync(0xffffffffu, v, kk);
          const ACC zw = __shfl_sync(0xffffffffu, w, kk);
          if (lane < kk) {
            const ACC l = Ld[lane][kk];
            v -= l * zk;
            w -= l * zw;
          }
        }
      }
      if (lane < bw) {
        ys[r * nc + c0 + lane] = v;
        if (two) ys[r2 * nc + c0 + lane] = w;
      }
    }
    __syncthreads();
    if (!BWD) {
      // rows [c1, nc) of the triangle in 32-row tiles: thread (row ii = lane,
      // right-hand sides warp + 8j) subtracts L(r0 + ii, block) y(block)
      for (int r0 = c1; r0 < nc; r0 += SB) {
        const int nrow = min(SB, nc - r0);
#pragma unroll
        for (int u = 0; u < SB * SB / 256; ++u) {
          const int e = tid + 256 * u, ii = e % SB, k = e / SB;
          Lr[ii][k] = (ii < nrow && k < bw) ? (ACC)L[(int64_t)(c0 + k) * ld + r0 + ii] : ACC(0);
        }
        __syncthreads();
        ACC acc[MAXR / 8];
#pragma unroll
        for (int j = 0; j < MAXR / 8; ++j) acc[j] = ACC(0);
        for (int k = 0; k < bw; ++k) {
          const ACC l = Lr[lane][k];
#pragma unroll
          for (int j = 0; j < MAXR / 8; ++j) {
            const int r = warp + 8 * j;
            if (r < nrhs) acc[j] += l * ys[r * nc + c0 + k];
          }
        }
        if (lane < nrow)
#pragma unroll
          for (int j = 0; j < MAXR / 8; ++j) {
            const int r = warp + 8 * j;
            if (r < nrhs) ys[r * nc + r0 + lane] -= acc[j];
          }
        __syncthreads();
      }
    }
  }
  for (int base = 0; base < mr; base += 256) {
    const int idx = base + tid;
    if (idx < mr) x[(int64_t)(idx / nc) * n + rls[idx % nc]] = ys[idx];
  }
}

template <typename ACC>
__global__ void k_permute_in(const double* __restrict__ x, int ldx, ACC* __restrict__ xp,
                             const int* __restrict__ perm, const double* __restrict__ scale,
                             int n, int nrhs) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * nrhs) return;
  int i = (int)(idx % n), r = (int)(idx / n);
  double v = x[(int64_t)r * ldx + i];
  if (scale) v *= scale[i];
  xp[(int64_t)r * n + perm[i]] = (ACC)v;
}

template <typename ACC>
__global__ void k_permute_out(const ACC* __restrict__ xp, const int* __restrict__ perm,
                              const double* __restrict__ scale, double* __restrict__ x, int ldx,
                              int n, int nrhs, bool add) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * nrhs) return;
  int i = (int)(idx % n), r = (int)(idx / n);
  double v = (double)xp[(int64_t)r * n + perm[i]];
  if (scale) v *= scale[i];
  double* d = x + (int64_t)r * ldx + i;
  *d = add ? *d + v : v;
}

__global__ void k_scale_vals(double* __restrict__ val, const int* __restrict__ row,
                             const int* __restrict__ col, const double* __restrict__ scale,
                             int64_t count) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  const int r = row[k];
  if (r < 0) return;
  val[k] = (scale[r] * val[k]) * scale[col[k]];
}

__global__ void __launch_bounds__(128) k_residual(const int64_t* __restrict__ rowptr,
                                                  const int* __restrict__ col,
                                                  const double* __restrict__ a, int n,
                                                  const double* __restrict__ x, int ldx,
                                                  const double* __restrict__ b, int ldb,
                                                  double* __restrict__ res, int nrhs) {
  // one row per thread, up to 16 right-hand sides per pass; the row's
  // entries are taken four at a time so that 64 loads of x are in flight
  constexpr int RR = 16;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t p0 = rowptr[i], p1 = rowptr[i + 1];
  for (int r0 = 0; r0 < nrhs; r0 += RR) {
    double acc[RR];
#pragma unroll
    for (int q = 0; q < RR; ++q) acc[q] = 0.0;
    for (int64_t p = p0; p < p1; p += 4) {
      double v[4];
      int j[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const bool ok = p + u < p1;
        v[u] = ok ? a[p + u] : 0.0;
        j[u] = ok ? col[p + u] : col[p0];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int q = 0; q < RR; ++q)
          if (r0 + q < nrhs) acc[q] = fma(v[u], x[(int64_t)(r0 + q) * ldx + j[u]], acc[q]);
    }
#pragma unroll
    for (int q = 0; q < RR; ++q)
      if (r0 + q < nrhs)
        res[(int64_t)(r0 + q) * n + i] = b[(int64_t)(r0 + q) * ldb + i] - acc[q];
  }
}

__device__ __forceinline__ void atomic_max_nonneg(double* p, double v) {
  // non-negative doubles order like their bit patterns
  atomicMax(reinterpret_cast<unsigned long long*>(p), (unsigned long long)__double_as_longlong(v));
}

__global__ void __launch_bounds__(256) k_maxnorms(const double* __restrict__ res,
                                                  const double* __restrict__ x, int ldx,
                                                  const double* __restrict__ b, int ldb, int n,
                                                  int nrhs, double* norms) {
  // per right-hand side r = blockIdx.y: max |res|, |x|, |b| over a grid-stride
  // range, reduced in the block before one atomic per value (a few hundred
  // blocks per right-hand side; per-warp atomics on the same three words were
  // the bottleneck)
  __shared__ double red[3][8];
  const int r = blockIdx.y;
  double mr = 0.0, mx = 0.0, mb = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    mr = fmax(mr, fabs(res[(int64_t)r * n + i]));
    mx = fmax(mx, fabs(x[(int64_t)r * ldx + i]));
    mb = fmax(mb, fabs(b[(int64_t)r * ldb + i]));
  }
  for (int o = 16; o > 0; o >>= 1) {
    mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mb = fmax(mb, __shfl_xor_sync(0xffffffffu, mb, o));
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    red[0][warp] = mr;
    red[1][warp] = mx;
    red[2][warp] = mb;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double m = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[threadIdx.x][w]);
    atomic_max_nonneg(&norms[3 * r + threadIdx.x], m);
  }
}

__global__ void k_rownorm(const int64_t* __restrict__ rowptr, const double* __restrict__ a,
                          int n, double* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double s = 0.0;
  if (i < n)
    for (int64_t p = rowptr[i]; p < rowptr[i + 1]; ++p) s += fabs(a[p]);
  for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
  if ((threadIdx.x & 31) == 0) atomic_max_nonneg(out, s);
}

__global__ void k_gather_clean(const double* __restrict__ val, const int64_t* __restrict__ srcptr,
                               const int64_t* __restrict__ src, int64_t nclean,
                               double* __restrict__ cval) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nclean) return;
  double s = 0.0;
  for (int64_t q = srcptr[k]; q < srcptr[k + 1]; ++q) s += val[src[q]];
  cval[k] = s;
}

__global__ void k_gather(const double* __restrict__ c, const int64_t* __restrict__ idx,
                         int64_t count, double* __restrict__ out) {
  int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < count) out[k] = c[idx[k]];
}

__global__ void k_axpy(double* __restrict__ x, int ldx, const double* __restrict__ d, int n,
                       int nrhs) {
  int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)n * nrhs) return;
  int i = (int)(idx % n), r = (int)(idx / n);
  x[(int64_t)r * ldx + i] += d[(int64_t)r * n + i];
}

// ---------------------------------------------------------------------------
// Large fronts: blocked sweeps over the fully-summed rows with explicit
// inverses of the diagonal blocks (computed once per factorization).  The
// pivot rows are gathered into a per-front slab (xs), solved block by block
// (solved rows go to a second slab, ys, so no CTA overwrites what another
// reads in the same step) and scattered back.  Each step is one launch of
// independent tasks; the step kernels use programmatic dependent launch.

constexpr int LB = LSOLVE_BW;

// Gather of the pivot rows of a large front, one row per thread (256 rows
// per task).  The contribution rows are handled by k_rect_fwd / k_rect_bwd
// straight from x; backward, their share of each pivot row (in tacc) is
// taken here and cleared, and both backward accumulators of the front start
// at zero.
template <typename T, typename ACC>
__device__ __forceinline__ void gather_body(const LTask& t, const LsArgs<T, ACC>& a, bool fwd) {
  const FrontDesc f = a.fr[t.f];
  if (a.dfc != nullptr) {
    // dataflow sweep next: its counters (the ticket with the first task) and,
    // backward, the accumulator of the 256-column block holding these rows
    if (t.r0 == 0) {
      const int2 o = a.dfo[t.f];
      for (int e = threadIdx.x; e < o.y; e += blockDim.x) a.dfc[o.x + e] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.dfc[0] = 0;
    if (!fwd) {
      ACC* tb = a.tt + a.ttoff[t.f] + (int64_t)(t.r0 / LSOLVE_BW2) * LSOLVE_BW2 * MAXR;
      for (int e = threadIdx.x; e < LSOLVE_BW2 * MAXR; e += blockDim.x) tb[e] = ACC(0);
    }
  } else if (!fwd && t.r0 == 0) {
    ACC* tf = a.tt + (int64_t)t.f * 2 * LSOLVE_BW2 * MAXR;
    for (int e = threadIdx.x; e < 2 * LSOLVE_BW2 * MAXR; e += blockDim.x) tf[e] = ACC(0);
  }
  const int i = t.r0 + threadIdx.x;
  if (threadIdx.x >= 256 || i >= f.n) return;
  ACC* xs = a.scratch + a.scr_off[t.f] * a.nrhs;
  const int v = a.rlist[f.rl + i];
  ACC val[MAXR];  // every load in flight before the first store
#pragma unroll
  for (int r = 0; r < MAXR; ++r) val[r] = r < a.nrhs ? a.x[(int64_t)r * a.n + v] : ACC(0);
  if (!fwd)
#pragma unroll
    for (int r = 0; r < MAXR; ++r)
      if (r < a.nrhs) {
        ACC* tp = a.tacc + (int64_t)r * a.n + v;
        val[r] -= *tp;
        *tp = ACC(0);
      }
#pragma unroll
  for (int r = 0; r < MAXR; ++r)
    if (r < a.nrhs) xs[(int64_t)r * f.m + i] = val[r];
}

// Scatter of the solved pivot rows (ys) of a large front back to x.
template <typename T, typename ACC>
__device__ __forceinline__ void scatter_body(const LTask& t, const LsArgs<T, ACC>& a, bool fwd) {
  const FrontDesc f = a.fr[t.f];
  const int i = t.r0 + threadIdx.x;
  if (threadIdx.x >= 256 || i >= f.n) return;
  const int v = a.rlist[f.rl + i];
  // the backward sweep with P leaves z in the xs slab
  const ACC* src = (a.pmode && !fwd ? a.scratch : a.ys) + a.scr_off[t.f] * a.nrhs + i;
  ACC val[MAXR];
#pragma unroll
  for (int r = 0; r < MAXR; ++r) val[r] = r < a.nrhs ? src[(int64_t)r * f.m] : ACC(0);
#pragma unroll
  for (int r = 0; r < MAXR; ++r)
    if (r < a.nrhs) a.x[(int64_t)r * a.n + v] = val[r];
}

template <typename T, typename ACC>
__global__ void k_lgather(const LTask* __restrict__ tasks, LsArgs<T, ACC> a, bool fwd) {
  gather_body<T, ACC>(tasks[blockIdx.x], a, fwd);
}

template <typename T, typename ACC>
__global__ void k_lscatter(const LTask* __restrict__ tasks, LsArgs<T, ACC> a, bool fwd) {
  scatter_body<T, ACC>(tasks[blockIdx.x], a, fwd);
}

// X = L^-1 for one diagonal block, thread j computes column j; L is read
// straight from the front (all threads read the same element: broadcast).
template <typename T>
__global__ void __launch_bounds__(LB) k_inv_diag(const T* __restrict__ arena,
                                                 const FrontDesc* __restrict__ fr,
                                                 const LTask* __restrict__ tasks,
                                                 T* __restrict__ inv,
                                                 const int64_t* __restrict__ inv_off, bool unit) {
  __shared__ T Xs[LB][LB + 1];  // Xs[j][i] = X(i, j)
  const LTask t = tasks[blockIdx.x];
  const FrontDesc f = fr[t.f];
  const T* L = arena + f.off;
  const int c0 = t.c0, bw = t.bw, j = threadIdx.x;
  auto l = [&](int i, int k) -> T {  // padded block: identity outside bw
    if (i >= bw || k >= bw) return (i == k) ? T(1) : T(0);
    if (i == k && unit) return T(1);
    return L[(int64_t)(c0 + k) * f.ld + c0 + i];
  };
  for (int i = 0; i < LB; ++i) {
    T acc = (i == j) ? T(1) : T(0);
    if (i > j)
      for (int k = j; k < i; ++k) acc -= l(i, k) * Xs[j][k];
    Xs[j][i] = (i >= j) ? acc / l(i, i) : T(0);
  }
  T* out = inv + inv_off[t.f] + (int64_t)(c0 / LB) * LB * LB;
  __syncthreads();
  for (int e = j; e < LB * LB; e += LB) out[e] = Xs[e / LB][e % LB];
}

// Block steps of SW = LSOLVE_BW2 columns.  Each diagonal block has an
// explicit inverse (built once per factorization from its 64x64 inverses), so
// a step is one parallel mat-vec on the diagonal block plus one update
// (forward) or reduction (backward) of the rows below, spread over many small
// CTAs whose L tiles are TW = 256 columns wide.  (Steps of 512 columns halve
// the number of dependent launches but measured no faster: the wider
// mat-vec takes twice as long and the larger inverses cost more to build.)
constexpr int SW = LSOLVE_BW2;
constexpr int TW = 256;
constexpr int DMV_ROWS = 8;   // rows of the diagonal mat-vec per CTA (32 CTAs per block)
constexpr int BRED_ROWS = LSOLVE_RED_ROWS;  // rows per backward-reduction CTA
template <typename ACC> struct RGn { static constexpr int v = sizeof(ACC) == 8 ? 8 : 16; };
// Row stride of the [k][RG] right-hand-side slabs in shared memory: padded by
// 16 bytes so that the transposing stores (consecutive lanes, consecutive k)
// spread over the banks (4-way instead of 16-way conflicts for FP32) while
// rows stay 16-byte aligned for the vector reads.
template <typename ACC> struct RGP { static constexpr int v = RGn<ACC>::v + 16 / (int)sizeof(ACC); };

// X = inverse of the SW-column diagonal block of a step (column-major, ld SW,
// lower): X_jj = Inv64_j and X_ij = -Inv64_i * sum_{k=j}^{i-1} L_ik X_kj for
// i > j, with 64x64 blocks; identity beyond bw.
template <typename T>
__global__ void __launch_bounds__(256) k_inv_block(const T* __restrict__ arena,
                                                const FrontDesc* __restrict__ fr,
                                                const LTask* __restrict__ tasks,
                                                const T* __restrict__ inv64,
                                                const int64_t* __restrict__ inv_off,
                                                T* __restrict__ inv2,
                                                T* __restrict__ inv2t,
                                                const int64_t* __restrict__ inv2_off) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T* As = reinterpret_cast<T*>(sm_raw);  // As[k*65 + r] = A(r, k)
  T* Bs = As + 64 * 65;                  // Bs[c*65 + k] = B(k, c)
  const LTask t = tasks[blockIdx.x];
  const FrontDesc f = fr[t.f];
  const T* L = arena + f.off;
  const int c0 = t.c0, bw = t.bw, tid = threadIdx.x;
  T* X = inv2 + inv2_off[t.f] + (int64_t)(c0 / SW) * SW * SW;
  const T* I64 = inv64 + inv_off[t.f] + (int64_t)(c0 / LB) * LB * LB;
  const int nb = (bw + LB - 1) / LB;
  for (int e = tid; e < SW * SW; e += blockDim.x) X[e] = T(0);
  __syncthreads();
  for (int j = 0; j < SW / LB; ++j)
    for (int e = tid; e < LB * LB; e += blockDim.x) {
      int i = e % LB, k = e / LB;
      X[(int64_t)(LB * j + k) * SW + LB * j + i] =
          (j < nb) ? I64[(int64_t)j * LB * LB + k * LB + i] : T(i == k ? 1 : 0);
    }
  __syncthreads();
  const int r = tid % LB, cq = tid / LB;  // output row, 16-column quarter
  for (int j = 0; j < nb; ++j)
    for (int i = j + 1; i < nb; ++i) {
      T acc[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) acc[q] = T(0);
      for (int k = j; k < i; ++k) {
        // both tiles read along their stored columns (consecutive threads,
        // consecutive addresses)
        for (int e = tid; e < LB * LB; e += blockDim.x) {
          const int rr = e % LB, kk = e / LB;
          const int grow = LB * i + rr, gcol = LB * k + kk;
          As[kk * 65 + rr] = (grow < bw && gcol < bw) ? L[(int64_t)(c0 + gcol) * f.ld + c0 + grow] : T(0);
        }
        for (int e = tid; e < LB * LB; e += blockDim.x) {
          const int kk = e % LB, rr = e / LB;
          Bs[rr * 65 + kk] = X[(int64_t)(LB * j + rr) * SW + LB * k + kk];  // B(kk, rr) = X_kj
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < LB; ++kk) {
          const T a = As[kk * 65 + r];
#pragma unroll
          for (int q = 0; q < 16; ++q) acc[q] += a * Bs[(cq * 16 + q) * 65 + kk];
        }
        __syncthreads();
      }
      // X_ij = -Inv64_i S
#pragma unroll
      for (int q = 0; q < 16; ++q) Bs[(cq * 16 + q) * 65 + r] = acc[q];
      for (int e = tid; e < LB * LB; e += blockDim.x) {
        int rr = e % LB, kk = e / LB;
        As[kk * 65 + rr] = I64[(int64_t)i * LB * LB + kk * LB + rr];
      }
      __syncthreads();
#pragma unroll
      for (int q = 0; q < 16; ++q) acc[q] = T(0);
#pragma unroll 8
      for (int kk = 0; kk < LB; ++kk) {
        const T a = As[kk * 65 + r];
#pragma unroll
        for (int q = 0; q < 16; ++q) acc[q] += a * Bs[(cq * 16 + q) * 65 + kk];
      }
#pragma unroll
      for (int q = 0; q < 16; ++q) X[(int64_t)(LB * j + cq * 16 + q) * SW + LB * i + r] = -acc[q];
      __syncthreads();
    }
  // transposed copy, XT[k*256 + i] = X(k, i), through 64 x 64 shared tiles
  T* XT = inv2t + inv2_off[t.f] + (int64_t)(c0 / SW) * SW * SW;
  for (int bj = 0; bj < SW / LB; ++bj)
    for (int bi = 0; bi < SW / LB; ++bi) {
      for (int e = tid; e < LB * LB; e += blockDim.x) {
        const int rr = e % LB, kk = e / LB;  // X(LB*bi + rr, LB*bj + kk)
        As[kk * 65 + rr] = X[(int64_t)(LB * bj + kk) * SW + LB * bi + rr];
      }
      __syncthreads();
      for (int e = tid; e < LB * LB; e += blockDim.x) {
        const int kk = e % LB, rr = e / LB;  // XT(LB*bj + kk, LB*bi + rr)
        XT[(int64_t)(LB * bi + rr) * SW + LB * bj + kk] = As[kk * 65 + rr];
      }
      __syncthreads();
    }
}

// P_ib = L_ib X_b (FP32), 64 rows per task: thread (rows 4tr .. 4tr + 3,
// columns 16tc .. 16tc + 15); the inner index in chunks of 32 staged by
// 16-byte copies (columns of L, rows of X from its row-major copy).  X_b is
// lower triangular, so chunk [i0, i0 + 32) adds nothing to columns > i0 + 31.
__global__ void __launch_bounds__(256) k_form_p(const float* __restrict__ arena,
                                                const FrontDesc* __restrict__ fr,
                                                const PTask* __restrict__ tasks,
                                                const float* __restrict__ inv2t,
                                                const int64_t* __restrict__ inv2_off,
                                                float* __restrict__ pmat) {
  __shared__ __align__(16) float As[32][64];   // As[i][r] = L(r0 + r, c0 + i0 + i)
  __shared__ __align__(16) float Bs[32][SW];   // Bs[i][k] = X(i0 + i, k)
  const PTask t = tasks[blockIdx.x];
  const FrontDesc f = fr[t.f];
  const float* L = arena + f.off;
  const float* XT = inv2t + inv2_off[t.f] + (int64_t)(t.c0 / SW) * SW * SW;
  const int tid = threadIdx.x, tr = tid & 15, tc = tid >> 4;
  const int nr = min(64, f.n - t.r0);
  float acc[4][16];
#pragma unroll
  for (int ii = 0; ii < 4; ++ii)
#pragma unroll
    for (int jj = 0; jj < 16; ++jj) acc[ii][jj] = 0.f;
  for (int i0 = 0; i0 < SW; i0 += 32) {
    __syncthreads();  // the previous chunk is no longer read
    for (int e = tid; e < 32 * 16; e += 256) {
      const int i = e / 16, r4 = 4 * (e % 16);
      float* dst = &As[i][r4];
      const float* src = &L[(int64_t)(t.c0 + i0 + i) * f.ld + t.r0 + r4];
      if (r4 + 4 <= nr) {
        cp_async16(dst, src);
      } else {
#pragma unroll
        for (int u = 0; u < 4; ++u) dst[u] = (r4 + u < nr) ? src[u] : 0.f;
      }
    }
    for (int e = tid; e < 32 * (SW / 4); e += 256) {
      const int i = e / (SW / 4), k4 = 4 * (e % (SW / 4));
      cp_async16(&Bs[i][k4], &XT[(int64_t)(i0 + i) * SW + k4]);
    }
    cp_async_wait_all();
    __syncthreads();
    if (16 * tc > i0 + 31) continue;
#pragma unroll 4
    for (int i = 0; i < 32; ++i) {
      const float4 a4 = *reinterpret_cast<const float4*>(&As[i][4 * tr]);
      const float av[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const float4 b4 = *reinterpret_cast<const float4*>(&Bs[i][16 * tc + 4 * m]);
        const float bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
        for (int ii = 0; ii < 4; ++ii)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[ii][4 * m + q] = fmaf(av[ii], bv[q], acc[ii][4 * m + q]);
      }
    }
  }
  float* out = pmat + t.pofs + (t.r0 - t.c1) + 4 * tr;
#pragma unroll
  for (int jj = 0; jj < 16; ++jj) {
    float* o = out + (int64_t)(16 * tc + jj) * t.ldp;
    if (4 * tr + 4 <= nr) {
      *reinterpret_cast<float4*>(o) = make_float4(acc[0][jj], acc[1][jj], acc[2][jj], acc[3][jj]);
    } else {
#pragma unroll
      for (int ii = 0; ii < 4; ++ii)
        if (4 * tr + ii < nr) o[ii] = acc[ii][jj];
    }
  }
}

template <typename ACC> struct Vec4;
template <> struct Vec4<float> {
  using V = float4;
  static constexpr int W = 4;
};
template <> struct Vec4<double> {
  using V = double2;
  static constexpr int W = 2;
};

// Diagonal block of a 256-column step as a product with its explicit
// inverse, DR output rows per task (256 / DR tasks per block), 256 threads:
//   forward   y_b = X v,    v = xs(block)        -> ys(block)
//   backward  z_b = X^T v,  v = xs(block) - tt   -> ys(block)
//             (dataflow sweeps: u_b = X^T xs(block), no accumulator)
// (X^T read from the transposed copy, so both directions read the matrix
// coalesced down a column.)  Thread (row i, k-phase g) sums k = g (mod
// 256 / DR); the phases are reduced through shared memory.  The per-step
// backward launch reads accumulator (c0/256)&1 and clears the other one,
// which the next (lower) block's reduction fills.  The inverse slice is
// staged before the wait for the data earlier steps write.
template <typename T, typename ACC, int DR = DMV_ROWS> constexpr size_t diag_mv_smem() {
  return sizeof(T) * DR * SW +
         sizeof(ACC) * ((256 / DR) * DR * (RGn<ACC>::v + 1) + SW * RGP<ACC>::v);
}
// MODE 0: one launch per step (programmatic dependent launch, two backward
// accumulators per front used in turn); MODE 1: a task of a dataflow sweep
// with the products P_ib = L_ib X_b (no accumulator in the diagonal tasks).
// wait() is called by every thread before the first read of data an earlier
// step wrote; those reads bypass L1 (__ldcg), since in a dataflow sweep the
// writer is another CTA of the same launch.
struct PdlWait {
  __device__ void operator()() const { pdl_wait(); }
};
// MODE 1: where a task's product tile comes from (P's rows start at the first
// row below the block), and whether a backward reduction task also stores
// the z rows it forms
template <typename T> struct PSrc {
  const T* base = nullptr;
  int64_t ld = 0;
  bool writer = false;
};
template <typename T, typename ACC, bool BWD, int DR, int MODE, typename W>
__device__ __forceinline__ void diag_body(const LTask& t, int sub, const LsArgs<T, ACC>& a,
                                          unsigned char* dsm, const W& wait) {
  constexpr int RG = RGn<ACC>::v, RS = RGP<ACC>::v;
  // DR output rows per task; 256 / DR k-phases per row
  constexpr int NG = 256 / DR;
  using V = typename Vec4<ACC>::V;
  constexpr int VW = Vec4<ACC>::W;
  T* Ms = reinterpret_cast<T*>(dsm);  // Ms[(k - klo)*DR + il] = M(i0 + il, k)
  ACC* part = reinterpret_cast<ACC*>(dsm + sizeof(T) * DR * SW);  // [NG][DR][RG + 1]
  ACC* vb = part + NG * DR * (RG + 1);                               // [SW][RG]
  const FrontDesc f = a.fr[t.f];
  const int c0 = t.c0, bw = t.bw, i0 = DR * sub;
  const int tid = threadIdx.x, il = tid % DR, g = tid / DR, i = i0 + il;
  const int64_t m = f.m;
  ACC* xs = a.scratch + a.scr_off[t.f] * a.nrhs;
  ACC* ysl = a.ys + a.scr_off[t.f] * a.nrhs;
  const int64_t moff = a.inv2_off[t.f] + (int64_t)(c0 / SW) * SW * SW;
  const T* M = (BWD ? a.inv2t : a.inv2) + moff;
  ACC* tf = a.tt + (int64_t)t.f * 2 * SW * MAXR;
  ACC* tcur = tf + ((c0 / SW) & 1) * SW * MAXR;
  ACC* tnext = tf + (((c0 / SW) + 1) & 1) * SW * MAXR;
  // entries k of v (and columns of the matrix slice) this task needs
  const int klo = BWD ? i0 : 0, khi = BWD ? bw : min(bw, i0 + DR), nk = khi - klo;
  __syncthreads();  // the previous task's shared data is no longer read
  if (MODE == 0) pdl_trigger();
  if (i0 < bw) {
    // the task's slice of the inverse, one wave of asynchronous copies
    constexpr int E = 16 / (int)sizeof(T), DQ = DR / E;  // 16-byte pieces per column
    for (int e = tid; e < nk * DQ; e += 256) {
      const int rr = E * (e % DQ), k = klo + e / DQ;
      cp_async16(&Ms[(k - klo) * DR + rr], &M[(int64_t)k * SW + i0 + rr]);
    }
  }
  wait();
  // rows beyond the block: nothing to compute (uniform per task)
  for (int rg = 0; rg < (i0 < bw ? a.nrhs : 0); rg += RG) {
    const int nr = min(RG, a.nrhs - rg);
    __syncthreads();
    {
      // all loads of the slab issued before any is used (nk * RG <= 256 NL)
      constexpr int NL = SW * RG / 256;
      ACC v[NL];
#pragma unroll
      for (int u = 0; u < NL; ++u) {
        const int e = tid + 256 * u;
        const int k = klo + e % max(nk, 1), r = e / max(nk, 1);
        v[u] = ACC(0);
        if (e < nk * RG && r < nr) {
          v[u] = __ldcg(&xs[(int64_t)(rg + r) * m + c0 + k]);
          if (BWD && MODE == 0) v[u] -= __ldcg(&tcur[(int64_t)(rg + r) * SW + k]);
        }
      }
#pragma unroll
      for (int u = 0; u < NL; ++u) {
        const int e = tid + 256 * u;
        if (e < nk * RG) vb[(klo + e % nk) * RS + e / nk] = v[u];
      }
    }
    cp_async_wait_all();
    __syncthreads();
    ACC acc[RG];
#pragma unroll
    for (int q = 0; q < RG; ++q) acc[q] = ACC(0);
    if (i < bw) {
      const int k0 = BWD ? i : 0, k1 = BWD ? bw : i + 1;
#pragma unroll 4
      for (int k = k0 + ((g - k0) % NG + NG) % NG; k < k1; k += NG) {
        const ACC l = (ACC)Ms[(k - klo) * DR + il];
        const V* vv = reinterpret_cast<const V*>(vb + k * RS);
#pragma unroll
        for (int q = 0; q < RG / VW; ++q) {
          const V x4 = vv[q];
          if constexpr (VW == 4) {
            acc[4 * q + 0] += l * x4.x;
            acc[4 * q + 1] += l * x4.y;
            acc[4 * q + 2] += l * x4.z;
            acc[4 * q + 3] += l * x4.w;
          } else {
            acc[2 * q + 0] += l * x4.x;
            acc[2 * q + 1] += l * x4.y;
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < RG; ++q) part[(g * DR + il) * (RG + 1) + q] = acc[q];
    __syncthreads();
    for (int e = tid; e < DR * RG; e += 256) {
      const int rr = e % DR, q = e / DR, ii = i0 + rr;
      if (ii < bw && q < nr) {
        ACC sum = ACC(0);
#pragma unroll
        for (int gg = 0; gg < NG; ++gg) sum += part[(gg * DR + rr) * (RG + 1) + q];
        ysl[(int64_t)(rg + q) * m + c0 + ii] = sum;
      }
    }
  }
  if (BWD && MODE == 0)
    for (int e = tid; e < DR * MAXR; e += 256) tnext[(int64_t)(e / DR) * SW + i0 + e % DR] = ACC(0);
}

// Fully-summed rows [r0, r0+32) (< n) below the block: xs_i -= L_i,blk y_blk;
// NT threads, thread (row, column group g of 256 / (NT/32) columns).  The
// 32 x 256 tile of L is staged in shared memory by one wave of asynchronous
// copies; y is read as 16-byte vectors (one broadcast per warp).
template <typename T, typename ACC, int NT> constexpr size_t upd_smem() {
  return sizeof(T) * 32 * TW +
         sizeof(ACC) * ((NT / 32) * 32 * (RGn<ACC>::v + 1) + TW * RGP<ACC>::v);
}
template <typename T, typename ACC, int NT, int MODE, typename W>
__device__ __forceinline__ void upd_body(const LTask& t, const LsArgs<T, ACC>& a,
                                         unsigned char* dsm, const W& wait,
                                         const PSrc<T>& ps = PSrc<T>{}) {
  constexpr int RG = RGn<ACC>::v, RS = RGP<ACC>::v, NGU = NT / 32, KPG = TW / NGU;
  using V = typename Vec4<ACC>::V;
  constexpr int VW = Vec4<ACC>::W;
  T* Lt = reinterpret_cast<T*>(dsm);  // Lt[k*32 + rr] = L(r0 + rr, c0 + k)
  ACC* red = reinterpret_cast<ACC*>(dsm + sizeof(T) * 32 * TW);  // [NGU][32][RG + 1]
  ACC* yb = red + NGU * 32 * (RG + 1);                              // [TW][RG]
  const FrontDesc f = a.fr[t.f];
  const T* L = a.arena + f.off;
  const int tid = threadIdx.x, rr = tid % 32, g = tid / 32;
  ACC* xs = a.scratch + a.scr_off[t.f] * a.nrhs;
  const ACC* ysl = a.ys + a.scr_off[t.f] * a.nrhs;
  const int nrow = min(32, f.n - t.r0);  // fully-summed rows only
  const int cfirst = t.c0, clast = t.c0 + t.bw;
  // the product's tile: L(r0 + rr, c0 + k), or with MODE 1 P(r0 + rr, k)
  const T* tb = MODE == 1 ? ps.base + (t.r0 - cfirst - SW) : L + (int64_t)cfirst * f.ld + t.r0;
  const int64_t tld = MODE == 1 ? ps.ld : (int64_t)f.ld;
  // ... times y_b, or with MODE 1 the block's final x_b
  const ACC* yin = MODE == 1 ? xs : ysl;
  __syncthreads();  // the previous task's shared data is no longer read
  if (MODE == 0) pdl_trigger();
  for (int rg = 0; rg < a.nrhs; rg += RG) {
    const int nr = min(RG, a.nrhs - rg);
    ACC acc[RG];
#pragma unroll
    for (int q = 0; q < RG; ++q) acc[q] = ACC(0);
    // the rows' current values, read as soon as the wait allows (their
    // round trip overlaps the product)
    constexpr int NX = (32 * RG + NT - 1) / NT;
    ACC xold[NX];
    for (int c0 = cfirst; c0 < clast; c0 += TW) {
      const int bw = min(TW, clast - c0);
      __syncthreads();  // the previous block's tiles are no longer read
      // 16-byte pieces of each column (rows t.r0 + r2, r2 a multiple of E:
      // 16-byte aligned, t.r0 being a multiple of 32 past a full block)
      constexpr int E = 16 / (int)sizeof(T), PQ = 32 / E;
      for (int e = tid; e < TW * PQ; e += NT) {
        const int r2 = E * (e % PQ), k = e / PQ;
        T* dst = &Lt[k * 32 + r2];
        const T* src = tb + (int64_t)(c0 - cfirst + k) * tld + r2;
        if (k < bw && r2 + E <= nrow) {
          cp_async16(dst, src);
        } else {
#pragma unroll
          for (int u = 0; u < E; ++u) dst[u] = (k < bw && r2 + u < nrow) ? src[u] : T(0);
        }
      }
      wait();
      if (c0 == cfirst) {
#pragma unroll
        for (int u = 0; u < NX; ++u) {
          const int e = tid + NT * u, r2 = e % 32, q = e / 32;
          xold[u] = (e < 32 * RG && r2 < nrow && q < nr)
                        ? __ldcg(&xs[(int64_t)(rg + q) * f.m + t.r0 + r2]) : ACC(0);
        }
      }
      {
        constexpr int NL = TW * RG / NT;
        ACC v[NL];
#pragma unroll
        for (int u = 0; u < NL; ++u) {
          const int e = tid + NT * u, k = e % TW, r = e / TW;
          v[u] = (k < bw && r < nr) ? __ldcg(&yin[(int64_t)(rg + r) * f.m + c0 + k]) : ACC(0);
        }
#pragma unroll
        for (int u = 0; u < NL; ++u) {
          const int e = tid + NT * u;
          yb[(e % TW) * RS + e / TW] = v[u];
        }
      }
      cp_async_wait_all();
      __syncthreads();
#pragma unroll 8
      for (int kk = 0; kk < KPG; ++kk) {
        const int k = g * KPG + kk;
        const ACC l = (ACC)Lt[k * 32 + rr];
        const V* yv = reinterpret_cast<const V*>(yb + k * RS);
#pragma unroll
        for (int q = 0; q < RG / VW; ++q) {
          const V y4 = yv[q];
          if constexpr (VW == 4) {
            acc[4 * q + 0] += l * y4.x;
            acc[4 * q + 1] += l * y4.y;
            acc[4 * q + 2] += l * y4.z;
            acc[4 * q + 3] += l * y4.w;
          } else {
            acc[2 * q + 0] += l * y4.x;
            acc[2 * q + 1] += l * y4.y;
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < RG; ++q) red[(g * 32 + rr) * (RG + 1) + q] = acc[q];
    __syncthreads();
    // 32 rows x RG sums, spread over all threads
#pragma unroll
    for (int u = 0; u < NX; ++u) {
      const int e = tid + NT * u, r2 = e % 32, q = e / 32, i2 = t.r0 + r2;
      if (e < 32 * RG && r2 < nrow && q < nr) {
        ACC sum = ACC(0);
#pragma unroll
        for (int gg = 0; gg < NGU; ++gg) sum += red[(gg * 32 + r2) * (RG + 1) + q];
        xs[(int64_t)(rg + q) * f.m + i2] = xold[u] - sum;
      }
    }
    __syncthreads();
  }
}

// Fully-summed rows [r0, r0 + BRED_ROWS) (< n) below the block contribute
// tt[k][r] += sum_i L(i, c0+k) z(i, r), k < bw, in 32-row sub-tiles of L
// staged in shared memory by one wave of asynchronous copies; thread (column
// k = tid % 256, row half h), the halves (NT = 512) reduced through shared
// memory.  Every task of a step adds into the same accumulator; the
// contribution rows' share was put into tacc by k_rect_bwd and taken out by
// the gather.
template <typename T, typename ACC> constexpr size_t red_smem() {
  return sizeof(T) * 32 * (TW + 1) + sizeof(ACC) * (TW * (RGn<ACC>::v + 1) + 32 * RGP<ACC>::v);
}
template <typename T, typename ACC, int NT, int MODE, typename W>
__device__ __forceinline__ void red_body(const LTask& t, const LsArgs<T, ACC>& a,
                                         unsigned char* dsm, const W& wait,
                                         const PSrc<T>& ps = PSrc<T>{}) {
  constexpr int RG = RGn<ACC>::v, RS = RGP<ACC>::v, SR = 32, NH = NT / TW;
  using V = typename Vec4<ACC>::V;
  constexpr int VW = Vec4<ACC>::W;
  T* Lt = reinterpret_cast<T*>(dsm);  // Lt[ii*(TW+1) + k] = L(s0 + ii, c0 + k)
  ACC* half = reinterpret_cast<ACC*>(dsm + sizeof(T) * SR * (TW + 1));  // [TW][RG + 1]
  ACC* xt = half + TW * (RG + 1);                                         // [SR][RG]
  const FrontDesc f = a.fr[t.f];
  const T* L = a.arena + f.off;
  const int c0 = t.c0, bw = t.bw, tid = threadIdx.x, k = tid % TW, h = tid / TW;
  ACC* xs = a.scratch + a.scr_off[t.f] * a.nrhs;
  const ACC* ysl = a.ys + a.scr_off[t.f] * a.nrhs;
  // the accumulator of the step block holding columns [c0, c0 + bw)
  ACC* tf = (MODE == 1 ? a.tt + a.ttoff[t.f] + (int64_t)(c0 / SW) * SW * MAXR
                       : a.tt + ((int64_t)t.f * 2 + ((c0 / SW) & 1)) * SW * MAXR) +
            (c0 % SW);
  const int rend = min(t.r0 + (MODE == 1 ? SR : BRED_ROWS), f.n);
  __syncthreads();  // the previous task's shared data is no longer read
  if (MODE == 0) pdl_trigger();
  for (int rg = 0; rg < a.nrhs; rg += RG) {
    const int nr = min(RG, a.nrhs - rg);
    ACC acc[RG];
#pragma unroll
    for (int q = 0; q < RG; ++q) acc[q] = ACC(0);
    for (int s0 = t.r0; s0 < rend; s0 += SR) {
      const int nrow = min(SR, rend - s0);
      __syncthreads();  // the previous sub-tile is no longer read
      for (int e = tid; e < SR * TW; e += NT) {
        const int ii = e % SR, kk = e / SR;
        T* dst = &Lt[ii * (TW + 1) + kk];
        if (ii < nrow && kk < bw)
          cp_async(dst, MODE == 1 ? ps.base + (int64_t)kk * ps.ld + (s0 + ii - c0 - SW)
                                  : &L[(int64_t)(c0 + kk) * f.ld + s0 + ii]);
        else *dst = T(0);
      }
      wait();
      for (int e = tid; e < SR * RG; e += NT) {
        const int ii = e % SR, r = e / SR;
        ACC z = ACC(0);
        if (ii < nrow && r < nr) {
          const int64_t xi = (int64_t)(rg + r) * f.m + s0 + ii;
          z = __ldcg(&ysl[xi]);
          if (MODE == 1) {
            // z = u - t of the row's block (complete: the wait covered it)
            const int row = s0 + ii, jb = row / SW;
            z -= __ldcg(&a.tt[a.ttoff[t.f] + ((int64_t)jb * MAXR + rg + r) * SW + (row - jb * SW)]);
            if (ps.writer) xs[xi] = z;
          }
        }
        xt[ii * RS + r] = z;
      }
      cp_async_wait_all();
      __syncthreads();
#pragma unroll 8
      for (int i2 = 0; i2 < SR / NH; ++i2) {
        const int ii = h * (SR / NH) + i2;
        const ACC l = (ACC)Lt[ii * (TW + 1) + k];
        const V* xv = reinterpret_cast<const V*>(&xt[ii * RS]);
#pragma unroll
        for (int q = 0; q < RG / VW; ++q) {
          const V x4 = xv[q];
          if constexpr (VW == 4) {
            acc[4 * q + 0] += l * x4.x;
            acc[4 * q + 1] += l * x4.y;
            acc[4 * q + 2] += l * x4.z;
            acc[4 * q + 3] += l * x4.w;
          } else {
            acc[2 * q + 0] += l * x4.x;
            acc[2 * q + 1] += l * x4.y;
          }
        }
      }
    }
    if (NH == 2) {
      if (h == 1)
#pragma unroll
        for (int q = 0; q < RG; ++q) half[k * (RG + 1) + q] = acc[q];
      __syncthreads();
    }
    if (h == 0 && k < bw)
#pragma unroll
      for (int q = 0; q < RG; ++q)
        if (q < nr) aadd(&tf[(int64_t)(rg + q) * SW + k], acc[q] + (NH == 2 ? half[k * (RG + 1) + q] : ACC(0)));
    __syncthreads();
  }
}

template <typename T, typename ACC, bool BWD>
__global__ void __launch_bounds__(256) k_diag_mv(const LTask* __restrict__ tasks,
                                                 LsArgs<T, ACC> a) {
  extern __shared__ __align__(16) unsigned char dsm[];
  diag_body<T, ACC, BWD, DMV_ROWS, 0>(tasks[blockIdx.x], blockIdx.y, a, dsm, PdlWait{});
}
template <typename T, typename ACC>
__global__ void __launch_bounds__(512) k_fwd_upd3(const LTask* __restrict__ tasks,
                                                  LsArgs<T, ACC> a) {
  extern __shared__ __align__(16) unsigned char dsm[];
  upd_body<T, ACC, 512, 0>(tasks[blockIdx.x], a, dsm, PdlWait{});
}
template <typename T, typename ACC>
__global__ void __launch_bounds__(512) k_bwd_red3(const LTask* __restrict__ tasks,
                                                  LsArgs<T, ACC> a) {
  extern __shared__ __align__(16) unsigned char dsm[];
  red_body<T, ACC, 512, 0>(tasks[blockIdx.x], a, dsm, PdlWait{});
}

// ---------------------------------------------------------------------------
// Dataflow sweep: the block steps of all large fronts of a level in one
// launch.  Persistent CTAs take tasks in list order through an atomic ticket
// (counter 0); every task's dependencies come earlier in the list, so a CTA
// only ever waits for tasks that running CTAs have already taken, whatever
// the number of CTAs resident.  Critical path per block step: the diagonal
// tasks' counter handoff plus one mat-vec, instead of a kernel launch.
constexpr int DF_SPIN_LIMIT = 1 << 20;  // polls per wait (under a second with the back-off)
constexpr int DF_ROWS = 16;  // output rows per diagonal task (LSOLVE_BW2 / 16 tasks per block)

// counters [w0, w0 + nw) >= need0 and counter w1 (>= 0) >= need1 (nw < 32),
// polled by warp 0, one counter per lane so that all of them cost one round
// trip; gives up (ST_TIMEOUT in *err) after DF_SPIN_LIMIT polls or once
// another wait gave up
struct DfWait {
  const int* cnt;
  unsigned* err;
  int w0, nw, need0, w1, need1;
  __device__ void operator()() const {
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      const int* c = nullptr;
      int need = 0;
      if (lane < nw) {
        c = cnt + w0 + lane;
        need = need0;
      } else if (lane == nw && w1 >= 0) {
        c = cnt + w1;
        need = need1;
      }
      bool done = c == nullptr, all = false, gaveup = false;
      unsigned ns = 32;
      for (int it = 0; it < DF_SPIN_LIMIT; ++it) {
        if (!done) done = *reinterpret_cast<const volatile int*>(c) >= need;
        all = __all_sync(0xffffffffu, done);
        if (all) break;
        if ((it & 63) == 63 && (*reinterpret_cast<volatile unsigned*>(err) & ST_TIMEOUT)) {
          gaveup = true;  // the same value in every lane: one load for the warp
          break;
        }
        __nanosleep(ns);
        if (ns < 256) ns *= 2;
      }
      if (!all && !gaveup && lane == 0) atomicOr(err, ST_TIMEOUT);
      __threadfence();
    }
    __syncthreads();
  }
};

// z = u - t for rows [r0, r0 + 32) of a front's first block (MODE 1
// backward: the blocks below are finished by the reductions that read them)
template <typename T, typename ACC, typename W>
__device__ __forceinline__ void fin_body(const LTask& t, const LsArgs<T, ACC>& a, const W& wait) {
  const FrontDesc f = a.fr[t.f];
  ACC* xs = a.scratch + a.scr_off[t.f] * a.nrhs;
  const ACC* ysl = a.ys + a.scr_off[t.f] * a.nrhs;
  const ACC* tb = a.tt + a.ttoff[t.f];
  const int nrow = min(32, f.n - t.r0);
  wait();
  for (int e = threadIdx.x; e < 32 * a.nrhs; e += blockDim.x) {
    const int ii = e % 32, r = e / 32, row = t.r0 + ii;
    if (ii < nrow) {
      const int64_t xi = (int64_t)r * f.m + row;
      xs[xi] = __ldcg(&ysl[xi]) - __ldcg(&tb[(int64_t)r * SW + row]);
    }
  }
}

template <typename T, typename ACC, bool BWD>
__global__ void __launch_bounds__(256) k_chain(const DfTask* __restrict__ tasks, int ntask,
                                               LsArgs<T, ACC> a, unsigned* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ int s_ti;
  constexpr int DR = DF_ROWS;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_ti = atomicAdd(a.dfc, 1);
    __syncthreads();
    const int ti = s_ti;
    if (ti >= ntask) break;
    const DfTask d = tasks[ti];
    const DfWait w{a.dfc, err, d.w0, d.nw, d.need0, d.w1, d.need1};
    const LTask t{d.f, d.c0, d.bw, d.r0, 0, 0};
    PSrc<T> ps;
    ps.base = a.pmat + d.pofs;
    ps.ld = d.ldp;
    ps.writer = d.sub != 0;
    if (!BWD) {
      if (d.kind == DF_DIAG_FWD) diag_body<T, ACC, false, DR, 1>(t, d.sub, a, dsm, w);
      else upd_body<T, ACC, 256, 1>(t, a, dsm, w, ps);
    } else {
      if (d.kind == DF_RED_BWD) red_body<T, ACC, 256, 1>(t, a, dsm, w, ps);
      else if (d.kind == DF_DIAG_BWD) diag_body<T, ACC, true, DR, 1>(t, d.sub, a, dsm, w);
      else fin_body<T, ACC>(t, a, w);
    }
    // every thread's results visible device-wide before the count
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(a.dfc + d.sig, 1);
  }
}
template <typename T, typename ACC> constexpr size_t chain_smem() {
  constexpr size_t d = diag_mv_smem<T, ACC, DF_ROWS>(), u = upd_smem<T, ACC, 256>(),
                   r = red_smem<T, ACC>();
  return d > u ? (d > r ? d : r) : (u > r ? u : r);
}

// The contribution-row kernels read L in 16-byte pieces of a column: every
// front's storage starts on a 64-element boundary with a leading dimension
// that is a multiple of 4, so a piece that starts on a row divisible by 4 is
// 16-byte aligned (and lies inside the column's padded length).
// Two FP32 fused multiply-adds in one instruction (fma.rn.f32x2, sm_100
// and later): c + a * b lane by lane on values packed two to a 64-bit
// register (the lower half is the first), each rounded exactly as fmaf.
// Halves the FMA instructions of the backward contribution-row product,
// which issues 16 multiply-adds per 4-byte entry of L at 16 right-hand sides
// (0.94 -> 0.86 ms per sweep at 80^3; the forward kernel, which holds eight
// columns of L in flight in registers, measured slower with it: 0.69 -> 0.88).
__device__ __forceinline__ unsigned long long f2fma(unsigned long long a, unsigned long long b,
                                                    unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ unsigned long long f2dup(float v) {
  const unsigned long long u = __float_as_uint(v);
  return u | (u << 32);
}
__device__ __forceinline__ float f2lo(unsigned long long v) { return __uint_as_float((unsigned)v); }
__device__ __forceinline__ float f2hi(unsigned long long v) {
  return __uint_as_float((unsigned)(v >> 32));
}

constexpr int RF_KU = 8;   // columns of L in flight per thread (forward)
constexpr int RB_SR = 16;  // rows per pipeline slice (backward)
template <typename T> constexpr int rb_nst() { return 3; }
// padded column run of a slice: 16-byte aligned, and lanes RB_LP apart hit
// distinct banks with 16-byte reads
template <typename T> constexpr int rb_lp() { return RB_SR + 16 / (int)sizeof(T); }
template <typename T> struct Pair;
template <> struct Pair<float> {
  using V = float2;
};
template <> struct Pair<double> {
  using V = double2;
};

// Contribution rows (i >= n) of a front, forward: x(rls[i], :) -= L(i, c0:c0+bw)
// y with y = x(rls[c0:c0+bw], :), the front's solved pivot rows, for the rows
// [r0, r0 + 2 RECT_FWD_T) of the task (r0 divisible by 4; rows below n in
// the first tile are skipped).  Thread t owns the adjacent rows r0 + 2t and
// r0 + 2t + 1 and reads them from each column as one 8-byte (FP32) or
// 16-byte (FP64) load straight into registers, the next RF_KU columns in
// flight while the current ones are multiplied; the task's block of y (RQ
// right-hand sides per pass) is staged in shared memory and read as 16-byte
// vectors that serve both rows.  Sibling fronts of a level share ancestor
// rows, so the results are added with atomics.  Dynamic shared memory:
// rect_fwd_smem(kpad), kpad >= every task's bw rounded up to RF_KU.
template <typename T, typename ACC, int RQ>
__global__ void __launch_bounds__(RECT_FWD_T) k_rect_fwd(const LTask* __restrict__ tasks,
                                                         LsArgs<T, ACC> a) {
  using V = typename Vec4<ACC>::V;
  using P2 = typename Pair<T>::V;
  constexpr int VW = Vec4<ACC>::W, KU = RF_KU;
  static_assert(RQ % VW == 0, "right-hand sides per pass");
  extern __shared__ __align__(16) unsigned char dsm[];
  int* rc = reinterpret_cast<int*>(dsm);        // [TW] pivot rows of the block
  ACC* yb = reinterpret_cast<ACC*>(rc + TW);   // [kpad][RQ]
  const LTask t = tasks[blockIdx.x];
  const FrontDesc f = a.fr[t.f];
  const int* rl = a.rlist + f.rl;
  const int tid = threadIdx.x, bw = t.bw, i0 = t.r0 + 2 * tid;
  const bool live0 = i0 >= f.n && i0 < f.m, live1 = i0 + 1 >= f.n && i0 + 1 < f.m;
  const bool any = i0 < f.m;  // rows beyond m: padding of the column, never used
  const int dst0 = live0 ? rl[i0] : 0, dst1 = live1 ? rl[i0 + 1] : 0;
  const P2* Lp = reinterpret_cast<const P2*>(a.arena + f.off + (int64_t)t.c0 * f.ld + (any ? i0 : t.r0));
  const int64_t lds = f.ld / 2;  // column stride in pairs
  const int kpad = (bw + KU - 1) / KU * KU;
  for (int k = tid; k < bw; k += RECT_FWD_T) rc[k] = rl[t.c0 + k];
  for (int rg = 0; rg < a.nrhs; rg += RQ) {
    const int nr = min(RQ, a.nrhs - rg);
    __syncthreads();  // rc written; the previous pass's block is no longer read
    for (int e = tid; e < kpad * RQ; e += RECT_FWD_T) {
      const int q = e % RQ, k = e / RQ;
      if (k < bw && q < nr) cp_async(&yb[e], &a.x[(int64_t)(rg + q) * a.n + rc[k]]);
      else yb[e] = ACC(0);
    }
    P2 ln[KU];
#pragma unroll
    for (int u = 0; u < KU; ++u) ln[u] = (any && u < bw) ? Lp[u * lds] : P2{};
    cp_async_wait_all();
    __syncthreads();
    ACC acc0[RQ], acc1[RQ];
#pragma unroll
    for (int q = 0; q < RQ; ++q) acc0[q] = acc1[q] = ACC(0);
    for (int k0 = 0; k0 < bw; k0 += KU) {
      P2 lc[KU];
#pragma unroll
      for (int u = 0; u < KU; ++u) lc[u] = ln[u];
#pragma unroll
      for (int u = 0; u < KU; ++u) {
        const int k = k0 + KU + u;
        ln[u] = (any && k < bw) ? Lp[(int64_t)k * lds] : P2{};
      }
#pragma unroll
      for (int u = 0; u < KU; ++u) {
        const ACC l0 = (ACC)lc[u].x, l1 = (ACC)lc[u].y;
        const V* yv = reinterpret_cast<const V*>(yb + (k0 + u) * RQ);
#pragma unroll
        for (int q = 0; q < RQ / VW; ++q) {
          const V y4 = yv[q];
          if constexpr (VW == 4) {
            acc0[4 * q + 0] += l0 * y4.x;
            acc0[4 * q + 1] += l0 * y4.y;
            acc0[4 * q + 2] += l0 * y4.z;
            acc0[4 * q + 3] += l0 * y4.w;
            acc1[4 * q + 0] += l1 * y4.x;
            acc1[4 * q + 1] += l1 * y4.y;
            acc1[4 * q + 2] += l1 * y4.z;
            acc1[4 * q + 3] += l1 * y4.w;
          } else {
            acc0[2 * q + 0] += l0 * y4.x;
            acc0[2 * q + 1] += l0 * y4.y;
            acc1[2 * q + 0] += l1 * y4.x;
            acc1[2 * q + 1] += l1 * y4.y;
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < RQ; ++q)
      if (q < nr) {
        if (live0) aadd(&a.x[(int64_t)(rg + q) * a.n + dst0], -acc0[q]);
        if (live1) aadd(&a.x[(int64_t)(rg + q) * a.n + dst1], -acc1[q]);
      }
  }
}

// Contribution rows of a front, backward: t(k, :) = sum_i L(i, c0 + k)
// x(rls[i], :) over the rows [r0, r0 + RECT_BWD_ROWS) of the task (r0
// divisible by 4; rows below n are skipped), added into tacc at the block's
// pivot rows rls[c0 + k] (tacc is laid out like x; the pivot rows' gather
// reads and clears it).  RB_SR-row slices of the tile of L (up to
// RECT_BWD_COLS columns, each column a padded run of RB_SR rows so the
// 16-byte reads of a warp are conflict-free) and of x are copied to shared
// memory asynchronously, several slices in flight.  Thread (column pair p,
// row half h) owns columns p and p + RECT_BWD_COLS / 2, so each 16-byte read
// of x serves two columns; the halves are reduced through shared memory,
// one set of atomics per task.
template <typename T, typename ACC, int RQ>
__global__ void __launch_bounds__(RECT_BWD_T) k_rect_bwd(const LTask* __restrict__ tasks,
                                                         LsArgs<T, ACC> a) {
  using V = typename Vec4<ACC>::V;
  constexpr int VW = Vec4<ACC>::W, SR = RB_SR, KC = RECT_BWD_COLS, NT = RECT_BWD_T;
  constexpr int NP = KC / 2, HR = SR / 2;  // column pairs; rows of a slice per half
  constexpr int NST = rb_nst<T>(), LP = rb_lp<T>(), CH = 16 / sizeof(T);
  static_assert(RQ % VW == 0 && NT == 2 * NP && HR % CH == 0, "thread layout");
  extern __shared__ __align__(16) unsigned char dsm[];
  T* Ls = reinterpret_cast<T*>(dsm);                        // [NST][KC][LP]
  ACC* xt = reinterpret_cast<ACC*>(Ls + NST * KC * LP);     // [NST][SR][RQ]
  ACC* half = xt + NST * SR * RQ;                           // [KC][RQ + 1]
  int* rr = reinterpret_cast<int*>(half + KC * (RQ + 1));  // [RECT_BWD_ROWS]
  const LTask t = tasks[blockIdx.x];
  const FrontDesc f = a.fr[t.f];
  const T* Lc = a.arena + f.off + (int64_t)t.c0 * f.ld + t.r0;
  const int* rl = a.rlist + f.rl;
  const int bw = t.bw, tid = threadIdx.x, p = tid % NP, h = tid / NP;
  const int rows = min(RECT_BWD_ROWS, f.m - t.r0), nst = (rows + SR - 1) / SR;
  const int rlo = f.n - t.r0;  // rows of the tile below this one are pivot rows: skipped
  for (int ii = tid; ii < rows; ii += NT) rr[ii] = rl[t.r0 + ii];
  auto issue = [&](int st, int rg, int nr) {
    T* d = Ls + (st % NST) * KC * LP;
    for (int e = tid; e < KC * SR / CH; e += NT) {
      const int kk = e / (SR / CH), row = (e % (SR / CH)) * CH, grow = st * SR + row;
      T* dp = d + kk * LP + row;
      if (kk < bw && grow < rows) cp_async16(dp, Lc + (int64_t)kk * f.ld + grow);
      else *reinterpret_cast<float4*>(dp) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    ACC* dx = xt + (st % NST) * SR * RQ;
    for (int e = tid; e < SR * RQ; e += NT) {
      const int r = e % RQ, ii = e / RQ, grow = st * SR + ii;
      if (grow >= rlo && grow < rows && r < nr)
        cp_async(&dx[e], &a.x[(int64_t)(rg + r) * a.n + rr[grow]]);
      else dx[e] = ACC(0);
    }
  };
  for (int rg = 0; rg < a.nrhs; rg += RQ) {
    const int nr = min(RQ, a.nrhs - rg);
    __syncthreads();  // rr written; the previous pass's buffers are no longer read
#pragma unroll
    for (int st = 0; st < NST - 1; ++st) {
      if (st < nst) issue(st, rg, nr);
      cp_async_commit();
    }
    ACC acc0[RQ], acc1[RQ];
#pragma unroll
    for (int q = 0; q < RQ; ++q) acc0[q] = acc1[q] = ACC(0);
    unsigned long long pa0[RQ / 2], pa1[RQ / 2];  // FP32: packed pairs (fma.rn.f32x2)
#pragma unroll
    for (int q = 0; q < RQ / 2; ++q) pa0[q] = pa1[q] = 0ull;
    for (int s = 0; s < nst; ++s) {
      cp_async_wait<NST - 2>();
      __syncthreads();  // slice s landed for all; slice s - 1's buffers are free
      if (s + NST - 1 < nst) issue(s + NST - 1, rg, nr);
      cp_async_commit();
      const T* l0p = Ls + (s % NST) * KC * LP + p * LP + h * HR;
      const T* l1p = l0p + NP * LP;
      const ACC* xb = xt + (s % NST) * SR * RQ + h * HR * RQ;
#pragma unroll
      for (int i4 = 0; i4 < HR; i4 += CH) {
        ACC l0[CH], l1[CH];
        if constexpr (CH == 4) {
          const float4 v0 = *reinterpret_cast<const float4*>(l0p + i4);
          const float4 v1 = *reinterpret_cast<const float4*>(l1p + i4);
          l0[0] = v0.x; l0[1] = v0.y; l0[2] = v0.z; l0[3] = v0.w;
          l1[0] = v1.x; l1[1] = v1.y; l1[2] = v1.z; l1[3] = v1.w;
        } else {
          const double2 v0 = *reinterpret_cast<const double2*>(l0p + i4);
          const double2 v1 = *reinterpret_cast<const double2*>(l1p + i4);
          l0[0] = v0.x; l0[1] = v0.y;
          l1[0] = v1.x; l1[1] = v1.y;
        }
#pragma unroll
        for (int u = 0; u < CH; ++u) {
          const V* xv = reinterpret_cast<const V*>(xb + (i4 + u) * RQ);
          if constexpr (VW == 4) {
            const unsigned long long d0 = f2dup(l0[u]), d1 = f2dup(l1[u]);
#pragma unroll
            for (int q = 0; q < RQ / 4; ++q) {
              const ulonglong2 x2 = reinterpret_cast<const ulonglong2*>(xv)[q];
              pa0[2 * q] = f2fma(d0, x2.x, pa0[2 * q]);
              pa0[2 * q + 1] = f2fma(d0, x2.y, pa0[2 * q + 1]);
              pa1[2 * q] = f2fma(d1, x2.x, pa1[2 * q]);
              pa1[2 * q + 1] = f2fma(d1, x2.y, pa1[2 * q + 1]);
            }
          } else {
#pragma unroll
            for (int q = 0; q < RQ / VW; ++q) {
              const V x4 = xv[q];
              acc0[2 * q + 0] += l0[u] * x4.x;
              acc0[2 * q + 1] += l0[u] * x4.y;
              acc1[2 * q + 0] += l1[u] * x4.x;
              acc1[2 * q + 1] += l1[u] * x4.y;
            }
          }
        }
      }
    }
    if constexpr (VW == 4) {
#pragma unroll
      for (int q = 0; q < RQ / 2; ++q) {
        acc0[2 * q] = f2lo(pa0[q]);
        acc0[2 * q + 1] = f2hi(pa0[q]);
        acc1[2 * q] = f2lo(pa1[q]);
        acc1[2 * q + 1] = f2hi(pa1[q]);
      }
    }
    cp_async_wait<0>();
    if (h == 1)
#pragma unroll
      for (int q = 0; q < RQ; ++q) {
        half[p * (RQ + 1) + q] = acc0[q];
        half[(p + NP) * (RQ + 1) + q] = acc1[q];
      }
    __syncthreads();
    if (h == 0) {
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int k = p + c * NP;
        if (k < bw) {
          const int64_t pr = rl[t.c0 + k];
#pragma unroll
          for (int q = 0; q < RQ; ++q)
            if (q < nr)
              aadd(&a.tacc[(int64_t)(rg + q) * a.n + pr],
                   (c == 0 ? acc0[q] : acc1[q]) + half[k * (RQ + 1) + q]);
        }
      }
    }
  }
}

inline int nblocks(int64_t count, int bs) { return (int)((count + bs - 1) / bs); }

// dynamic shared memory of the contribution-row kernels
template <typename T, typename ACC, int RQ> constexpr size_t rect_fwd_smem(int kpad) {
  return sizeof(int) * TW + sizeof(ACC) * (size_t)kpad * RQ;
}
template <typename T, typename ACC, int RQ> constexpr size_t rect_bwd_smem() {
  return sizeof(T) * rb_nst<T>() * RECT_BWD_COLS * rb_lp<T>() +
         sizeof(ACC) * (rb_nst<T>() * RB_SR * RQ + RECT_BWD_COLS * (RQ + 1)) +
         sizeof(int) * RECT_BWD_ROWS;
}
}  // namespace

template <typename T, typename ACC>
void launch_solve_fwd(const T* arena, const FrontDesc* fr, int nfronts, const int* rlist,
                      ACC* x, int n, int nrhs, ACC* scratch, const int64_t* scr_off,
                      bool unit_diag, cudaStream_t s) {
  if (nfronts <= 0) return;
  if (nrhs > MAXR) throw CudaError("solve: more than 32 right-hand sides per launch");
  k_solve_fwd<T, ACC><<<nfronts, 256, 0, s>>>(arena, fr, rlist, x, n, nrhs, scratch, scr_off,
                                              unit_diag);
}

template <typename T, typename ACC>
void launch_small_tri(bool fwd, const T* arena, const FrontDesc* fr, int nfronts,
                      const int* rlist, ACC* x, ACC* tacc, int n, int nrhs, int maxn,
                      bool unit_diag, cudaStream_t s) {
  if (nfronts <= 0) return;
  if (nrhs > MAXR) throw CudaError("solve: more than 32 right-hand sides per launch");
  const size_t sm = (size_t)maxn * nrhs * sizeof(ACC) + (size_t)maxn * sizeof(int);
  if (sm > TRI_SMEM) throw CudaError("solve: small front with too many pivot rows");
  if (fwd)
    k_tri<T, ACC, false><<<nfronts, 256, sm, s>>>(arena, fr, rlist, x, tacc, n, nrhs, unit_diag);
  else
    k_tri<T, ACC, true><<<nfronts, 256, sm, s>>>(arena, fr, rlist, x, tacc, n, nrhs, unit_diag);
}

template <typename ACC>
void launch_permute_in(const double* x, int ldx, ACC* xp, const int* perm, const double* scale,
                       int n, int nrhs, cudaStream_t s) {
  int64_t c = (int64_t)n * nrhs;
  if (c == 0) return;
  k_permute_in<ACC><<<nblocks(c, 256), 256, 0, s>>>(x, ldx, xp, perm, scale, n, nrhs);
}

template <typename ACC>
void launch_permute_out_add(const ACC* xp, const int* perm, const double* scale, double* x,
                            int ldx, int n, int nrhs, bool add, cudaStream_t s) {
  int64_t c = (int64_t)n * nrhs;
  if (c == 0) return;
  k_permute_out<ACC><<<nblocks(c, 256), 256, 0, s>>>(xp, perm, scale, x, ldx, n, nrhs, add);
}

void launch_scale_vals(double* val, const int* row, const int* col, const double* scale,
                       int64_t count, cudaStream_t s) {
  if (count <= 0) return;
  k_scale_vals<<<nblocks(count, 256), 256, 0, s>>>(val, row, col, scale, count);
}

void launch_residual(const int64_t* rowptr, const int* col, const double* aval, int n,
                     const double* x, int ldx, const double* b, int ldb, double* r, int nrhs,
                     cudaStream_t s) {
  if (n == 0) return;
  k_residual<<<nblocks(n, 128), 128, 0, s>>>(rowptr, col, aval, n, x, ldx, b, ldb, r, nrhs);
}

void launch_maxnorms(const double* res, const double* x, int ldx, const double* b, int ldb,
                     int n, int nrhs, double* norms, cudaStream_t s) {
  if (n == 0) return;
  dim3 grid(std::min(nblocks(n, 256), 152), nrhs);
  k_maxnorms<<<grid, 256, 0, s>>>(res, x, ldx, b, ldb, n, nrhs, norms);
}

void launch_rownorm_inf(const int64_t* rowptr, const double* aval, int n, double* out,
                        cudaStream_t s) {
  if (n == 0) return;
  k_rownorm<<<nblocks(n, 256), 256, 0, s>>>(rowptr, aval, n, out);
}

void launch_gather_clean(const double* val, const int64_t* srcptr, const int64_t* src,
                         int64_t nclean, double* cval, cudaStream_t s) {
  if (nclean == 0) return;
  k_gather_clean<<<nblocks(nclean, 256), 256, 0, s>>>(val, srcptr, src, nclean, cval);
}

void launch_gather(const double* cval, const int64_t* idx, int64_t count, double* out,
                   cudaStream_t s) {
  if (count == 0) return;
  k_gather<<<nblocks(count, 256), 256, 0, s>>>(cval, idx, count, out);
}

void launch_axpy_inplace(double* x, int ldx, const double* d, int n, int nrhs, cudaStream_t s) {
  int64_t c = (int64_t)n * nrhs;
  if (c == 0) return;
  k_axpy<<<nblocks(c, 256), 256, 0, s>>>(x, ldx, d, n, nrhs);
}

template <typename T, typename ACC>
void launch_lsolve(int kind, const LTask* tasks, int ntask, LsArgs<T, ACC> a, int aux,
                   cudaStream_t s) {
  if (ntask <= 0) return;
  if (a.nrhs > MAXR) throw CudaError("solve: more than 32 right-hand sides per launch");
  switch (kind) {
    case LS_GATHER_FWD:
    case LS_GATHER_BWD:
      k_lgather<T, ACC><<<ntask, 256, 0, s>>>(tasks, a, kind == LS_GATHER_FWD);
      break;
    case LS_SCATTER_FWD:
    case LS_SCATTER_BWD:
      k_lscatter<T, ACC><<<ntask, 256, 0, s>>>(tasks, a, kind == LS_SCATTER_FWD);
      break;
    case LS_FWD_DIAG2:
      launch_pdl(k_diag_mv<T, ACC, false>, dim3(ntask, SW / DMV_ROWS), 256, diag_mv_smem<T, ACC>(), s,
                 tasks, a);
      break;
    case LS_FWD_UPD2:
      launch_pdl(k_fwd_upd3<T, ACC>, dim3(ntask), 512, upd_smem<T, ACC, 512>(), s, tasks, a);
      break;
    case LS_RECT_FWD: {
      // aux: the widest task's columns rounded up to the pipeline slice
      const int kpad = std::min(std::max(aux, RF_KU), TW);
      if (a.nrhs <= 4)
        k_rect_fwd<T, ACC, 4><<<ntask, RECT_FWD_T, rect_fwd_smem<T, ACC, 4>(kpad), s>>>(tasks, a);
      else
        k_rect_fwd<T, ACC, RQ_MID<ACC>>
            <<<ntask, RECT_FWD_T, rect_fwd_smem<T, ACC, RQ_MID<ACC>>(kpad), s>>>(tasks, a);
      break;
    }
    case LS_RECT_BWD:
      if (a.nrhs <= 4)
        k_rect_bwd<T, ACC, 4><<<ntask, RECT_BWD_T, rect_bwd_smem<T, ACC, 4>(), s>>>(tasks, a);
      else
        k_rect_bwd<T, ACC, RQ_MID<ACC>>
            <<<ntask, RECT_BWD_T, rect_bwd_smem<T, ACC, RQ_MID<ACC>>(), s>>>(tasks, a);
      break;
    case LS_BWD_RED2:
      launch_pdl(k_bwd_red3<T, ACC>, dim3(ntask), 512, red_smem<T, ACC>(), s, tasks, a);
      break;
    case LS_BWD_DIAG2:
      launch_pdl(k_diag_mv<T, ACC, true>, dim3(ntask, SW / DMV_ROWS), 256, diag_mv_smem<T, ACC>(), s,
                 tasks, a);
      break;
  }
}

// persistent CTAs of a dataflow sweep: resident CTAs per SM x SMs (set once)
static int g_chain_ctas = 0;

void launch_chain(bool bwd, const DfTask* tasks, int ntask, LsArgs<float, float> a, unsigned* err,
                  cudaStream_t s) {
  if (ntask <= 0) return;
  const int grid = std::max(1, std::min(ntask, g_chain_ctas));
  if (bwd) k_chain<float, float, true><<<grid, 256, chain_smem<float, float>(), s>>>(tasks, ntask, a, err);
  else k_chain<float, float, false><<<grid, 256, chain_smem<float, float>(), s>>>(tasks, ntask, a, err);
  SG_CUDA(cudaGetLastError());
}

template <typename T>
void launch_inv_diag(const T* arena, const FrontDesc* fr, const LTask* tasks, int ntask,
                     T* inv, const int64_t* inv_off, bool unit, cudaStream_t s) {
  if (ntask <= 0) return;
  k_inv_diag<T><<<ntask, LB, 0, s>>>(arena, fr, tasks, inv, inv_off, unit);
}

template <typename T, int RQ>
void set_rect_smem() {
  SG_CUDA(cudaFuncSetAttribute(k_rect_fwd<T, T, RQ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)rect_fwd_smem<T, T, RQ>(TW)));
  SG_CUDA(cudaFuncSetAttribute(k_rect_bwd<T, T, RQ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)rect_bwd_smem<T, T, RQ>()));
}

template <typename T>
void prepare_solve_kernels() {
  SG_CUDA(cudaFuncSetAttribute(k_inv_block<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(2 * 64 * 65 * sizeof(T))));
  SG_CUDA(cudaFuncSetAttribute(k_diag_mv<T, T, false>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)diag_mv_smem<T, T>()));
  SG_CUDA(cudaFuncSetAttribute(k_diag_mv<T, T, true>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)diag_mv_smem<T, T>()));
  SG_CUDA(cudaFuncSetAttribute(k_tri<T, T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)TRI_SMEM));
  SG_CUDA(cudaFuncSetAttribute(k_tri<T, T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)TRI_SMEM));
  set_rect_smem<T, 4>();
  set_rect_smem<T, RQ_MID<T>>();
  SG_CUDA(cudaFuncSetAttribute(k_fwd_upd3<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)upd_smem<T, T, 512>()));
  SG_CUDA(cudaFuncSetAttribute(k_bwd_red3<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)red_smem<T, T>()));
  if constexpr (std::is_same<T, float>::value) {
    const int cs = (int)chain_smem<T, T>();
    SG_CUDA(cudaFuncSetAttribute(k_chain<T, T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs));
    SG_CUDA(cudaFuncSetAttribute(k_chain<T, T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs));
    int dev = 0, nsm = 0, per0 = 0, per1 = 0;
    SG_CUDA(cudaGetDevice(&dev));
    SG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    SG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per0, k_chain<T, T, false>, 256, cs));
    SG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, k_chain<T, T, true>, 256, cs));
    g_chain_ctas = std::max(1, nsm * std::max(1, std::min(per0, per1)));
  }
}

void launch_form_p(const float* arena, const FrontDesc* fr, const PTask* tasks, int ntask,
                   const float* inv2t, const int64_t* inv2_off, float* pmat, cudaStream_t s) {
  if (ntask <= 0) return;
  k_form_p<<<ntask, 256, 0, s>>>(arena, fr, tasks, inv2t, inv2_off, pmat);
  SG_CUDA(cudaGetLastError());
}

template <typename T>
void launch_inv_block(const T* arena, const FrontDesc* fr, const LTask* tasks, int ntask,
                   const T* inv64, const int64_t* inv_off, T* inv2, T* inv2t,
                   const int64_t* inv2_off, cudaStream_t s) {
  if (ntask <= 0) return;
  k_inv_block<T><<<ntask, 256, 2 * 64 * 65 * sizeof(T), s>>>(arena, fr, tasks, inv64, inv_off,
                                                           inv2, inv2t, inv2_off);
}
template void prepare_solve_kernels<float>();
template void prepare_solve_kernels<double>();
template void launch_inv_block<float>(const float*, const FrontDesc*, const LTask*, int,
                                   const float*, const int64_t*, float*, float*,
                                   const int64_t*, cudaStream_t);
template void launch_inv_block<double>(const double*, const FrontDesc*, const LTask*, int,
                                    const double*, const int64_t*, double*, double*,
                                    const int64_t*, cudaStream_t);

template void launch_lsolve<float, float>(int, const LTask*, int, LsArgs<float, float>, int,
                                          cudaStream_t);
template void launch_lsolve<double, double>(int, const LTask*, int, LsArgs<double, double>, int,
                                            cudaStream_t);
template void launch_inv_diag<float>(const float*, const FrontDesc*, const LTask*, int, float*,
                                     const int64_t*, bool, cudaStream_t);
template void launch_inv_diag<double>(const double*, const FrontDesc*, const LTask*, int,
                                      double*, const int64_t*, bool, cudaStream_t);
template void launch_solve_fwd<float, float>(const float*, const FrontDesc*, int, const int*,
                                             float*, int, int, float*, const int64_t*, bool,
                                             cudaStream_t);
template void launch_solve_fwd<double, double>(const double*, const FrontDesc*, int,
                                               const int*, double*, int, int, double*,
                                               const int64_t*, bool, cudaStream_t);
template void launch_small_tri<float, float>(bool, const float*, const FrontDesc*, int,
                                             const int*, float*, float*, int, int, int, bool,
                                             cudaStream_t);
template void launch_small_tri<double, double>(bool, const double*, const FrontDesc*, int,
                                               const int*, double*, double*, int, int, int, bool,
                                               cudaStream_t);
template void launch_permute_in<float>(const double*, int, float*, const int*, const double*,
                                       int, int, cudaStream_t);
template void launch_permute_in<double>(const double*, int, double*, const int*, const double*,
                                        int, int, cudaStream_t);
template void launch_permute_out_add<float>(const float*, const int*, const double*, double*,
                                            int, int, int, bool, cudaStream_t);
template void launch_permute_out_add<double>(const double*, const int*, const double*, double*,
                                             int, int, int, bool, cudaStream_t);

}  // namespace sylver_gb300
