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
// dynamic shared memory of the on-chip small-front kernels (right-hand-side
// rows and their destinations)
constexpr size_t SMALL_SOLVE_SMEM = 160 * 1024;

template <typename T> __device__ __forceinline__ void aadd(T* p, T v) { atomicAdd(p, v); }

// The large-front solve steps use programmatic dependent launch
// (pdl_trigger / pdl_wait): a step lets the next one launch at once, and
// its CTAs stage the factor data they need (which no step writes) before
// they wait for the previous step's grid.

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

template <typename T, typename ACC>
__global__ void __launch_bounds__(256) k_solve_bwd(const T* __restrict__ arena,
                                                   const FrontDesc* __restrict__ fr,
                                                   const int* __restrict__ rlist,
                                                   ACC* __restrict__ x, int n, int nrhs,
                                                   ACC* __restrict__ scratch,
                                                   const int64_t* __restrict__ scr_off,
                                                   bool unit) {
  __shared__ ACC tt[SB][MAXR];
  __shared__ ACC Ld[SB][SB + 1];  // Ld[k][i] = L(c0 + i, c0 + k)
  const FrontDesc f = fr[blockIdx.x];
  const T* L = arena + f.off;
  const int ld = f.ld, m = f.m, nc = f.n;
  const int* rl = rlist + f.rl;
  ACC* xs = scratch + scr_off[blockIdx.x] * nrhs;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  for (int base = 0; base < m * nrhs; base += GB * 256) {
    ACC v[GB];
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u, i = idx % m, r = idx / m;
      v[u] = idx < m * nrhs ? x[(int64_t)r * n + rl[i]] : ACC(0);
    }
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u;
      if (idx < m * nrhs) xs[idx] = v[u];
    }
  }
  __shared__ ACC rdg[SB];
  __syncthreads();
  const int nblk = (nc + SB - 1) / SB;
  for (int b = nblk - 1; b >= 0; --b) {
    const int c0 = b * SB, bw = min(SB, nc - c0), c1 = c0 + bw;
    for (int kk = warp; kk < bw; kk += nwarps) {
      const T* col = L + (int64_t)(c0 + kk) * ld;
      for (int r0 = 0; r0 < nrhs; r0 += RC) {
        ACC acc[RC];
#pragma unroll
        for (int q = 0; q < RC; ++q) acc[q] = ACC(0);
#pragma unroll 4
        for (int i = c1 + lane; i < m; i += 32) {
          ACC l = (ACC)col[i];
#pragma unroll
          for (int q = 0; q < RC; ++q)
            if (r0 + q < nrhs) acc[q] += l * xs[(int64_t)(r0 + q) * m + i];
        }
#pragma unroll
        for (int q = 0; q < RC; ++q) {
          ACC s = acc[q];
          for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
          if (lane == 0 && r0 + q < nrhs) tt[kk][r0 + q] = s;
        }
      }
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
    // diagonal block (transposed): one right-hand side per warp at a time
    for (int r = warp; r < nrhs; r += nwarps) {
      ACC v = (lane < bw) ? xs[(int64_t)r * m + c0 + lane] - tt[lane][r] : ACC(0);
      for (int kk = bw - 1; kk >= 0; --kk) {
        if (lane == kk) v = v * rdg[kk];
        ACC zk = __shfl_sync(0xffffffffu, v, kk);
        if (lane < kk) v -= Ld[lane][kk] * zk;
      }
      if (lane < bw) xs[(int64_t)r * m + c0 + lane] = v;
    }
    __syncthreads();
  }
  for (int base = 0; base < m * nrhs; base += GB * 256) {
    ACC v[GB];
    int dsti[GB];
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u, i = idx % m;
      const bool ok = idx < m * nrhs && i < nc;
      v[u] = ok ? xs[idx] : ACC(0);
      dsti[u] = ok ? rl[i] : -1;
    }
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u;
      if (dsti[u] >= 0) x[(int64_t)(idx / m) * n + dsti[u]] = v[u];
    }
  }
}

// Small fronts whose right-hand-side rows fit in shared memory: the rows
// (ys[r*m + i], r < nrhs) and their destinations stay on chip from the gather
// to the scatter, so the column blocks touch global memory only for L.
template <typename T, typename ACC>
__global__ void __launch_bounds__(256, sizeof(ACC) == 4 ? 3 : 2) k_solve_fwd_s(const T* __restrict__ arena,
                                                     const FrontDesc* __restrict__ fr,
                                                     const int* __restrict__ rlist,
                                                     ACC* __restrict__ x, int n, int nrhs,
                                                     bool unit) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ ACC Ld[SB][SB + 1];  // Ld[k][i] = L(c0 + i, c0 + k)
  __shared__ ACC rdg[SB];         // 1 / L(c0 + k, c0 + k)
  const FrontDesc f = fr[blockIdx.x];
  const T* L = arena + f.off;
  const int ld = f.ld, m = f.m, nc = f.n, mr = m * nrhs;
  ACC* ys = reinterpret_cast<ACC*>(dsm);
  int* rls = reinterpret_cast<int*>(ys + mr);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < m; i += 256) rls[i] = rlist[f.rl + i];
  __syncthreads();
  // the pivot rows are gathered; the rows below start at zero and collect
  // this front's contribution, which the scatter adds to the ancestors'
  // rows (sibling fronts of the launch add to the same rows)
  for (int base = 0; base < mr; base += GB * 256) {
    ACC v[GB];
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u, i = idx % m;
      v[u] = (idx < mr && i < nc) ? x[(int64_t)(idx / m) * n + rls[i]] : ACC(0);
    }
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u;
      if (idx < mr) ys[idx] = v[u];
    }
  }
  __syncthreads();
  for (int c0 = 0; c0 < nc; c0 += SB) {
    const int bw = min(SB, nc - c0), c1 = c0 + bw;
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
    for (int r = warp; r < nrhs; r += 8) {
      ACC v = (lane < bw) ? ys[r * m + c0 + lane] : ACC(0);
      for (int kk = 0; kk < bw; ++kk) {
        const ACC vk = __shfl_sync(0xffffffffu, v, kk) * rdg[kk];
        if (lane == kk) v = vk;
        if (lane > kk && lane < bw) v -= Ld[kk][lane] * vk;
      }
      if (lane < bw) ys[r * m + c0 + lane] = v;
    }
    __syncthreads();
    // rows below the block: one row per thread, its block row of L loaded
    // at once, eight right-hand sides per pass
    for (int i = c1 + tid; i < m; i += 256) {
      ACC lv[SB];
#pragma unroll
      for (int kk = 0; kk < SB; ++kk) lv[kk] = (kk < bw) ? (ACC)L[(int64_t)(c0 + kk) * ld + i] : ACC(0);
      for (int r0 = 0; r0 < nrhs; r0 += RC) {
        ACC acc[RC];
#pragma unroll
        for (int q = 0; q < RC; ++q) acc[q] = ACC(0);
#pragma unroll
        for (int kk = 0; kk < SB; ++kk) {
          const int row = c0 + min(kk, bw - 1);
#pragma unroll
          for (int q = 0; q < RC; ++q) acc[q] += lv[kk] * ys[min(r0 + q, nrhs - 1) * m + row];
        }
#pragma unroll
        for (int q = 0; q < RC; ++q)
          if (r0 + q < nrhs) ys[(r0 + q) * m + i] -= acc[q];
      }
    }
    __syncthreads();
  }
  for (int base = 0; base < mr; base += GB * 256) {
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u;
      if (idx >= mr) break;
      const int i = idx % m;
      ACC* dst = x + (int64_t)(idx / m) * n + rls[i];
      if (i < nc) *dst = ys[idx];
      else aadd(dst, ys[idx]);
    }
  }
}

template <typename T, typename ACC>
__global__ void __launch_bounds__(256) k_solve_bwd_s(const T* __restrict__ arena,
                                                     const FrontDesc* __restrict__ fr,
                                                     const int* __restrict__ rlist,
                                                     ACC* __restrict__ x, int n, int nrhs,
                                                     bool unit) {
  extern __shared__ __align__(16) unsigned char dsm[];
  __shared__ ACC tt[SB][MAXR];
  __shared__ ACC Ld[SB][SB + 1];  // Ld[k][i] = L(c0 + i, c0 + k)
  __shared__ ACC rdg[SB];
  const FrontDesc f = fr[blockIdx.x];
  const T* L = arena + f.off;
  const int ld = f.ld, m = f.m, nc = f.n, mr = m * nrhs;
  ACC* ys = reinterpret_cast<ACC*>(dsm);
  int* rls = reinterpret_cast<int*>(ys + mr);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < m; i += 256) rls[i] = rlist[f.rl + i];
  __syncthreads();
  for (int base = 0; base < mr; base += GB * 256) {
    ACC v[GB];
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u;
      v[u] = idx < mr ? x[(int64_t)(idx / m) * n + rls[idx % m]] : ACC(0);
    }
#pragma unroll
    for (int u = 0; u < GB; ++u) {
      const int idx = base + tid + 256 * u;
      if (idx < mr) ys[idx] = v[u];
    }
  }
  __syncthreads();
  constexpr int RB = 16;  // right-hand sides per pass of a column
  const int nblk = (nc + SB - 1) / SB;
  for (int b = nblk - 1; b >= 0; --b) {
    const int c0 = b * SB, bw = min(SB, nc - c0), c1 = c0 + bw;
    // tt[kk][r] = sum_{i >= c1} L(i, c0 + kk) x(i, r): one column per warp
    for (int kk = warp; kk < bw; kk += 8) {
      const T* col = L + (int64_t)(c0 + kk) * ld;
      for (int r0 = 0; r0 < nrhs; r0 += RB) {
        ACC acc[RB];
#pragma unroll
        for (int q = 0; q < RB; ++q) acc[q] = ACC(0);
#pragma unroll 2
        for (int i = c1 + lane; i < m; i += 32) {
          const ACC l = (ACC)col[i];
#pragma unroll
          for (int q = 0; q < RB; ++q) acc[q] += l * ys[min(r0 + q, nrhs - 1) * m + i];
        }
#pragma unroll
        for (int q = 0; q < RB; ++q) {
          ACC sv = acc[q];
          for (int o = 16; o > 0; o >>= 1) sv += __shfl_xor_sync(0xffffffffu, sv, o);
          if (lane == 0 && r0 + q < nrhs) tt[kk][r0 + q] = sv;
        }
      }
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
    // diagonal block (transposed): one right-hand side per warp at a time
    for (int r = warp; r < nrhs; r += 8) {
      ACC v = (lane < bw) ? ys[r * m + c0 + lane] - tt[lane][r] : ACC(0);
      for (int kk = bw - 1; kk >= 0; --kk) {
        if (lane == kk) v = v * rdg[kk];
        const ACC zk = __shfl_sync(0xffffffffu, v, kk);
        if (lane < kk) v -= Ld[lane][kk] * zk;
      }
      if (lane < bw) ys[r * m + c0 + lane] = v;
    }
    __syncthreads();
  }
  for (int base = 0; base < nc * nrhs; base += 256) {
    const int idx = base + tid;
    if (idx < nc * nrhs) {
      const int i = idx % nc, r = idx / nc;
      x[(int64_t)r * n + rls[i]] = ys[r * m + i];
    }
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
// Large fronts: blocked multi-CTA sweeps with explicit inverses of the 64x64
// diagonal blocks (computed once per factorization).  Forward step b: every
// CTA forms y_b = L_bb^-1 x_b itself and updates its own rows below the
// block; y_b goes to a separate slab so no CTA overwrites what others read.
// Backward step b: CTAs reduce L_{i,b}^T x_i over their rows into tt, and
// the last CTA to finish (atomic ticket, no waiting) solves the block.

constexpr int LB = LSOLVE_BW;

template <typename T, typename ACC>
__global__ void k_lgather(const LTask* __restrict__ tasks, LsArgs<T, ACC> a, bool fwd) {
  const LTask t = tasks[blockIdx.x];
  const FrontDesc f = a.fr[t.f];
  if (!fwd && t.r0 == 0) {
    // both backward accumulators of this front start at zero, and so do its
    // contribution-row sums
    ACC* tf = a.tt + (int64_t)t.f * 2 * LSOLVE_BW2 * MAXR;
    for (int e = threadIdx.x; e < 2 * LSOLVE_BW2 * MAXR; e += blockDim.x) tf[e] = ACC(0);
    const int nb = (f.n + LSOLVE_BW2 - 1) / LSOLVE_BW2;
    ACC* cb = a.tcb + (a.inv2_off[t.f] / ((int64_t)LSOLVE_BW2 * LSOLVE_BW2)) * LSOLVE_BW2 * MAXR;
    for (int e = threadIdx.x; e < nb * LSOLVE_BW2 * MAXR; e += blockDim.x) cb[e] = ACC(0);
  }
  const int i = t.r0 + threadIdx.x;
  if (i >= f.m) return;
  ACC* xs = a.scratch + a.scr_off[t.f] * a.nrhs;
  const int v = a.rlist[f.rl + i];
  const bool zero = fwd && i >= f.n;
  ACC val[MAXR];  // every load in flight before the first store
#pragma unroll
  for (int r = 0; r < MAXR; ++r)
    val[r] = (r < a.nrhs && !zero) ? a.x[(int64_t)r * a.n + v] : ACC(0);
#pragma unroll
  for (int r = 0; r < MAXR; ++r)
    if (r < a.nrhs) xs[(int64_t)r * f.m + i] = val[r];
}

template <typename T, typename ACC>
__global__ void k_lscatter(const LTask* __restrict__ tasks, LsArgs<T, ACC> a, bool fwd) {
  const LTask t = tasks[blockIdx.x];
  const FrontDesc f = a.fr[t.f];
  const int i = t.r0 + threadIdx.x;
  if (i >= f.m) return;
  if (!fwd && i >= f.n) return;
  const int64_t so = a.scr_off[t.f] * a.nrhs;
  const int v = a.rlist[f.rl + i];
  const ACC* src = (i >= f.n ? a.scratch : a.ys) + so + i;
  ACC val[MAXR];
#pragma unroll
  for (int r = 0; r < MAXR; ++r) val[r] = r < a.nrhs ? src[(int64_t)r * f.m] : ACC(0);
#pragma unroll
  for (int r = 0; r < MAXR; ++r) {
    if (r >= a.nrhs) break;
    ACC* dst = a.x + (int64_t)r * a.n + v;
    if (i >= f.n) aadd(dst, val[r]);
    else *dst = val[r];
  }
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

// Block steps of BW2 = 256 columns.  Each diagonal block has an explicit
// inverse (built once per factorization from its four 64x64 inverses), so a
// step is one parallel mat-vec on the diagonal block plus one update (forward)
// or reduction (backward) of the rows below, spread over many small CTAs.
constexpr int BW2 = LSOLVE_BW2;
constexpr int DMV_ROWS = 8;   // rows of the diagonal mat-vec per CTA (32 CTAs per block)
constexpr int BRED_ROWS = LSOLVE_RED_ROWS;  // rows per backward-reduction CTA
constexpr int CB_CHUNK = LSOLVE_CB_ROWS;    // contribution rows per backward CB CTA
template <typename ACC> struct RGn { static constexpr int v = sizeof(ACC) == 8 ? 8 : 16; };

// X = inverse of the 256-column diagonal block (column-major, ld 256, lower):
// X_jj = Inv64_j and X_ij = -Inv64_i * sum_{k=j}^{i-1} L_ik X_kj for i > j,
// with 64x64 blocks; identity beyond bw.
template <typename T>
__global__ void __launch_bounds__(256) k_inv256(const T* __restrict__ arena,
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
  T* X = inv2 + inv2_off[t.f] + (int64_t)(c0 / BW2) * BW2 * BW2;
  const T* I64 = inv64 + inv_off[t.f] + (int64_t)(c0 / LB) * LB * LB;
  const int nb = (bw + LB - 1) / LB;
  for (int e = tid; e < BW2 * BW2; e += blockDim.x) X[e] = T(0);
  __syncthreads();
  for (int j = 0; j < 4; ++j)
    for (int e = tid; e < LB * LB; e += blockDim.x) {
      int i = e % LB, k = e / LB;
      X[(int64_t)(LB * j + k) * BW2 + LB * j + i] =
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
        for (int e = tid; e < LB * LB; e += blockDim.x) {
          int rr = e % LB, kk = e / LB;
          int grow = LB * i + rr, gcol = LB * k + kk;
          As[kk * 65 + rr] = (grow < bw && gcol < bw) ? L[(int64_t)(c0 + gcol) * f.ld + c0 + grow] : T(0);
          Bs[rr * 65 + kk] = X[(int64_t)(LB * j + rr) * BW2 + LB * k + kk];  // B(kk, rr) = X_kj
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
      for (int q = 0; q < 16; ++q) X[(int64_t)(LB * j + cq * 16 + q) * BW2 + LB * i + r] = -acc[q];
      __syncthreads();
    }
  // transposed copy, XT[k*256 + i] = X(k, i), through 64 x 64 shared tiles
  T* XT = inv2t + inv2_off[t.f] + (int64_t)(c0 / BW2) * BW2 * BW2;
  for (int bj = 0; bj < BW2 / LB; ++bj)
    for (int bi = 0; bi < BW2 / LB; ++bi) {
      for (int e = tid; e < LB * LB; e += blockDim.x) {
        const int rr = e % LB, kk = e / LB;  // X(LB*bi + rr, LB*bj + kk)
        As[kk * 65 + rr] = X[(int64_t)(LB * bj + kk) * BW2 + LB * bi + rr];
      }
      __syncthreads();
      for (int e = tid; e < LB * LB; e += blockDim.x) {
        const int kk = e % LB, rr = e / LB;  // XT(LB*bj + kk, LB*bi + rr)
        XT[(int64_t)(LB * bi + rr) * BW2 + LB * bj + kk] = As[kk * 65 + rr];
      }
      __syncthreads();
    }
}

// Diagonal block of a 256-column solve step, as a product with its explicit
// inverse, split over gridDim.y = 4 CTAs of 64 output rows:
//   forward   y_b = X v,    v = xs(block)        -> ys(block)
//   backward  z_b = X^T v,  v = xs(block) - tt   -> ys(block)
// Solved rows (< n) live in ys in both directions, so no CTA overwrites
// values another CTA of the same launch still reads.
// (X^T read from the transposed copy, so both directions read the matrix
// coalesced down a column).  Thread (row i, k-phase g) sums k = g (mod 4);
// the four phases are reduced through shared memory.  The backward step
// reads accumulator (c0/256)&1 and clears the other one, which the next
// (lower) block's reduction fills.
template <typename ACC> struct Vec4;
template <> struct Vec4<float> {
  using V = float4;
  static constexpr int W = 4;
};
template <> struct Vec4<double> {
  using V = double2;
  static constexpr int W = 2;
};

// Forward update of rows [r0, r0 + 128) below the block [c0, c0 + bw) of a
// large front, one row per thread: x(i, :) -= L(i, c0:c0+bw) y(c0:c0+bw, :)
// with sixteen right-hand sides per pass in registers and the block's solved
// rows in shared memory.  For steps with many rows (the lower levels, many
// fronts with narrow blocks), where the k-split update's per-CTA staging and
// reduction cost more than the product.
template <typename T, typename ACC>
__global__ void __launch_bounds__(LSOLVE_ROWS_T) k_fwd_rows(const LTask* __restrict__ tasks,
                                                            LsArgs<T, ACC> a) {
  using V = typename Vec4<ACC>::V;
  constexpr int VW = Vec4<ACC>::W, RP = 16, KU = 16;
  __shared__ __align__(16) ACC yb[BW2 * RP];  // yb[k*16 + q] = y(c0 + k, rg + q)
  const LTask t = tasks[blockIdx.x];
  const FrontDesc f = a.fr[t.f];
  ACC* xs = a.scratch + a.scr_off[t.f] * a.nrhs;
  const ACC* ysl = a.ys + a.scr_off[t.f] * a.nrhs;
  const int tid = threadIdx.x, i = t.r0 + tid, bw = t.bw;
  const T* Li = a.arena + f.off + (int64_t)t.c0 * f.ld + i;
  for (int rg = 0; rg < a.nrhs; rg += RP) {
    const int nr = min(RP, a.nrhs - rg);
    __syncthreads();  // the previous pass's block is no longer read
    for (int e = tid; e < bw * RP; e += LSOLVE_ROWS_T) {
      const int k = e % bw, q = e / bw;
      yb[k * RP + q] = q < nr ? ysl[(int64_t)(rg + q) * f.m + t.c0 + k] : ACC(0);
    }
    __syncthreads();
    if (i >= f.m) continue;
    ACC acc[RP];
#pragma unroll
    for (int q = 0; q < RP; ++q) acc[q] = ACC(0);
    for (int k0 = 0; k0 < bw; k0 += KU) {
      ACC l[KU];
#pragma unroll
      for (int u = 0; u < KU; ++u)
        l[u] = (k0 + u < bw) ? (ACC)Li[(int64_t)(k0 + u) * f.ld] : ACC(0);
#pragma unroll
      for (int u = 0; u < KU; ++u) {
        const V* yv = reinterpret_cast<const V*>(yb + min(k0 + u, bw - 1) * RP);
#pragma unroll
        for (int q = 0; q < RP / VW; ++q) {
          const V y4 = yv[q];
          if constexpr (VW == 4) {
            acc[4 * q + 0] += l[u] * y4.x;
            acc[4 * q + 1] += l[u] * y4.y;
            acc[4 * q + 2] += l[u] * y4.z;
            acc[4 * q + 3] += l[u] * y4.w;
          } else {
            acc[2 * q + 0] += l[u] * y4.x;
            acc[2 * q + 1] += l[u] * y4.y;
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < RP; ++q)
      if (q < nr) xs[(int64_t)(rg + q) * f.m + i] -= acc[q];
  }
}

template <typename T, typename ACC, bool BWD>
__global__ void __launch_bounds__(256) k_diag_mv(const LTask* __restrict__ tasks,
                                                 LsArgs<T, ACC> a) {
  constexpr int RG = RGn<ACC>::v;
  constexpr int DR = DMV_ROWS;  // output rows per CTA; 256 / DR k-phases per row
  constexpr int NG = 256 / DR;
  using V = typename Vec4<ACC>::V;
  constexpr int VW = Vec4<ACC>::W;
  extern __shared__ __align__(16) unsigned char dsm[];
  T* Ms = reinterpret_cast<T*>(dsm);  // Ms[(k - klo)*DR + il] = M(i0 + il, k)
  ACC* part = reinterpret_cast<ACC*>(dsm + sizeof(T) * DR * BW2);  // [NG][DR][RG + 1]
  __shared__ __align__(16) ACC vb[BW2 * RG];
  const LTask t = tasks[blockIdx.x];
  const FrontDesc f = a.fr[t.f];
  const int c0 = t.c0, bw = t.bw, i0 = DR * blockIdx.y;
  const int tid = threadIdx.x, il = tid % DR, g = tid / DR, i = i0 + il;
  const int64_t m = f.m;
  ACC* xs = a.scratch + a.scr_off[t.f] * a.nrhs;
  ACC* ysl = a.ys + a.scr_off[t.f] * a.nrhs;
  const int64_t moff = a.inv2_off[t.f] + (int64_t)(c0 / BW2) * BW2 * BW2;
  const T* M = (BWD ? a.inv2t : a.inv2) + moff;
  ACC* tf = a.tt + (int64_t)t.f * 2 * BW2 * MAXR;
  ACC* tcur = tf + ((c0 / BW2) & 1) * BW2 * MAXR;
  ACC* tnext = tf + (((c0 / BW2) + 1) & 1) * BW2 * MAXR;
  const ACC* tcbb = a.tcb + (a.inv2_off[t.f] / ((int64_t)BW2 * BW2) + c0 / BW2) * BW2 * MAXR;
  // entries k of v (and columns of the matrix slice) this CTA needs
  const int klo = BWD ? i0 : 0, khi = BWD ? bw : min(bw, i0 + DR), nk = khi - klo;
  pdl_trigger();
  if (i0 < bw) {
    // the CTA's slice of the inverse, one wave of asynchronous copies
    for (int e = tid; e < nk * DR; e += 256) {
      const int rr = e % DR, k = klo + e / DR;
      cp_async(&Ms[e], &M[(int64_t)k * BW2 + i0 + rr]);
    }
  }
  pdl_wait();
  // rows beyond the block: nothing to compute (uniform per CTA)
  for (int rg = 0; rg < (i0 < bw ? a.nrhs : 0); rg += RG) {
    const int nr = min(RG, a.nrhs - rg);
    __syncthreads();
    {
      // all loads of the slab issued before any is used (nk * RG <= 256 NL)
      constexpr int NL = BW2 * RG / 256;
      ACC v[NL];
#pragma unroll
      for (int u = 0; u < NL; ++u) {
        const int e = tid + 256 * u;
        const int k = klo + e % max(nk, 1), r = e / max(nk, 1);
        v[u] = ACC(0);
        if (e < nk * RG && r < nr) {
          v[u] = xs[(int64_t)(rg + r) * m + c0 + k];
          if (BWD) v[u] -= tcur[k * MAXR + rg + r] + tcbb[k * MAXR + rg + r];
        }
      }
#pragma unroll
      for (int u = 0; u < NL; ++u) {
        const int e = tid + 256 * u;
        if (e < nk * RG) vb[(klo + e % nk) * RG + e / nk] = v[u];
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
        const V* vv = reinterpret_cast<const V*>(vb + k * RG);
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
  if (BWD)
    for (int e = tid; e < DR * MAXR; e += 256) tnext[i0 * MAXR + e] = ACC(0);
}

// rows [r0, r0+32) below the block: xs_i -= L_i,blk y_blk; thread (row,
// 16-column group g), 512 threads.  The 32 x 256 tile of L is staged in shared memory by one wave
// of asynchronous copies; y is read as 16-byte vectors (one broadcast per
// warp).
template <typename T, typename ACC>
__global__ void __launch_bounds__(512) k_fwd_upd3(const LTask* __restrict__ tasks,
                                                  LsArgs<T, ACC> a) {
  constexpr int RG = RGn<ACC>::v;
  using V = typename Vec4<ACC>::V;
  constexpr int VW = Vec4<ACC>::W;
  extern __shared__ __align__(16) unsigned char dsm[];
  T* Lt = reinterpret_cast<T*>(dsm);  // Lt[k*32 + rr] = L(r0 + rr, c0 + k)
  ACC* red = reinterpret_cast<ACC*>(dsm + sizeof(T) * 32 * BW2);  // [16][32][RG + 1]
  __shared__ __align__(16) ACC yb[BW2 * RG];
  const LTask t = tasks[blockIdx.x];
  const FrontDesc f = a.fr[t.f];
  const T* L = a.arena + f.off;
  const int tid = threadIdx.x, rr = tid % 32, g = tid / 32;
  ACC* xs = a.scratch + a.scr_off[t.f] * a.nrhs;
  const ACC* ysl = a.ys + a.scr_off[t.f] * a.nrhs;
  const int nrow = min(32, f.m - t.r0);
  const int cfirst = t.c0, clast = t.c0 + t.bw;
  pdl_trigger();
  for (int rg = 0; rg < a.nrhs; rg += RG) {
    const int nr = min(RG, a.nrhs - rg);
    ACC acc[RG];
#pragma unroll
    for (int q = 0; q < RG; ++q) acc[q] = ACC(0);
    for (int c0 = cfirst; c0 < clast; c0 += BW2) {
      const int bw = min(BW2, clast - c0);
      __syncthreads();  // the previous block's tiles are no longer read
      for (int e = tid; e < BW2 * 32; e += 512) {
        const int r2 = e & 31, k = e >> 5;
        if (k < bw && r2 < nrow) cp_async(&Lt[e], &L[(int64_t)(c0 + k) * f.ld + t.r0 + r2]);
        else Lt[e] = T(0);
      }
      pdl_wait();
      {
        constexpr int NL = BW2 * RG / 512;
        ACC v[NL];
#pragma unroll
        for (int u = 0; u < NL; ++u) {
          const int e = tid + 512 * u, k = e % BW2, r = e / BW2;
          v[u] = (k < bw && r < nr) ? ysl[(int64_t)(rg + r) * f.m + c0 + k] : ACC(0);
        }
#pragma unroll
        for (int u = 0; u < NL; ++u) {
          const int e = tid + 512 * u;
          yb[(e % BW2) * RG + e / BW2] = v[u];
        }
      }
      cp_async_wait_all();
      __syncthreads();
#pragma unroll 8
      for (int kk = 0; kk < 16; ++kk) {
        const int k = g * 16 + kk;
        const ACC l = (ACC)Lt[k * 32 + rr];
        const V* yv = reinterpret_cast<const V*>(yb + k * RG);
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
    for (int e = tid; e < 32 * RG; e += 512) {
      const int r2 = e % 32, q = e / 32, i2 = t.r0 + r2;
      if (r2 < nrow && q < nr) {
        ACC sum = ACC(0);
#pragma unroll
        for (int gg = 0; gg < 16; ++gg) sum += red[(gg * 32 + r2) * (RG + 1) + q];
        xs[(int64_t)(rg + q) * f.m + i2] -= sum;
      }
    }
    __syncthreads();
  }
}

// rows [r0, r0+BR) contribute tt[k][r] += sum_i L(i, c0+k) xs(i, r), k < bw.
// The BR x 256 tile of L is staged in shared memory by one wave of
// asynchronous copies; thread (column k = tid % 256, row half h = tid / 256),
// 512 threads, the halves reduced through shared memory.  Every CTA of a
// step adds into the same accumulator, so taller tiles mean fewer atomics
// per address.
template <typename T, typename ACC>
__global__ void __launch_bounds__(512) k_bwd_red3(const LTask* __restrict__ tasks,
                                                  LsArgs<T, ACC> a) {
  constexpr int RG = RGn<ACC>::v;
  using V = typename Vec4<ACC>::V;
  constexpr int VW = Vec4<ACC>::W;
  extern __shared__ __align__(16) unsigned char dsm[];
  constexpr int BR = BRED_ROWS;
  T* Lt = reinterpret_cast<T*>(dsm);  // Lt[ii*(BW2+1) + k] = L(r0 + ii, c0 + k)
  ACC* half = reinterpret_cast<ACC*>(dsm + sizeof(T) * BR * (BW2 + 1));  // [BW2][RG + 1]
  __shared__ __align__(16) ACC xt[BR][RG];
  const LTask t = tasks[blockIdx.x];
  const FrontDesc f = a.fr[t.f];
  const T* L = a.arena + f.off;
  const int c0 = t.c0, bw = t.bw, tid = threadIdx.x, k = tid % BW2, h = tid / BW2;
  // rows below the block: solved rows (< n) in ys, contribution rows in xs
  const ACC* xs = a.scratch + a.scr_off[t.f] * a.nrhs;
  const ACC* ysl = a.ys + a.scr_off[t.f] * a.nrhs;
  ACC* tf = a.tt + ((int64_t)t.f * 2 + ((c0 / BW2) & 1)) * BW2 * MAXR;
  // fully-summed rows [r0, n) only; the contribution rows' share comes from
  // k_bwd_cb
  const int nrow = min(BR, f.n - t.r0);
  pdl_trigger();
  for (int e = tid; e < BR * BW2; e += 512) {
    const int ii = e % BR, kk = e / BR;
    T* dst = &Lt[ii * (BW2 + 1) + kk];
    if (ii < nrow && kk < bw) cp_async(dst, &L[(int64_t)(c0 + kk) * f.ld + t.r0 + ii]);
    else *dst = T(0);
  }
  pdl_wait();
  for (int rg = 0; rg < a.nrhs; rg += RG) {
    const int nr = min(RG, a.nrhs - rg);
    ACC acc[RG];
#pragma unroll
    for (int q = 0; q < RG; ++q) acc[q] = ACC(0);
    for (int e = tid; e < BR * RG; e += blockDim.x) {
      const int ii = e % BR, r = e / BR, row = t.r0 + ii;
      const ACC* src = (row < f.n) ? ysl : xs;
      xt[ii][r] = (ii < nrow && r < nr) ? src[(int64_t)(rg + r) * f.m + row] : ACC(0);
    }
    cp_async_wait_all();
    __syncthreads();
#pragma unroll 8
    for (int i2 = 0; i2 < BR / 2; ++i2) {
      const int ii = h * (BR / 2) + i2;
      const ACC l = (ACC)Lt[ii * (BW2 + 1) + k];
      const V* xv = reinterpret_cast<const V*>(&xt[ii][0]);
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
    if (h == 1)
#pragma unroll
      for (int q = 0; q < RG; ++q) half[k * (RG + 1) + q] = acc[q];
    __syncthreads();
    if (h == 0 && k < bw)
#pragma unroll
      for (int q = 0; q < RG; ++q)
        if (q < nr) aadd(&tf[k * MAXR + rg + q], acc[q] + half[k * (RG + 1) + q]);
    __syncthreads();
  }
}

// Contribution rows of a front, backward: their share of block c0's
// reduction, tcb(k, r) += sum_i L(i, c0+k) x(i, r) over the CB_CHUNK rows
// [r0, r0 + CB_CHUNK) >= n, in 32-row sub-tiles staged with double-buffered
// cp.async; one set of atomics per CTA.  Thread (column k = tid % 256, row
// half h = tid / 256), 512 threads.
template <typename T, typename ACC>
__global__ void __launch_bounds__(512) k_bwd_cb(const LTask* __restrict__ tasks,
                                                LsArgs<T, ACC> a) {
  constexpr int RG = RGn<ACC>::v;
  constexpr int SR = 32;
  using V = typename Vec4<ACC>::V;
  constexpr int VW = Vec4<ACC>::W;
  extern __shared__ __align__(16) unsigned char dsm[];
  T* Lt = reinterpret_cast<T*>(dsm);  // [2][SR*(BW2+1)]
  ACC* xt = reinterpret_cast<ACC*>(dsm + sizeof(T) * 2 * SR * (BW2 + 1));  // [2][SR*RG]
  ACC* half = xt + 2 * SR * RG;       // [BW2][RG + 1]
  const LTask t = tasks[blockIdx.x];
  const FrontDesc f = a.fr[t.f];
  const T* L = a.arena + f.off;
  const int c0 = t.c0, bw = t.bw, tid = threadIdx.x, k = tid % BW2, h = tid / BW2;
  const ACC* xs = a.scratch + a.scr_off[t.f] * a.nrhs;
  ACC* tf = a.tcb + (a.inv2_off[t.f] / ((int64_t)BW2 * BW2) + c0 / BW2) * BW2 * MAXR;
  const int rend = min(t.r0 + CB_CHUNK, f.m);
  const int nsub = (rend - t.r0 + SR - 1) / SR;
  for (int rg = 0; rg < a.nrhs; rg += RG) {
    const int nr = min(RG, a.nrhs - rg);
    ACC acc[RG];
#pragma unroll
    for (int q = 0; q < RG; ++q) acc[q] = ACC(0);
    auto issue = [&](int sub, int buf) {
      const int s0 = t.r0 + sub * SR, nrow = min(SR, rend - s0);
      T* dst = Lt + buf * SR * (BW2 + 1);
      for (int e = tid; e < SR * BW2; e += 512) {
        const int ii = e % SR, kk = e / SR;
        T* d = &dst[ii * (BW2 + 1) + kk];
        if (ii < nrow && kk < bw) cp_async(d, &L[(int64_t)(c0 + kk) * f.ld + s0 + ii]);
        else *d = T(0);
      }
      ACC* xd = xt + buf * SR * RG;
      for (int e = tid; e < SR * RG; e += 512) {
        const int ii = e % SR, r = e / SR;
        if (ii < nrow && r < nr) cp_async(&xd[ii * RG + r], &xs[(int64_t)(rg + r) * f.m + s0 + ii]);
        else xd[ii * RG + r] = ACC(0);
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
    };
    __syncthreads();
    issue(0, 0);
    for (int sub = 0; sub < nsub; ++sub) {
      const int buf = sub & 1;
      if (sub + 1 < nsub) {
        issue(sub + 1, buf ^ 1);
        asm volatile("cp.async.wait_group 1;" ::: "memory");
      } else {
        asm volatile("cp.async.wait_group 0;" ::: "memory");
      }
      __syncthreads();
      const T* lt = Lt + buf * SR * (BW2 + 1);
      const ACC* xb = xt + buf * SR * RG;
#pragma unroll 8
      for (int i2 = 0; i2 < SR / 2; ++i2) {
        const int ii = h * (SR / 2) + i2;
        const ACC l = (ACC)lt[ii * (BW2 + 1) + k];
        const V* xv = reinterpret_cast<const V*>(&xb[ii * RG]);
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
      __syncthreads();  // buffer buf is read; the next issue may overwrite it
    }
    if (h == 1)
#pragma unroll
      for (int q = 0; q < RG; ++q) half[k * (RG + 1) + q] = acc[q];
    __syncthreads();
    if (h == 0 && k < bw)
#pragma unroll
      for (int q = 0; q < RG; ++q)
        if (q < nr) aadd(&tf[k * MAXR + rg + q], acc[q] + half[k * (RG + 1) + q]);
  }
}

inline int nblocks(int64_t count, int bs) { return (int)((count + bs - 1) / bs); }

// dynamic shared memory of the staged solve-step kernels
template <typename T> constexpr size_t diag_mv_smem() {
  return sizeof(T) * DMV_ROWS * BW2 + sizeof(T) * 256 * (RGn<T>::v + 1);
}
template <typename T> constexpr size_t fwd_upd_smem() {
  return sizeof(T) * 32 * BW2 + sizeof(T) * 16 * 32 * (RGn<T>::v + 1);
}
template <typename T> constexpr size_t bwd_cb_smem() {
  return sizeof(T) * 2 * 32 * (BW2 + 1) + sizeof(T) * (2 * 32 * RGn<T>::v + BW2 * (RGn<T>::v + 1));
}
template <typename T> constexpr size_t bwd_red_smem() {
  return sizeof(T) * BRED_ROWS * (BW2 + 1) + sizeof(T) * BW2 * (RGn<T>::v + 1);
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

template <typename ACC>
size_t small_solve_smem(int maxm, int nrhs) {
  return (size_t)maxm * nrhs * sizeof(ACC) + (size_t)maxm * sizeof(int);
}

template <typename T, typename ACC>
bool launch_solve_small(bool fwd, const T* arena, const FrontDesc* fr, int nfronts,
                        const int* rlist, ACC* x, int n, int nrhs, int maxm, bool unit_diag,
                        cudaStream_t s) {
  const size_t sm = small_solve_smem<ACC>(maxm, nrhs);
  if (sm > SMALL_SOLVE_SMEM || nrhs > MAXR) return false;
  if (nfronts <= 0) return true;
  if (fwd)
    k_solve_fwd_s<T, ACC><<<nfronts, 256, sm, s>>>(arena, fr, rlist, x, n, nrhs, unit_diag);
  else
    k_solve_bwd_s<T, ACC><<<nfronts, 256, sm, s>>>(arena, fr, rlist, x, n, nrhs, unit_diag);
  return true;
}

template <typename T, typename ACC>
void launch_solve_bwd(const T* arena, const FrontDesc* fr, int nfronts, const int* rlist,
                      ACC* x, int n, int nrhs, ACC* scratch, const int64_t* scr_off,
                      bool unit_diag, cudaStream_t s) {
  if (nfronts <= 0) return;
  if (nrhs > MAXR) throw CudaError("solve: more than 32 right-hand sides per launch");
  k_solve_bwd<T, ACC><<<nfronts, 256, 0, s>>>(arena, fr, rlist, x, n, nrhs, scratch, scr_off,
                                              unit_diag);
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
void launch_lsolve(int kind, const LTask* tasks, int ntask, LsArgs<T, ACC> a, cudaStream_t s) {
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
      launch_pdl(k_diag_mv<T, ACC, false>, dim3(ntask, BW2 / DMV_ROWS), 256, diag_mv_smem<T>(), s,
                 tasks, a);
      break;
    case LS_FWD_UPD2:
      launch_pdl(k_fwd_upd3<T, ACC>, dim3(ntask), 512, fwd_upd_smem<T>(), s, tasks, a);
      break;
    case LS_BWD_CB:
      k_bwd_cb<T, ACC><<<ntask, 512, bwd_cb_smem<T>(), s>>>(tasks, a);
      break;
    case LS_FWD_ROWS:
      k_fwd_rows<T, ACC><<<ntask, LSOLVE_ROWS_T, 0, s>>>(tasks, a);
      break;
    case LS_BWD_RED2:
      launch_pdl(k_bwd_red3<T, ACC>, dim3(ntask), 512, bwd_red_smem<T>(), s, tasks, a);
      break;
    case LS_BWD_DIAG2:
      launch_pdl(k_diag_mv<T, ACC, true>, dim3(ntask, BW2 / DMV_ROWS), 256, diag_mv_smem<T>(), s,
                 tasks, a);
      break;
  }
}

template <typename T>
void launch_inv_diag(const T* arena, const FrontDesc* fr, const LTask* tasks, int ntask,
                     T* inv, const int64_t* inv_off, bool unit, cudaStream_t s) {
  if (ntask <= 0) return;
  k_inv_diag<T><<<ntask, LB, 0, s>>>(arena, fr, tasks, inv, inv_off, unit);
}

template <typename T>
void prepare_solve_kernels() {
  SG_CUDA(cudaFuncSetAttribute(k_inv256<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(2 * 64 * 65 * sizeof(T))));
  SG_CUDA(cudaFuncSetAttribute(k_diag_mv<T, T, false>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)diag_mv_smem<T>()));
  SG_CUDA(cudaFuncSetAttribute(k_diag_mv<T, T, true>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)diag_mv_smem<T>()));
  SG_CUDA(cudaFuncSetAttribute(k_solve_fwd_s<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)SMALL_SOLVE_SMEM));
  SG_CUDA(cudaFuncSetAttribute(k_solve_bwd_s<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)SMALL_SOLVE_SMEM));
  SG_CUDA(cudaFuncSetAttribute(k_fwd_upd3<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)fwd_upd_smem<T>()));
  SG_CUDA(cudaFuncSetAttribute(k_bwd_red3<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)bwd_red_smem<T>()));
  SG_CUDA(cudaFuncSetAttribute(k_bwd_cb<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)bwd_cb_smem<T>()));
}

template <typename T>
void launch_inv256(const T* arena, const FrontDesc* fr, const LTask* tasks, int ntask,
                   const T* inv64, const int64_t* inv_off, T* inv2, T* inv2t,
                   const int64_t* inv2_off, cudaStream_t s) {
  if (ntask <= 0) return;
  k_inv256<T><<<ntask, 256, 2 * 64 * 65 * sizeof(T), s>>>(arena, fr, tasks, inv64, inv_off,
                                                           inv2, inv2t, inv2_off);
}
template void prepare_solve_kernels<float>();
template void prepare_solve_kernels<double>();
template void launch_inv256<float>(const float*, const FrontDesc*, const LTask*, int,
                                   const float*, const int64_t*, float*, float*,
                                   const int64_t*, cudaStream_t);
template void launch_inv256<double>(const double*, const FrontDesc*, const LTask*, int,
                                    const double*, const int64_t*, double*, double*,
                                    const int64_t*, cudaStream_t);

template void launch_lsolve<float, float>(int, const LTask*, int, LsArgs<float, float>,
                                          cudaStream_t);
template void launch_lsolve<double, double>(int, const LTask*, int, LsArgs<double, double>,
                                            cudaStream_t);
template void launch_inv_diag<float>(const float*, const FrontDesc*, const LTask*, int, float*,
                                     const int64_t*, bool, cudaStream_t);
template void launch_inv_diag<double>(const double*, const FrontDesc*, const LTask*, int,
                                      double*, const int64_t*, bool, cudaStream_t);
template void launch_solve_fwd<float, float>(const float*, const FrontDesc*, int, const int*,
                                             float*, int, int, float*, const int64_t*, bool,
                                             cudaStream_t);
template void launch_solve_bwd<float, float>(const float*, const FrontDesc*, int, const int*,
                                             float*, int, int, float*, const int64_t*, bool,
                                             cudaStream_t);
template void launch_solve_fwd<double, double>(const double*, const FrontDesc*, int,
                                               const int*, double*, int, int, double*,
                                               const int64_t*, bool, cudaStream_t);
template void launch_solve_bwd<double, double>(const double*, const FrontDesc*, int,
                                               const int*, double*, int, int, double*,
                                               const int64_t*, bool, cudaStream_t);
template bool launch_solve_small<float, float>(bool, const float*, const FrontDesc*, int,
                                               const int*, float*, int, int, int, bool,
                                               cudaStream_t);
template bool launch_solve_small<double, double>(bool, const double*, const FrontDesc*, int,
                                                 const int*, double*, int, int, int, bool,
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
