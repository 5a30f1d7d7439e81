// Blocked Cholesky of the fully-summed columns of large FP32 fronts.
//
// The fully-summed columns are eliminated in outer panels of up to 256
// columns.  Inside a panel, steps of 64 columns run two kernels:
//   k_blk_diag  (one CTA per front): the 64-column block column of the panel
//               (the 64 x 64 diagonal block and the panel rows below it,
//               at most 256 rows, held in shared memory) factorised in four
//               sub-steps of 16 columns: one warp factorises the 16 x 16
//               diagonal sub-block in registers and inverts it, all threads
//               solve the rows below with that inverse and update the rest
//               of the block column;
//   k_blk_panel (one CTA per 64 rows below the block): the rows below the
//               panel solve L_R L11^T = A_R by the same four sub-steps (with
//               L11 and the 16 x 16 inverses from k_blk_diag), then every row
//               applies the in-panel update A(R, J) -= L_R L_J^T.
// The trailing update of the remaining fully-summed columns after each
// outer panel (K = panel width) and the contribution-block update (K = n)
// run on the tensor cores (k_update_tc), so the SIMT kernels here only touch
// one panel at a time.
//
// Reference behaviour replaced: factorize_diag_block, solve_block,
// update_block and update_diag_block (src/kernels/factor.hxx:56-260) as
// driven by factor_front_posdef (src/factor.hxx:19-148).  The triangular
// solves multiply by the explicit inverses of 16 x 16 diagonal sub-blocks
// (a block forward substitution), which keeps their error at the level of
// a plain substitution.
#include "device.hpp"

namespace sylver_gb300 {

namespace {

constexpr int BB = BLK_B;        // block column width (64)
constexpr int SB = 16;           // sub-block width
constexpr int NSB = BB / SB;     // sub-blocks per block column
constexpr int PR = BLK_W;        // most rows of a block column inside a panel
constexpr int PLD = PR + 1;      // shared leading dimension of the block column
constexpr int BLD = BB + 1;
constexpr int BJ = BLK_W - BB;   // most panel rows below a diagonal block
constexpr int BJP = BJ + 1;
constexpr int XSZ = NSB * SB * SB;  // floats of the four sub-block inverses

// One warp: Cholesky of the 16 x 16 sub-block (rows/cols q0.. of the shared
// block column P, leading dimension pld) in registers, lane i < 16 holding
// row i; writes L back, and X = L^-1 into xs (xs[i*SB + j] = X(i, j)) and
// xg (global, xg[j*SB + i] = X(i, j)).  A non-positive pivot is replaced by
// one (and reported when it lies inside the bw real columns).
__device__ __noinline__ void warp_chol16(float* __restrict__ P, int pld, int q0, int bwreal,
                                            float* __restrict__ xs, float* __restrict__ xg,
                                            unsigned* __restrict__ status) {
  const int lane = threadIdx.x & 31;
  const int li = lane & (SB - 1);
  float a[SB];
#pragma unroll
  for (int k = 0; k < SB; ++k) a[k] = (k <= li) ? P[(q0 + k) * pld + q0 + li] : 0.f;
  bool bad = false;
#pragma unroll
  for (int k = 0; k < SB; ++k) {
    float d = __shfl_sync(0xffffffffu, a[k], k);
    if (!(d > 0.f)) {
      if (q0 + k < bwreal) bad = true;
      d = 1.f;
    }
    const float piv = sqrtf(d);
    if (li == k) a[k] = piv;
    else if (li > k) a[k] = a[k] / piv;
#pragma unroll
    for (int j = k + 1; j < SB; ++j) {
      const float ljk = __shfl_sync(0xffffffffu, a[k], j);
      if (li >= j) a[j] = fmaf(-a[k], ljk, a[j]);
    }
  }
  if (lane < SB) {
#pragma unroll
    for (int k = 0; k < SB; ++k)
      if (k <= li) P[(q0 + k) * pld + q0 + li] = a[k];
  }
  if (lane == 0 && bad) atomicOr(status, ST_NOT_POSDEF);
  // column li of X: X(i, li) = (delta - sum_{k<i} L(i,k) X(k, li)) / L(i, i)
  float x[SB];
#pragma unroll
  for (int i = 0; i < SB; ++i) {
    float v = (i == li) ? 1.f : 0.f;
#pragma unroll
    for (int k = 0; k < i; ++k) v = fmaf(-__shfl_sync(0xffffffffu, a[k], i), x[k], v);
    x[i] = v / __shfl_sync(0xffffffffu, a[i], i);
  }
  if (lane < SB) {
#pragma unroll
    for (int i = 0; i < SB; ++i) {
      xs[i * SB + li] = x[i];
      xg[li * SB + i] = x[i];
    }
  }
}

__global__ void __launch_bounds__(256) k_blk_diag(float* __restrict__ arena,
                                                  const BlkTask* __restrict__ tasks,
                                                  float* __restrict__ xinv,
                                                  unsigned* __restrict__ status) {
  extern __shared__ __align__(16) float sm[];
  float* P = sm;              // P[j*PLD + r] = A(c + r, c + j), then L
  float* Xs = P + BB * PLD;   // four 16 x 16 inverses, Xs[p*256 + i*16 + j] = X_p(i, j)
  const BlkTask t = tasks[blockIdx.x];
  float* a = arena + t.off;
  const int64_t ld = t.ld;
  const int c = t.c, bw = t.bw, tid = threadIdx.x;
  const int nrows = t.pend - c;          // bw + panel rows below the block
  const int NR = max(nrows, BB);         // rows beyond a ragged block: identity
  float* xg = xinv + (int64_t)t.xi * XSZ;
  for (int e = tid; e < BB * NR; e += 256) {
    const int r = e % NR, j = e / NR;
    if (j < bw && r < nrows && r >= j) cp_async(&P[j * PLD + r], &a[(int64_t)(c + j) * ld + c + r]);
    else P[j * PLD + r] = (j < bw && r < nrows) ? 0.f : (r == j ? 1.f : 0.f);
  }
  cp_async_wait_all();
  __syncthreads();
  for (int p = 0; p < NSB; ++p) {
    const int q0 = p * SB;
    if (q0 >= bw) break;  // uniform
    if (tid < 32) warp_chol16(P, PLD, q0, bw, Xs + p * SB * SB, xg + p * SB * SB, status);
    __syncthreads();
    // rows below the sub-block: L(r, q0:q0+16) = A(r, q0:q0+16) X_p^T
    const float* X = Xs + p * SB * SB;
    for (int r = q0 + SB + tid; r < NR; r += 256) {
      float v[SB];
#pragma unroll
      for (int k = 0; k < SB; ++k) v[k] = P[(q0 + k) * PLD + r];
#pragma unroll
      for (int j = 0; j < SB; ++j) {
        float o = 0.f;
#pragma unroll
        for (int k = 0; k <= j; ++k) o = fmaf(v[k], X[j * SB + k], o);
        P[(q0 + j) * PLD + r] = o;
      }
    }
    __syncthreads();
    // rest of the block column: A(r, cc) -= L(r, q0:+16) L(cc, q0:+16)^T,
    // cc in [q0+16, 64), r >= cc; thread (row r0 + tid%64 + 64s, column
    // group tid/64: cc = q0 + 16 + g + 4u)
    const int c1 = q0 + SB;
    if (c1 < bw) {
      const int g = tid >> 6;
      for (int r = c1 + (tid & 63); r < NR; r += 64) {
        float lr[SB];
#pragma unroll
        for (int k = 0; k < SB; ++k) lr[k] = P[(q0 + k) * PLD + r];
#pragma unroll
        for (int u = 0; u < (BB - SB) / 4; ++u) {
          const int cc = c1 + g + 4 * u;
          if (cc < bw && cc <= r) {
            float s = 0.f;
#pragma unroll
            for (int k = 0; k < SB; ++k) s = fmaf(lr[k], P[(q0 + k) * PLD + cc], s);
            P[cc * PLD + r] -= s;
          }
        }
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < BB * nrows; e += 256) {
    const int r = e % nrows, j = e / nrows;
    if (j < bw && r >= j) a[(int64_t)(c + j) * ld + c + r] = P[j * PLD + r];
  }
}

__global__ void __launch_bounds__(256, 2) k_blk_panel(float* __restrict__ arena,
                                                   const BlkTask* __restrict__ tasks,
                                                   const float* __restrict__ xinv) {
  extern __shared__ __align__(16) float sm[];
  float* L11 = sm;              // L11[k*BLD + i] = L(c+i, c+k)
  float* Xs = L11 + BB * BLD;   // Xs[p*256 + j*16 + i] = X_p(i, j)
  float* Lr = Xs + XSZ;         // Lr[k*BLD + r]: A, then L, of this CTA's rows
  float* LJ = Lr + BB * BLD;    // LJ[k*BJP + j] = L(cb + j, c + k)
  const BlkTask t = tasks[blockIdx.x];
  float* a = arena + t.off;
  const int64_t ld = t.ld;
  const int c = t.c, bw = t.bw, cb = c + bw, pend = t.pend, r0 = t.r0, tid = threadIdx.x;
  const int nr = min(BB, t.m - r0);
  const int nJ = pend - cb;
  const bool solve = r0 + nr > pend;  // some rows lie below the panel
  if (solve) {
    for (int e = tid; e < BB * BB; e += 256) {
      const int i = e % BB, k = e / BB;
      if (i < bw && k < bw && i >= k) cp_async(&L11[k * BLD + i], &a[(int64_t)(c + k) * ld + c + i]);
      else L11[k * BLD + i] = (i == k) ? 1.f : 0.f;
    }
    const float* xg = xinv + (int64_t)t.xi * XSZ;
    for (int e = tid; e < XSZ; e += 256) cp_async(&Xs[e], &xg[e]);
  }
  for (int e = tid; e < BB * BB; e += 256) {
    const int r = e % BB, k = e / BB;
    if (r < nr && k < bw) cp_async(&Lr[k * BLD + r], &a[(int64_t)(c + k) * ld + r0 + r]);
    else Lr[k * BLD + r] = 0.f;
  }
  for (int e = tid; e < BB * nJ; e += 256) {
    const int j = e % nJ, k = e / nJ;
    if (k < bw) cp_async(&LJ[k * BJP + j], &a[(int64_t)(c + k) * ld + cb + j]);
    else LJ[k * BJP + j] = 0.f;
  }
  cp_async_wait_all();
  __syncthreads();
  if (solve) {
    // block forward substitution over the four sub-blocks; thread (row
    // tid%64, four columns 4*(tid/64) .. +3 of the sub-block)
    const int r = tid & 63, j0 = 4 * (tid >> 6);
    const bool mine = r0 + r >= pend && r < nr;  // rows inside the panel already hold L
    for (int p = 0; p < NSB; ++p) {
      const int q0 = p * SB;
      if (q0 >= bw) break;
      float v[4];
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        float s = Lr[(q0 + j0 + jj) * BLD + r];
        for (int k = 0; k < q0; ++k) s = fmaf(-Lr[k * BLD + r], L11[k * BLD + q0 + j0 + jj], s);
        v[jj] = s;
      }
      __syncthreads();
      if (mine)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) Lr[(q0 + j0 + jj) * BLD + r] = v[jj];
      __syncthreads();
      const float* X = Xs + p * SB * SB;
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        const int j = j0 + jj;
        float o = 0.f;
        for (int k = 0; k <= j; ++k) o = fmaf(Lr[(q0 + k) * BLD + r], X[k * SB + j], o);
        v[jj] = o;
      }
      __syncthreads();
      if (mine)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          Lr[(q0 + j0 + jj) * BLD + r] = v[jj];
          if (q0 + j0 + jj < bw) a[(int64_t)(c + q0 + j0 + jj) * ld + r0 + r] = v[jj];
        }
      __syncthreads();
    }
  }
  if (nJ <= 0) return;
  // A(r0 + r, cb + j) -= sum_k L(r0 + r, c + k) L(cb + j, c + k), lower part
  const int rr = tid & 15, cc = tid >> 4;
  constexpr int NV = BJ / 16;
  float acc[4][NV];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[u][v] = 0.f;
  const int nv = (nJ + 15) / 16;
  // the entries to update, loaded up front so their latency overlaps the
  // products
  float cval[4][NV];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const int r = rr + 16 * u, j = cc + 16 * v;
      cval[u][v] = (v < nv && r < nr && j < nJ && r0 + r >= cb + j)
                       ? a[(int64_t)(cb + j) * ld + r0 + r] : 0.f;
    }
#pragma unroll 4
  for (int k = 0; k < BB; ++k) {
    float av[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) av[u] = Lr[k * BLD + rr + 16 * u];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      if (v < nv) {
        const float b = LJ[k * BJP + cc + 16 * v];
#pragma unroll
        for (int u = 0; u < 4; ++u) acc[u][v] = fmaf(av[u], b, acc[u][v]);
      }
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const int r = rr + 16 * u, j = cc + 16 * v;
      if (r < nr && j < nJ && r0 + r >= cb + j)
        a[(int64_t)(cb + j) * ld + r0 + r] = cval[u][v] - acc[u][v];
    }
}

constexpr size_t diag_smem() { return sizeof(float) * ((size_t)BB * PLD + XSZ); }
constexpr size_t panel_smem() { return sizeof(float) * (2 * BB * BLD + XSZ + BB * BJP); }

}  // namespace

void prepare_blocked_kernels() {
  SG_CUDA(cudaFuncSetAttribute(k_blk_diag, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)diag_smem()));
  SG_CUDA(cudaFuncSetAttribute(k_blk_panel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)panel_smem()));
}

void launch_blk_diag(float* arena, const BlkTask* t, int ntask, float* xinv, unsigned* status,
                     cudaStream_t s) {
  if (ntask <= 0) return;
  k_blk_diag<<<ntask, 256, diag_smem(), s>>>(arena, t, xinv, status);
}

void launch_blk_panel(float* arena, const BlkTask* t, int ntask, const float* xinv,
                      cudaStream_t s) {
  if (ntask <= 0) return;
  k_blk_panel<<<ntask, 256, panel_smem(), s>>>(arena, t, xinv);
}

}  // namespace sylver_gb300
