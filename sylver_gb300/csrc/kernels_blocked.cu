// Blocked Cholesky of the fully-summed columns of large FP32 fronts.
//
// The fully-summed columns are eliminated in outer panels of W <= 256
// columns, each in four launches:
//   k_blk_diag  (one CTA per front): Cholesky of the panel's W x W diagonal
//               block, held packed in shared memory, in sub-steps of 16
//               columns: one warp factorises the 16 x 16 diagonal sub-block in
//               registers and inverts it, all threads solve the rows below it
//               with that inverse and update the next sub-block column, and
//               while warp 0 factorises that one the other warps update the
//               rest of the trailing triangle in 32 x 32 register tiles;
//   k_blk_panel (one CTA per 64 rows below the panel): those rows solve
//               L_R L_WW^T = A_R by block forward substitution over the same
//               16-column sub-blocks (the 16 x 16 inverses come from
//               k_blk_diag);
//   k_update_tc: the trailing fully-summed columns are updated with K = W
//               on the tensor cores; its operands (the rows below the panel,
//               transposed and split into three BF16 parts) are written by
//               k_blk_panel.
// After the last panel the contribution block gets one update with K = n on
// the tensor cores as well.
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

constexpr int PW = BLK_W;         // widest panel (256)
constexpr int SB = 16;            // sub-block width
constexpr int NSBMAX = PW / SB;   // sub-blocks of the widest panel
constexpr int XSZ = NSBMAX * SB * SB;  // floats of the sub-block inverses of one panel
constexpr int TLD = SB + 1;
constexpr int DTHREADS = 512;
constexpr int PTHREADS = 256;
constexpr int ALD = 64 + 1;       // rows of one panel-kernel CTA (+1)

// start of column j of a packed lower triangle with PW rows
__device__ __forceinline__ int pcol(int j) { return j * PW - (j * (j - 1)) / 2; }
// (i, j), i >= j, of the packed lower triangle
__device__ __forceinline__ int pidx(int i, int j) { return pcol(j) + i - j; }

// One warp: Cholesky of the 16 x 16 tile T (T[j*TLD + i] = A(i, j), lower)
// in registers, lane i < 16 holding row i; writes L back to T and X = L^-1
// to xs (xs[i*SB + j] = X(i, j)) and xg (global, xg[j*SB + i] = X(i, j)).
// A non-positive pivot is replaced by one and reported when its column is
// below bwreal.
__device__ __noinline__ void warp_chol16(float* __restrict__ T, int q0, int bwreal,
                                         float* __restrict__ xs, float* __restrict__ xg,
                                         unsigned* __restrict__ status) {
  const int lane = threadIdx.x & 31;
  const int li = lane & (SB - 1);
  float a[SB], rinv[SB];
#pragma unroll
  for (int k = 0; k < SB; ++k) a[k] = (k <= li) ? T[k * TLD + li] : 0.f;
  bool bad = false;
  // The pivot chain is the critical path of the panel: 1/sqrt(d) comes from
  // the hardware estimate refined by one Newton step (about 1 ulp), and
  // both the column scaling and the inverse multiply by it -- IEEE sqrt and
  // division cost three times as long per 16 columns.
#pragma unroll
  for (int k = 0; k < SB; ++k) {
    float d = __shfl_sync(0xffffffffu, a[k], k);
    if (!(d > 0.f)) {
      if (q0 + k < bwreal) bad = true;
      d = 1.f;
    }
    float r = rsqrtf(d);
    r = r * fmaf(-0.5f * d * r, r, 1.5f);
    rinv[k] = r;
    if (li == k) a[k] = d * r;
    else if (li > k) a[k] = a[k] * r;
#pragma unroll
    for (int j = k + 1; j < SB; ++j) {
      const float ljk = __shfl_sync(0xffffffffu, a[k], j);
      if (li >= j) a[j] = fmaf(-a[k], ljk, a[j]);
    }
  }
  if (lane < SB) {
#pragma unroll
    for (int k = 0; k < SB; ++k)
      if (k <= li) T[k * TLD + li] = a[k];
  }
  if (lane == 0 && bad) atomicOr(status, ST_NOT_POSDEF);
  // column li of X: X(i, li) = (delta - sum_{k<i} L(i,k) X(k, li)) / L(i, i)
  float x[SB];
#pragma unroll
  for (int i = 0; i < SB; ++i) {
    float v = (i == li) ? 1.f : 0.f;
#pragma unroll
    for (int k = 0; k < i; ++k) v = fmaf(-__shfl_sync(0xffffffffu, a[k], i), x[k], v);
    x[i] = v * rinv[i];
  }
  if (lane < SB) {
#pragma unroll
    for (int i = 0; i < SB; ++i) {
      xs[i * SB + li] = x[i];
      xg[li * SB + i] = x[i];
    }
  }
}

__global__ void __launch_bounds__(DTHREADS) k_blk_diag(float* __restrict__ arena,
                                                       const BlkTask* __restrict__ tasks,
                                                       float* __restrict__ xinv,
                                                       unsigned* __restrict__ status) {
  extern __shared__ __align__(16) float sm[];
  float* Lp = sm;                      // packed lower triangle, PW rows
  float* Xs = Lp + PW * (PW + 1) / 2;  // inverse of the current sub-block
  float* T = Xs + SB * SB;             // 16 x 16 sub-block for the warp
  const BlkTask t = tasks[blockIdx.x];
  float* a = arena + t.off;
  const int64_t ld = t.ld;
  const int k0 = t.c, w = t.bw, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wp = (w + SB - 1) / SB * SB;  // rows/cols beyond w: identity
  float* xg = xinv + (int64_t)t.xi * XSZ;
  for (int j = warp; j < wp; j += DTHREADS / 32) {
    float* col = Lp + pcol(j) - j;
    for (int i = j + lane; i < wp; i += 32) {
      if (i < w && j < w) cp_async(&col[i], &a[(int64_t)(k0 + j) * ld + k0 + i]);
      else col[i] = (i == j) ? 1.f : 0.f;
    }
  }
  cp_async_wait_all();
  __syncthreads();
  // (a) one warp factorises and inverts the 16 x 16 diagonal sub-block at q
  auto factor_sub = [&](int q) {
    for (int e = lane; e < SB * SB; e += 32) {
      const int i = e % SB, k = e / SB;
      T[k * TLD + i] = (i >= k) ? Lp[pidx(q + i, q + k)] : 0.f;
    }
    __syncwarp();
    warp_chol16(T, q, w, Xs, xg + (q / SB) * SB * SB, status);
    __syncwarp();
    for (int e = lane; e < SB * SB; e += 32) {
      const int i = e % SB, k = e / SB;
      if (i >= k) Lp[pidx(q + i, q + k)] = T[k * TLD + i];
    }
  };
  if (warp == 0) factor_sub(0);
  __syncthreads();
  // Lookahead: after the rows below sub-block q0 are solved (b), the next
  // sub-block column is updated first (c1); warp 0 then factorises it while
  // the other warps update the rest of the trailing triangle (c2), so the
  // serial pivot chain overlaps the update.
  for (int q0 = 0; q0 < wp; q0 += SB) {
    const int c1 = q0 + SB;
    if (c1 >= wp) break;
    // (b) rows below: L(r, q0:+16) = A(r, q0:+16) X^T, one thread per row
    for (int r = c1 + tid; r < wp; r += DTHREADS) {
      float v[SB];
#pragma unroll
      for (int k = 0; k < SB; ++k) v[k] = Lp[pidx(r, q0 + k)];
#pragma unroll
      for (int j = 0; j < SB; ++j) {
        float o = 0.f;
#pragma unroll
        for (int k = 0; k <= j; ++k) o = fmaf(v[k], Xs[j * SB + k], o);
        Lp[pidx(r, q0 + j)] = o;
      }
    }
    __syncthreads();
    // (c1) the next sub-block column: rows [c1, wp) x cols [c1, c1 + 16);
    // thread (row c1 + tid % 256, eight columns c1 + 8 * (tid / 256) ..)
    {
      const int r = c1 + (tid & 255), cbase = c1 + 8 * (tid >> 8);
      if (r < wp) {
        float lr[SB];
#pragma unroll
        for (int k = 0; k < SB; ++k) lr[k] = Lp[pidx(r, q0 + k)];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int cc = cbase + u;
          if (cc <= r) {
            float sacc = 0.f;
#pragma unroll
            for (int k = 0; k < SB; ++k) sacc = fmaf(lr[k], Lp[pidx(cc, q0 + k)], sacc);
            Lp[pidx(r, cc)] -= sacc;
          }
        }
      }
    }
    __syncthreads();
    if (warp == 0) {
      factor_sub(c1);
    } else {
      // (c2) trailing triangle [c2s, wp)^2 -= L(:, q0:+16) L(:, q0:+16)^T in
      // 32 x 32 tiles, one warp per tile (warps 1..); lane owns rows
      // r0 + (lane&7) + 8u (u < 4) and columns cc0 + (lane>>3) + 4v (v < 8)
      const int c2s = c1 + SB;
      const int nt = (wp - c2s + 31) / 32;
      for (int tile = warp - 1; tile < nt * (nt + 1) / 2; tile += DTHREADS / 32 - 1) {
        int ti = 0;
        while ((ti + 1) * (ti + 2) / 2 <= tile) ++ti;
        const int tj = tile - ti * (ti + 1) / 2;
        const int r0 = c2s + 32 * ti, cc0 = c2s + 32 * tj;
        float acc[4][8];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 8; ++v) acc[u][v] = 0.f;
        const int rl = lane & 7, cl = lane >> 3;
#pragma unroll 4
        for (int k = 0; k < SB; ++k) {
          const float* colk = Lp + pcol(q0 + k) - (q0 + k);
          float rv[4], cv[8];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int r = r0 + rl + 8 * u;
            rv[u] = r < wp ? colk[r] : 0.f;
          }
#pragma unroll
          for (int v = 0; v < 8; ++v) {
            const int cc = cc0 + cl + 4 * v;
            cv[v] = cc < wp ? colk[cc] : 0.f;
          }
#pragma unroll
          for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 8; ++v) acc[u][v] = fmaf(rv[u], cv[v], acc[u][v]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 8; ++v) {
            const int r = r0 + rl + 8 * u, cc = cc0 + cl + 4 * v;
            if (r < wp && cc <= r) Lp[pidx(r, cc)] -= acc[u][v];
          }
      }
    }
    __syncthreads();
  }
  for (int j = warp; j < w; j += DTHREADS / 32) {
    const float* col = Lp + pcol(j) - j;
    for (int i = j + lane; i < w; i += 32) a[(int64_t)(k0 + j) * ld + k0 + i] = col[i];
  }
}

// Rows [r0, r0 + 64) below the panel [k0, k0 + w): L_R L_WW^T = A_R by block
// forward substitution over 16-column sub-blocks.  Thread (row tid % 64,
// columns 4*(tid/64) .. +3 of the sub-block).
__global__ void __launch_bounds__(PTHREADS, 2) k_blk_panel(float* __restrict__ arena,
                                                           const BlkTask* __restrict__ tasks,
                                                           const float* __restrict__ xinv,
                                                           uint16_t* __restrict__ planes,
                                                           int64_t pstride, int pitch) {
  extern __shared__ __align__(16) float sm[];
  float* Ar = sm;                // Ar[k*ALD + r] = A(r0 + r, k0 + k), then L
  float* Lrow = Ar + PW * ALD;   // Lrow[k*16 + jj] = L(k0 + q0 + jj, k0 + k), k < q0
  float* Xs = Lrow + PW * SB;    // X of the sub-block, Xs[j*16 + i] = X(i, j)
  const BlkTask t = tasks[blockIdx.x];
  float* a = arena + t.off;
  const int64_t ld = t.ld;
  const int k0 = t.c, w = t.bw, r0 = t.r0, tid = threadIdx.x;
  const int nr = min(64, t.m - r0);
  const int wp = (w + SB - 1) / SB * SB;
  const float* xg = xinv + (int64_t)t.xi * XSZ;
  for (int e = tid; e < 64 * wp; e += PTHREADS) {
    const int r = e % 64, k = e / 64;
    if (r < nr && k < w) cp_async(&Ar[k * ALD + r], &a[(int64_t)(k0 + k) * ld + r0 + r]);
    else Ar[k * ALD + r] = 0.f;
  }
  const int r = tid & 63, j0 = 4 * (tid >> 6);
  for (int q0 = 0; q0 < wp; q0 += SB) {
    // block row q0/16 of L (left of the sub-block) and the sub-block inverse
    for (int e = tid; e < SB * q0; e += PTHREADS) {
      const int jj = e % SB, k = e / SB;
      if (q0 + jj < w) cp_async(&Lrow[e], &a[(int64_t)(k0 + k) * ld + k0 + q0 + jj]);
      else Lrow[e] = 0.f;
    }
    for (int e = tid; e < SB * SB; e += PTHREADS) cp_async(&Xs[e], &xg[(q0 / SB) * SB * SB + e]);
    cp_async_wait_all();
    __syncthreads();
    // correction by the earlier sub-blocks: one shared load of A and one
    // 16-byte load of the block row per four fused multiply-adds
    float v[4];
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) v[jj] = Ar[(q0 + j0 + jj) * ALD + r];
#pragma unroll 4
    for (int k = 0; k < q0; ++k) {
      const float ar = Ar[k * ALD + r];
      const float4 l4 = *reinterpret_cast<const float4*>(&Lrow[k * SB + j0]);
      v[0] = fmaf(-ar, l4.x, v[0]);
      v[1] = fmaf(-ar, l4.y, v[1]);
      v[2] = fmaf(-ar, l4.z, v[2]);
      v[3] = fmaf(-ar, l4.w, v[3]);
    }
    __syncthreads();
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) Ar[(q0 + j0 + jj) * ALD + r] = v[jj];
    __syncthreads();
    // L(r, q0 + j) = sum_k A'(r, q0 + k) X(j, k) (X lower triangular, zeros
    // stored above the diagonal)
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) v[jj] = 0.f;
#pragma unroll
    for (int k = 0; k < SB; ++k) {
      const float ak = Ar[(q0 + k) * ALD + r];
      const float4 x4 = *reinterpret_cast<const float4*>(&Xs[k * SB + j0]);
      v[0] = fmaf(ak, x4.x, v[0]);
      v[1] = fmaf(ak, x4.y, v[1]);
      v[2] = fmaf(ak, x4.z, v[2]);
      v[3] = fmaf(ak, x4.w, v[3]);
    }
    __syncthreads();
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
      Ar[(q0 + j0 + jj) * ALD + r] = v[jj];
      if (r < nr && q0 + j0 + jj < w) a[(int64_t)(k0 + q0 + j0 + jj) * ld + r0 + r] = v[jj];
    }
  }
  if (t.base >= 0) {
    // the rows just solved, transposed and split into three BF16 planes, for
    // the trailing tensor-core update (k contiguous: coalesced writes)
    __syncthreads();
    const int64_t row0 = (int64_t)t.base + (r0 - t.pend);
    for (int e = tid; e < nr * pitch; e += PTHREADS) {
      const int rr = e / pitch, k = e % pitch;
      uint16_t b0, b1, b2;
      bf16x3_split(k < w ? Ar[k * ALD + rr] : 0.f, b0, b1, b2);
      const int64_t o = (row0 + rr) * pitch + k;
      planes[o] = b0;
      planes[pstride + o] = b1;
      planes[2 * pstride + o] = b2;
    }
  }
}

constexpr size_t diag_smem() {
  return sizeof(float) * ((size_t)PW * (PW + 1) / 2 + SB * SB + SB * TLD);
}
constexpr size_t panel_smem() {
  return sizeof(float) * ((size_t)PW * ALD + PW * SB + SB * SB);
}

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
  k_blk_diag<<<ntask, DTHREADS, diag_smem(), s>>>(arena, t, xinv, status);
}

void launch_blk_panel(float* arena, const BlkTask* t, int ntask, const float* xinv,
                      uint16_t* planes, int64_t pstride, int pitch, cudaStream_t s) {
  if (ntask <= 0) return;
  k_blk_panel<<<ntask, PTHREADS, panel_smem(), s>>>(arena, t, xinv, planes, pstride, pitch);
}

}  // namespace sylver_gb300
