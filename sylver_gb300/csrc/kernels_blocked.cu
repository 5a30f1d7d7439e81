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
constexpr int DTHREADS = 512;
constexpr int PROWS = 64;         // rows of one panel-kernel CTA
constexpr int PTHREADS = 2 * PROWS;
constexpr int ALD = PROWS + 1;

// start of column j of a packed lower triangle with PW rows
__device__ __forceinline__ int pcol(int j) { return j * PW - (j * (j - 1)) / 2; }
// (i, j), i >= j, of the packed lower triangle
__device__ __forceinline__ int pidx(int i, int j) { return pcol(j) + i - j; }

// One warp: Cholesky of the 16 x 16 diagonal sub-block at (q, q) of the
// packed triangle Lp, in registers (lane i < 16 holds row i; lanes 16..31
// repeat lanes 0..15).  With bk != nullptr the sub-block is first updated
// by the 16 columns left of it: A(q+i, q+k) -= sum_m L(q+i, m) L(q+k, m),
// bk[m*16 + i] = L(q + i, q - 16 + m).  Writes L back to Lp and to tt
// (tt[k*16 + i] = L(i, k), 16-byte aligned) and X = L^-1 to xs and xg (both
// xs[k*16 + i] = X(i, k)).  A non-positive pivot is replaced by one and
// reported when its column is below bwreal.
__device__ __noinline__ void warp_chol16(float* __restrict__ Lp, int q, int bwreal,
                                         const float* __restrict__ bk, float* __restrict__ tt,
                                         float* __restrict__ xs, float* __restrict__ xg,
                                         unsigned* __restrict__ status) {
  const int lane = threadIdx.x & 31;
  const int li = lane & (SB - 1);
  float a[SB], rinv[SB];
#pragma unroll
  for (int k = 0; k < SB; ++k) a[k] = (k <= li) ? Lp[pidx(q + li, q + k)] : 0.f;
  if (bk != nullptr) {
#pragma unroll 4
    for (int m = 0; m < SB; ++m) {
      const float own = bk[m * SB + li];
#pragma unroll
      for (int k4 = 0; k4 < SB; k4 += 4) {
        const float4 b4 = *reinterpret_cast<const float4*>(&bk[m * SB + k4]);
        a[k4] = fmaf(-own, b4.x, a[k4]);
        a[k4 + 1] = fmaf(-own, b4.y, a[k4 + 1]);
        a[k4 + 2] = fmaf(-own, b4.z, a[k4 + 2]);
        a[k4 + 3] = fmaf(-own, b4.w, a[k4 + 3]);
      }
    }
  }
  bool bad = false;
  // The pivot chain is the critical path of the panel: 1/sqrt(d) comes from
  // the hardware estimate refined by one Newton step (about 1 ulp), and
  // both the column scaling and the inverse multiply by it -- IEEE sqrt and
  // division cost three times as long per 16 columns.  Lane k + 1 forms the
  // next pivot from its own l(k+1, k), so only one shuffle per column sits
  // on the chain; the column itself reaches the other lanes through tt
  // (16-byte loads).
  float dn = __shfl_sync(0xffffffffu, a[0], 0);
#pragma unroll
  for (int k = 0; k < SB; ++k) {
    float d = dn;
    if (!(d > 0.f)) {
      if (q + k < bwreal) bad = true;
      d = 1.f;
    }
    float r = rsqrtf(d);
    r = r * fmaf(-0.5f * d * r, r, 1.5f);
    rinv[k] = r;
    const float lik = (li == k) ? d * r : a[k] * r;
    a[k] = lik;
    if (k + 1 < SB) dn = __shfl_sync(0xffffffffu, fmaf(-lik, lik, a[k + 1]), k + 1);
    if (lane < SB) tt[k * SB + li] = lik;
    __syncwarp();
#pragma unroll
    for (int j4 = ((k + 1) & ~3); j4 < SB; j4 += 4) {
      const float4 c4 = *reinterpret_cast<const float4*>(&tt[k * SB + j4]);
      const float cj[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int j = j4 + u;
        if (j > k && li >= j) a[j] = fmaf(-lik, cj[u], a[j]);
      }
    }
  }
  // L to the packed triangle (tt holds it densely for the inverse)
  if (lane < SB) {
#pragma unroll
    for (int k = 0; k < SB; ++k)
      if (k <= li) Lp[pidx(q + li, q + k)] = a[k];
  }
  __syncwarp();
  if (lane == 0 && bad) atomicOr(status, ST_NOT_POSDEF);
  // column li of X: X(i, li) = (delta - sum_{k<i} L(i,k) X(k, li)) / L(i, i)
  float x[SB];
#pragma unroll
  for (int i = 0; i < SB; ++i) {
    float v = (i == li) ? 1.f : 0.f;
#pragma unroll
    for (int k = 0; k < i; ++k) v = fmaf(-tt[k * SB + i], x[k], v);
    x[i] = v * rinv[i];
  }
  if (lane < SB) {
#pragma unroll
    for (int i = 0; i < SB; i += 4) {
      const float4 x4 = make_float4(x[i], x[i + 1], x[i + 2], x[i + 3]);
      *reinterpret_cast<float4*>(&xs[li * SB + i]) = x4;
      *reinterpret_cast<float4*>(&xg[li * SB + i]) = x4;
    }
  }
}

__global__ void __launch_bounds__(DTHREADS) k_blk_diag(float* __restrict__ arena,
                                                       const BlkTask* __restrict__ tasks,
                                                       float* __restrict__ xinv,
                                                       unsigned* __restrict__ status) {
  extern __shared__ __align__(16) float sm[];
  float* Xs = sm;                      // inverse of the current sub-block, Xs[k*16 + j] = X(j, k)
  float* Bk = Xs + SB * SB;            // Bk[m*16 + i] = L(c1 + i, q0 + m), the next sub-block's rows
  float* Tt = Bk + SB * SB;            // dense copy of the factorised sub-block (warp 0)
  float* Lp = Tt + SB * SB;            // packed lower triangle, PW rows
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
  if (warp == 0) warp_chol16(Lp, 0, w, nullptr, Tt, Xs, xg, status);
  __syncthreads();
  // Per 16-column sub-block q0: (b) all threads solve the rows below it with
  // its inverse; then warp 0 updates the next diagonal sub-block by it and
  // factorises that (the serial pivot chain) while the warps of the other
  // three schedulers update the next sub-block column below its diagonal
  // block (c1) and the rest of the trailing triangle (c2); the warps that
  // share warp 0's scheduler (warp % 4 == 0) wait, so the pivot chain
  // issues without competition.
  for (int q0 = 0; q0 < wp; q0 += SB) {
    const int c1 = q0 + SB;
    if (c1 >= wp) break;
    // (b) L(r, q0 + j) = sum_k A(r, q0 + k) X(j, k) for rows r >= c1; four
    // lanes per row, lane group g owning columns 4g .. 4g + 3
    const int nb = (wp - c1) * 4;
    for (int e0 = 0; e0 < nb; e0 += DTHREADS) {
      const int e = e0 + tid;
      const int r = c1 + (e >> 2), g = e & 3;
      float o[4] = {0.f, 0.f, 0.f, 0.f};
      if (e < nb) {
#pragma unroll
        for (int k = 0; k < SB; ++k) {
          const float vk = Lp[pidx(r, q0 + k)];
          const float4 x4 = *reinterpret_cast<const float4*>(&Xs[k * SB + 4 * g]);
          o[0] = fmaf(vk, x4.x, o[0]);
          o[1] = fmaf(vk, x4.y, o[1]);
          o[2] = fmaf(vk, x4.z, o[2]);
          o[3] = fmaf(vk, x4.w, o[3]);
        }
      }
      __syncwarp();
      if (e < nb) {
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          Lp[pidx(r, q0 + 4 * g + jj)] = o[jj];
          if (r < c1 + SB) Bk[(4 * g + jj) * SB + (r - c1)] = o[jj];
        }
      }
    }
    __syncthreads();
    if (warp == 0) {
      warp_chol16(Lp, c1, w, Bk, Tt, Xs, xg + (c1 / SB) * SB * SB, status);
    } else if (warp & 3) {
      // the 12 update warps, numbered 0..11
      const int uw = warp - 1 - (warp >> 2), utid = uw * 32 + lane;
      constexpr int UTHREADS = DTHREADS / 32 * 3 / 4 * 32;
      // (c1) rows [c1 + 16, wp) x columns [c1, c1 + 16): lane group g of a
      // row updates columns c1 + 4g .. + 3
      const int c2s = c1 + SB;
      const int nc = (wp - c2s) * 4;
      for (int e = utid; e < nc; e += UTHREADS) {
        const int r = c2s + (e >> 2), g = e & 3;
        float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int k = 0; k < SB; ++k) {
          const float lk = Lp[pidx(r, q0 + k)];
          const float4 b4 = *reinterpret_cast<const float4*>(&Bk[k * SB + 4 * g]);
          o[0] = fmaf(lk, b4.x, o[0]);
          o[1] = fmaf(lk, b4.y, o[1]);
          o[2] = fmaf(lk, b4.z, o[2]);
          o[3] = fmaf(lk, b4.w, o[3]);
        }
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) Lp[pidx(r, c1 + 4 * g + jj)] -= o[jj];
      }
      // (c2) trailing triangle [c2s, wp)^2 -= L(:, q0:+16) L(:, q0:+16)^T in
      // 16 x 16 tiles, one update warp per tile; lane owns rows
      // r0 + (lane&7) + 8u (u < 2) and columns cc0 + (lane>>3) + 4v (v < 4)
      const int nt = (wp - c2s + 15) / 16;
      for (int tile = uw; tile < nt * (nt + 1) / 2; tile += UTHREADS / 32) {
        int ti = 0;
        while ((ti + 1) * (ti + 2) / 2 <= tile) ++ti;
        const int tj = tile - ti * (ti + 1) / 2;
        const int r0 = c2s + 16 * ti, cc0 = c2s + 16 * tj;
        float acc[2][4];
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
        const int rl = lane & 7, cl = lane >> 3;
#pragma unroll 4
        for (int k = 0; k < SB; ++k) {
          const float* colk = Lp + pcol(q0 + k) - (q0 + k);
          float rv[2], cv[4];
#pragma unroll
          for (int u = 0; u < 2; ++u) rv[u] = colk[r0 + rl + 8 * u];
#pragma unroll
          for (int v = 0; v < 4; ++v) cv[v] = colk[cc0 + cl + 4 * v];
#pragma unroll
          for (int u = 0; u < 2; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(rv[u], cv[v], acc[u][v]);
        }
#pragma unroll
        for (int u = 0; u < 2; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const int r = r0 + rl + 8 * u, cc = cc0 + cl + 4 * v;
            if (cc <= r) Lp[pidx(r, cc)] -= acc[u][v];
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

// K columns k .. k + 3 (k a multiple of 4) of local row rr of the panel
// kernel's tile, split into the three BF16 planes and stored as 8-byte
// vectors at element offset o (a multiple of 4) of each plane; columns >= w
// are zero.
__device__ __forceinline__ void put_split4(const float* __restrict__ Ar, int rr, int k, int w,
                                           uint16_t* __restrict__ pl, int64_t ps, int64_t o) {
  uint32_t lo[3], hi[3];
  uint16_t b[3][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
    bf16x3_split(k + u < w ? Ar[(k + u) * ALD + rr] : 0.f, b[0][u], b[1][u], b[2][u]);
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    lo[q] = (uint32_t)b[q][0] | ((uint32_t)b[q][1] << 16);
    hi[q] = (uint32_t)b[q][2] | ((uint32_t)b[q][3] << 16);
    *reinterpret_cast<uint2*>(pl + q * ps + o) = make_uint2(lo[q], hi[q]);
  }
}

// Floats of the staged block rows of L_WW: block row q >= 1 (columns k < 16q
// of rows 16q .. 16q + 15) starts at lw_off(q), 16 values per k.
__host__ __device__ constexpr int lw_off(int q) { return 128 * q * (q - 1); }

// Rows [r0, r0 + 64) below the panel [k0, k0 + w): L_R L_WW^T = A_R by block
// forward substitution over 16-column sub-blocks.  Each row is solved by two
// lanes of one warp (lane & 15 picks the row, lane >> 4 the half of the
// sub-block's columns); rows never depend on one another, so after the block
// rows of L_WW and the sub-block inverses are staged once, the sub-steps need
// no block-wide barrier.
__global__ void __launch_bounds__(PTHREADS) k_blk_panel(float* __restrict__ arena,
                                                        const BlkTask* __restrict__ tasks,
                                                        const float* __restrict__ xinv,
                                                        uint16_t* __restrict__ planes,
                                                        int64_t pstride, int pw, int pitch,
                                                        uint16_t* __restrict__ cbplanes,
                                                        int64_t cbpstride) {
  extern __shared__ __align__(16) float sm[];
  float* Ar = sm;                          // Ar[k*ALD + r] = A(r0 + r, k0 + k), then L
  float* Lw = Ar + pw * ALD;               // block rows of L_WW (lw_off layout)
  float* Xs = Lw + lw_off(pw / SB);        // Xs[q*256 + k*16 + j] = X_q(j, k)
  const BlkTask t = tasks[blockIdx.x];
  float* a = arena + t.off;
  const int64_t ld = t.ld;
  const int k0 = t.c, w = t.bw, r0 = t.r0, tid = threadIdx.x;
  const int nr = min(PROWS, t.m - r0);
  const int nsb = (w + SB - 1) / SB, wp = nsb * SB;
  const float* xg = xinv + (int64_t)t.xi * XSZ;
  for (int e = tid; e < PROWS * wp; e += PTHREADS) {
    const int r = e % PROWS, k = e / PROWS;
    if (r < nr && k < w) cp_async(&Ar[k * ALD + r], &a[(int64_t)(k0 + k) * ld + r0 + r]);
    else Ar[k * ALD + r] = 0.f;
  }
  for (int q = 1; q < nsb; ++q) {
    float* dst = Lw + lw_off(q);
    const int q0 = q * SB;
    for (int e = tid; e < SB * q0; e += PTHREADS) {
      const int jj = e % SB, k = e / SB;
      if (q0 + jj < w) cp_async(&dst[e], &a[(int64_t)(k0 + k) * ld + k0 + q0 + jj]);
      else dst[e] = 0.f;
    }
  }
  for (int e = tid; e < nsb * SB * SB; e += PTHREADS) cp_async(&Xs[e], &xg[e]);
  cp_async_wait_all();
  __syncthreads();
  const int lane = tid & 31, h = lane >> 4;
  const int r = (tid >> 5) * 16 + (lane & 15);
  for (int q = 0; q < nsb; ++q) {
    const int q0 = q * SB, c0 = q0 + 8 * h;  // this lane's eight columns
    // correction by the earlier sub-blocks: one shared load of the row and
    // two 16-byte loads of the block row per eight fused multiply-adds
    float v[8];
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) v[jj] = Ar[(c0 + jj) * ALD + r];
    const float* lq = Lw + lw_off(q) + 8 * h;
#pragma unroll 4
    for (int k = 0; k < q0; ++k) {
      const float ar = Ar[k * ALD + r];
      const float4 la = *reinterpret_cast<const float4*>(lq + k * SB);
      const float4 lb = *reinterpret_cast<const float4*>(lq + k * SB + 4);
      v[0] = fmaf(-ar, la.x, v[0]);
      v[1] = fmaf(-ar, la.y, v[1]);
      v[2] = fmaf(-ar, la.z, v[2]);
      v[3] = fmaf(-ar, la.w, v[3]);
      v[4] = fmaf(-ar, lb.x, v[4]);
      v[5] = fmaf(-ar, lb.y, v[5]);
      v[6] = fmaf(-ar, lb.z, v[6]);
      v[7] = fmaf(-ar, lb.w, v[7]);
    }
    // the whole corrected row of the sub-block from the partner lane
    float lo[8], hi[8];
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) {
      const float o = __shfl_xor_sync(0xffffffffu, v[jj], 16);
      lo[jj] = h ? o : v[jj];
      hi[jj] = h ? v[jj] : o;
    }
    // L(r, c0 + jj) = sum_k A'(r, q0 + k) X_q(8h + jj, k); X_q is lower
    // triangular with zeros stored above the diagonal
    const float* xq = Xs + q * SB * SB + 8 * h;
    float o[8];
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) o[jj] = 0.f;
#pragma unroll
    for (int k = 0; k < SB; ++k) {
      const float vk = k < 8 ? lo[k] : hi[k - 8];
      const float4 xa = *reinterpret_cast<const float4*>(xq + k * SB);
      const float4 xb = *reinterpret_cast<const float4*>(xq + k * SB + 4);
      o[0] = fmaf(vk, xa.x, o[0]);
      o[1] = fmaf(vk, xa.y, o[1]);
      o[2] = fmaf(vk, xa.z, o[2]);
      o[3] = fmaf(vk, xa.w, o[3]);
      o[4] = fmaf(vk, xb.x, o[4]);
      o[5] = fmaf(vk, xb.y, o[5]);
      o[6] = fmaf(vk, xb.z, o[6]);
      o[7] = fmaf(vk, xb.w, o[7]);
    }
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) {
      Ar[(c0 + jj) * ALD + r] = o[jj];
      if (r < nr && c0 + jj < w) a[(int64_t)(k0 + c0 + jj) * ld + r0 + r] = o[jj];
    }
    __syncwarp();
  }
  if (t.base >= 0 || t.cbbase >= 0) __syncthreads();
  if (t.cbbase >= 0) {
    // contribution rows: their K columns of the contribution-block update's
    // operand planes (zeros past the panel up to n rounded to 64)
    const int rf = max(0, t.n - r0);
    const int kend = min(pw, (t.n + TC_KCHUNK - 1) / TC_KCHUNK * TC_KCHUNK - k0);
    const int k4 = kend / 4;
    if (kend > 0)
      for (int e = tid; e < (nr - rf) * k4; e += PTHREADS) {
        const int rr = rf + e / k4, k = 4 * (e % k4);
        put_split4(Ar, rr, k, w, cbplanes, cbpstride,
                   ((int64_t)t.cbbase + (r0 + rr - t.n)) * t.cbpitch + k0 + k);
      }
  }
  if (t.base >= 0) {
    // the rows just solved, transposed and split into three BF16 planes, for
    // the trailing tensor-core update (k contiguous: coalesced writes)
    const int64_t row0 = (int64_t)t.base + (r0 - t.pend);
    const int koff = k0 % pitch;
    const int k4 = pw / 4;
    for (int e = tid; e < nr * k4; e += PTHREADS) {
      const int rr = e / k4, k = 4 * (e % k4);
      put_split4(Ar, rr, k, w, planes, pstride, (row0 + rr) * pitch + koff + k);
    }
  }
}

constexpr size_t diag_smem() {
  return sizeof(float) * ((size_t)PW * (PW + 1) / 2 + 3 * SB * SB);
}
constexpr size_t panel_smem(int pitch) {
  return sizeof(float) * ((size_t)pitch * ALD + lw_off(pitch / SB) + (size_t)pitch * SB);
}

}  // namespace

void prepare_blocked_kernels() {
  SG_CUDA(cudaFuncSetAttribute(k_blk_diag, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)diag_smem()));
  SG_CUDA(cudaFuncSetAttribute(k_blk_panel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)panel_smem(PW)));
}

void launch_blk_diag(float* arena, const BlkTask* t, int ntask, float* xinv, unsigned* status,
                     cudaStream_t s) {
  if (ntask <= 0) return;
  k_blk_diag<<<ntask, DTHREADS, diag_smem(), s>>>(arena, t, xinv, status);
}

void launch_blk_panel(float* arena, const BlkTask* t, int ntask, const float* xinv,
                      uint16_t* planes, int64_t pstride, int pw, int pitch, uint16_t* cbplanes,
                      int64_t cbpstride, cudaStream_t s) {
  if (ntask <= 0) return;
  k_blk_panel<<<ntask, PTHREADS, panel_smem(pw), s>>>(arena, t, xinv, planes, pstride, pw,
                                                       pitch, cbplanes, cbpstride);
}

}  // namespace sylver_gb300
