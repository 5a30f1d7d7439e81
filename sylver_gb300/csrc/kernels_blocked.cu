// Blocked Cholesky of the fully-summed columns of large FP32 fronts.
//
// The fully-summed columns are eliminated in outer panels of up to 256
// columns.  Inside a panel, steps of 64 columns run two kernels:
//   k_blk_diag  (one CTA per front): Cholesky of the 64 x 64 diagonal block
//               L11, its explicit inverse X = L11^-1 (kept for the next
//               kernel), and the rows of L below the block that lie inside
//               the panel, L_J = A_J X^T;
//   k_blk_panel (one CTA per 64 rows below the block): L_R = A_R X^T for the
//               rows below the panel (rows inside it read L_J back), then the
//               in-panel update A(R, J) -= L_R L_J^T.
// The trailing update of the remaining fully-summed columns after each
// outer panel (K = panel width) and the contribution-block update (K = n)
// run on the tensor cores (k_update_tc), so the SIMT kernels here only touch
// one panel at a time.
//
// Reference behaviour replaced: factorize_diag_block, solve_block,
// update_block and update_diag_block (src/kernels/factor.hxx:56-260) as
// driven by factor_front_posdef (src/factor.hxx:19-148).  The triangular
// solve of the panel rows is a product with the explicit inverse of the
// diagonal block instead of a substitution; the FP64 refinement absorbs the
// difference.
#include "device.hpp"

namespace sylver_gb300 {

namespace {

constexpr int BB = BLK_B;   // inner block width
constexpr int BLD = BB + 1;  // padded shared-memory leading dimension
constexpr int BJ = BLK_W - BB;  // most panel rows below a diagonal block
constexpr int BJP = BJ + 1;

// L(rows, 0:64) = A(rows, 0:64) X^T for a 64-row tile staged in As
// (As[k*BLD + r]); X staged as Xt[k*BLD + j] = X(j, k).  Thread (rr, cc)
// owns rows rr + 16u and columns cc + 16v, u, v < 4.
__device__ __forceinline__ void tile_times_xt(const float* __restrict__ As,
                                              const float* __restrict__ Xt, int rr, int cc,
                                              float (&o)[4][4]) {
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) o[u][v] = 0.f;
#pragma unroll 8
  for (int k = 0; k < BB; ++k) {
    float av[4], xv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) av[u] = As[k * BLD + rr + 16 * u];
#pragma unroll
    for (int v = 0; v < 4; ++v) xv[v] = Xt[k * BLD + cc + 16 * v];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) o[u][v] = fmaf(av[u], xv[v], o[u][v]);
  }
}

__global__ void __launch_bounds__(256) k_blk_diag(float* __restrict__ arena,
                                                  const BlkTask* __restrict__ tasks,
                                                  float* __restrict__ xinv,
                                                  unsigned* __restrict__ status) {
  extern __shared__ __align__(16) float sm[];
  float* S = sm;             // S[j*BLD + i] = A(c+i, c+j), then L11
  float* Xt = S + BB * BLD;  // Xt[a*BLD + b] = X(b, a)  (X = L11^-1)
  float* As = Xt + BB * BLD; // staging of 64 panel rows
  __shared__ float dsq[BB];
  const BlkTask t = tasks[blockIdx.x];
  float* a = arena + t.off;
  const int64_t ld = t.ld;
  const int c = t.c, bw = t.bw, tid = threadIdx.x;

  // diagonal block, padded to 64 x 64 with the identity
  for (int e = tid; e < BB * BB; e += 256) {
    const int i = e % BB, j = e / BB;
    float v;
    if (i < bw && j < bw) v = (i >= j) ? a[(int64_t)(c + j) * ld + c + i] : 0.f;
    else v = (i == j) ? 1.f : 0.f;
    S[j * BLD + i] = v;
  }
  // outer-product elimination without square roots: after step k,
  // S(i, j) = A(i, j) - sum_{q<=k} S(i,q) S(j,q) / d_q for i >= j > k
  {
    const int i = tid & (BB - 1), g = tid >> 6;
    for (int k = 0; k < BB - 1; ++k) {
      __syncthreads();
      float d = S[k * BLD + k];
      if (!(d > 0.f)) d = 1.f;
      const float aik = S[k * BLD + i] / d;
      if (i > k)
        for (int j = k + 1 + g; j <= i; j += 4) S[j * BLD + i] -= aik * S[k * BLD + j];
    }
  }
  __syncthreads();
  if (tid < BB) {
    float d = S[tid * BLD + tid];
    if (!(d > 0.f)) {
      if (tid < bw) atomicOr(status, ST_NOT_POSDEF);
      d = 1.f;
    }
    dsq[tid] = sqrtf(d);
  }
  __syncthreads();
  for (int e = tid; e < BB * BB; e += 256) {
    const int i = e % BB, j = e / BB;
    if (i > j) S[j * BLD + i] /= dsq[j];
    else if (i == j) S[j * BLD + i] = dsq[j];
  }
  __syncthreads();
  for (int e = tid; e < BB * BB; e += 256) {
    const int i = e % BB, j = e / BB;
    if (i < bw && j < bw && i >= j) a[(int64_t)(c + j) * ld + c + i] = S[j * BLD + i];
  }
  // X = L11^-1, column j by four lanes; lane q sums the terms k = q (mod 4)
  // and keeps the entries X(i, j) with i = q (mod 4), which only it reads
  {
    const int j = tid >> 2, q = tid & 3;
    for (int i = 0; i < BB; ++i) {
      float part = 0.f;
      if (i > j)
        for (int k = j + ((q - j) & 3); k < i; k += 4) part += S[k * BLD + i] * Xt[j * BLD + k];
      part += __shfl_xor_sync(0xffffffffu, part, 1);
      part += __shfl_xor_sync(0xffffffffu, part, 2);
      if ((i & 3) == q)
        Xt[j * BLD + i] = (i < j) ? 0.f : ((i == j ? 1.f : 0.f) - part) / S[i * BLD + i];
    }
  }
  __syncthreads();
  float* xo = xinv + (int64_t)t.xi * BB * BB;  // X(i, j) at [j*64 + i]
  for (int e = tid; e < BB * BB; e += 256) {
    const int i = e % BB, j = e / BB;
    xo[e] = Xt[j * BLD + i];
  }
  // rows of L inside the panel below the block: L_J = A_J X^T
  const int r0 = c + bw, nJ = t.pend - r0;
  const int rr = tid & 15, cc = tid >> 4;
  for (int q0 = 0; q0 < nJ; q0 += BB) {
    const int nr = min(BB, nJ - q0);
    for (int e = tid; e < BB * BB; e += 256) {
      const int r = e % BB, k = e / BB;
      As[k * BLD + r] = (r < nr && k < bw) ? a[(int64_t)(c + k) * ld + r0 + q0 + r] : 0.f;
    }
    __syncthreads();
    float o[4][4];
    tile_times_xt(As, Xt, rr, cc, o);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int r = rr + 16 * u, j = cc + 16 * v;
        if (r < nr && j < bw) a[(int64_t)(c + j) * ld + r0 + q0 + r] = o[u][v];
      }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_blk_panel(float* __restrict__ arena,
                                                   const BlkTask* __restrict__ tasks,
                                                   const float* __restrict__ xinv) {
  extern __shared__ __align__(16) float sm[];
  float* Xt = sm;              // Xt[k*BLD + j] = X(j, k)
  float* Lr = Xt + BB * BLD;   // Lr[k*BLD + r]: A, then L, of this CTA's rows
  float* LJ = Lr + BB * BLD;   // LJ[k*BJP + j] = L(cb + j, c + k)
  const BlkTask t = tasks[blockIdx.x];
  float* a = arena + t.off;
  const int64_t ld = t.ld;
  const int c = t.c, bw = t.bw, cb = c + bw, pend = t.pend, r0 = t.r0, tid = threadIdx.x;
  const int nr = min(BB, t.m - r0);
  const int nJ = pend - cb;
  const bool solve = r0 + nr > pend;  // some rows lie below the panel
  if (solve) {
    const float* xi = xinv + (int64_t)t.xi * BB * BB;
    for (int e = tid; e < BB * BB; e += 256) {
      const int j = e % BB, k = e / BB;  // X(j, k) at [k*64 + j]
      Xt[k * BLD + j] = xi[e];
    }
  }
  for (int e = tid; e < BB * BB; e += 256) {
    const int r = e % BB, k = e / BB;
    Lr[k * BLD + r] = (r < nr && k < bw) ? a[(int64_t)(c + k) * ld + r0 + r] : 0.f;
  }
  for (int e = tid; e < BB * nJ; e += 256) {
    const int j = e % nJ, k = e / nJ;
    LJ[k * BJP + j] = (k < bw) ? a[(int64_t)(c + k) * ld + cb + j] : 0.f;
  }
  __syncthreads();
  const int rr = tid & 15, cc = tid >> 4;
  if (solve) {
    float o[4][4];
    tile_times_xt(Lr, Xt, rr, cc, o);
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int r = rr + 16 * u, j = cc + 16 * v;
        if (r0 + r >= pend && r < nr) {
          Lr[j * BLD + r] = o[u][v];
          if (j < bw) a[(int64_t)(c + j) * ld + r0 + r] = o[u][v];
        }
      }
    __syncthreads();
  }
  if (nJ <= 0) return;
  // A(r0 + r, cb + j) -= sum_k L(r0 + r, c + k) L(cb + j, c + k), lower part
  constexpr int NV = BJ / 16;
  float acc[4][NV];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[u][v] = 0.f;
  const int nv = (nJ + 15) / 16;
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
      if (r < nr && j < nJ && r0 + r >= cb + j) a[(int64_t)(cb + j) * ld + r0 + r] -= acc[u][v];
    }
}

constexpr size_t diag_smem() { return sizeof(float) * 3 * BB * BLD; }
constexpr size_t panel_smem() { return sizeof(float) * (2 * BB * BLD + BB * BJP); }

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
