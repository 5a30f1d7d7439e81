// SIMT tile update C[rows, cols] -= sum_k A[row, k] B[col, k] on one 64x64
// (FP64) or 128x128 (FP32) tile, shared by the Cholesky schedule
// (kernels_factor.cu) and the LDL^T block steps (kernels_ldlt.cu).
//
// Arithmetic order (the CPU oracle of the LDL^T path repeats it): for every
// entry, acc = 0, acc = fma(A[row,k], B[col,k], acc) for k = k0, k0+1, ...,
// k1-1, then C = C - acc.  Only entries with col <= row are written.
#pragma once

#include "device.hpp"

namespace sylver_gb300 {

// 16x16 thread grid, RMxRN register micro-tiles split in two halves (rows
// ty*RM/2.. and TM/2+ty*RM/2..), double-buffered KT-deep shared tiles.
// Must be called by all 256 threads of the CTA (it synchronises).
template <typename T, int TM, int TN, int KT>
__device__ __forceinline__ void tile_update_body(T* __restrict__ C, int ldc,
                                                 const T* __restrict__ A, int lda,
                                                 const T* __restrict__ B, int ldb, int row0,
                                                 int col0, int rowEnd, int colEnd, int k0,
                                                 int k1, T (&As)[2][KT][TM],
                                                 T (&Bs)[2][KT][TN]) {
  constexpr int RM = TM / 16, RN = TN / 16;
  constexpr int HM = RM / 2, HN = RN / 2;
  constexpr int LA = (KT * TM) / 256, LB = (KT * TN) / 256;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  T ra[LA], rb[LB];
  auto gload = [&](int kc) {
#pragma unroll
    for (int q = 0; q < LA; ++q) {
      int e = tid + q * 256;
      int i = e % TM, kk = e / TM;
      int row = row0 + i, k = kc + kk;
      ra[q] = (row < rowEnd && k < k1) ? A[(int64_t)k * lda + row] : T(0);
    }
#pragma unroll
    for (int q = 0; q < LB; ++q) {
      int e = tid + q * 256;
      int i = e % TN, kk = e / TN;
      int col = col0 + i, k = kc + kk;
      rb[q] = (col < colEnd && k < k1) ? B[(int64_t)k * ldb + col] : T(0);
    }
  };
  auto sstore = [&](int buf) {
#pragma unroll
    for (int q = 0; q < LA; ++q) {
      int e = tid + q * 256;
      As[buf][e / TM][e % TM] = ra[q];
    }
#pragma unroll
    for (int q = 0; q < LB; ++q) {
      int e = tid + q * 256;
      Bs[buf][e / TN][e % TN] = rb[q];
    }
  };
  T acc[RM][RN];
#pragma unroll
  for (int i = 0; i < RM; ++i)
#pragma unroll
    for (int j = 0; j < RN; ++j) acc[i][j] = T(0);

  int kc = k0;
  gload(kc);
  sstore(0);
  __syncthreads();
  int buf = 0;
  for (; kc < k1; kc += KT) {
    const bool more = kc + KT < k1;
    if (more) gload(kc + KT);
#pragma unroll
    for (int kk = 0; kk < KT; ++kk) {
      T av[RM], bv[RN];
#pragma unroll
      for (int i = 0; i < HM; ++i) {
        av[i] = As[buf][kk][ty * HM + i];
        av[HM + i] = As[buf][kk][TM / 2 + ty * HM + i];
      }
#pragma unroll
      for (int j = 0; j < HN; ++j) {
        bv[j] = Bs[buf][kk][tx * HN + j];
        bv[HN + j] = Bs[buf][kk][TN / 2 + tx * HN + j];
      }
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < RN; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
    }
    if (more) {
      sstore(buf ^ 1);
      __syncthreads();
      buf ^= 1;
    }
  }
#pragma unroll
  for (int i = 0; i < RM; ++i) {
    int row = row0 + ((i < HM) ? ty * HM + i : TM / 2 + ty * HM + (i - HM));
    if (row >= rowEnd) continue;
#pragma unroll
    for (int j = 0; j < RN; ++j) {
      int col = col0 + ((j < HN) ? tx * HN + j : TN / 2 + tx * HN + (j - HN));
      if (col >= colEnd || col > row) continue;
      C[(int64_t)col * ldc + row] -= acc[i][j];
    }
  }
}

}  // namespace sylver_gb300
