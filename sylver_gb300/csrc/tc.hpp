// Tensor-core (tcgen05) Schur-complement update: descriptors and launchers.
#pragma once

#include <cuda.h>

#include "device.hpp"

namespace sylver_gb300 {

// One 128 x 128 tile of C -= P_a P_b^T for a contribution block:
// C(i, j) = arena[c_off + j*ldc + i] for i in [row0, row0+128) < rowEnd,
// j in [col0, col0+128) < colEnd, only i >= j written.  A rows start at
// stacked panel row a_row, B rows at b_row; nk chunks of 32 along k.
struct TcTask {
  int64_t c_off;
  int ldc, row0, col0, rowEnd, colEnd, a_row, b_row, nk;
};

// Transposed hi/lo copy of front rows [n, m) x columns [c0, c0 + K) into
// stacked panel rows [base, base + m - n).
struct TcSplit {
  int64_t off;
  int ld, m, n, K, base, c0;
};

size_t tc_smem_bytes();
void prepare_tc_kernels();
void make_panel_map(CUtensorMap* map, const float* base, int64_t rows, int pitch);
void launch_split_t(const float* arena, const TcSplit* sp, int nsplit, int64_t max_rows,
                    float* hi, float* lo, int pitch, cudaStream_t s);
void launch_update_tc(const CUtensorMap& hi, const CUtensorMap& lo, float* arena,
                      const TcTask* t, int ntask, unsigned* err, cudaStream_t s);

}  // namespace sylver_gb300
