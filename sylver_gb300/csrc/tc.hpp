// Tensor-core (tcgen05) Schur-complement update: descriptors and launchers.
#pragma once

#include <cuda.h>

#include "device.hpp"

namespace sylver_gb300 {

// One 128 x 128 tile of C -= P_a P_b^T for a contribution block:
// C(i, j) = arena[c_off + j*ldc + i] for i in [row0, row0+128) < rowEnd,
// j in [col0, col0+128) < colEnd, only i >= j written.  A rows start at
// stacked panel row a_row, B rows at b_row; nk chunks of TC_KCHUNK along k
// starting at chunk kc0.
struct TcTask {
  int64_t c_off;
  int ldc, row0, col0, rowEnd, colEnd, a_row, b_row, nk;
  int kc0;
};

// Transposed 3xBF16 copy of front rows [n, m) x columns [c0, c0 + K) into
// stacked panel rows [base, base + m - n) of the three planes.
struct TcSplit {
  int64_t off;
  int ld, m, n, K, base, c0;
};

size_t tc_smem_bytes();
void prepare_tc_kernels();
// Tensor map of one BF16 plane: rows x pitch elements (pitch a multiple of
// TC_KCHUNK), boxes of TC_KCHUNK x 128.
void make_panel_map(CUtensorMap* map, const uint16_t* base, int64_t rows, int pitch);
// planes: three BF16 planes, plane q at planes + q * pstride.
void launch_split_t(const float* arena, const TcSplit* sp, int nsplit, int64_t max_rows,
                    uint16_t* planes, int64_t pstride, int pitch, cudaStream_t s);
// maps: the tensor maps of the three planes.
void launch_update_tc(const CUtensorMap* maps, float* arena, const TcTask* t, int ntask,
                      unsigned* err, cudaStream_t s);

}  // namespace sylver_gb300
