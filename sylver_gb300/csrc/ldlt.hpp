// Threshold-pivoted LDL^T on the GPU: planning, factorization driver,
// solves with D and delayed pivots.
#pragma once

#include "numeric.hpp"

namespace sylver_gb300 {

void plan_ldlt(FKeep& fk);
int factorize_ldlt(FKeep& fk, const double* val_dev, cudaStream_t s);
void ldlt_solve_pivot_order(FKeep& fk, int job, float* xp, int nrhs, cudaStream_t s);
void ldlt_solve_pivot_order(FKeep& fk, int job, double* xp, int nrhs, cudaStream_t s);
int ldlt_export_diag(const FKeep& fk, double* d, int* piv_order);
int ldlt_export_fronts(const FKeep& fk, int* m, int* n, int* nelim);
// Device tables of the forward solve of an LDL^T factorization (level-ordered
// front descriptors, slab offsets, row-variable lists) and the largest
// per-level slab row count; false before a factorization.
bool ldlt_solve_tables(const FKeep& fk, const FrontDesc** fr, const int64_t** scr,
                       const int** rows, int64_t* scratch_rows);

}  // namespace sylver_gb300
