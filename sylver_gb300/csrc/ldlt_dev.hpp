// Device-side descriptors and launchers of the threshold-pivoted LDL^T path.
#pragma once

#include "device.hpp"

namespace sylver_gb300 {

constexpr int LDLT_BW = 32;   // diagonal block width of the a-posteriori pivoting
constexpr int LDLT_RT = 128;  // rows per CTA in apply / commit / calc_ld

// One front taking part in a block-column step (or in TPP / calc_ld).
struct LdltFront {
  int64_t off;      // front (0,0) in the arena; ld x m column-major, lower used
  int64_t pan_off;  // scratch: L panel, w columns, indexed by front row (ld = m)
  int64_t ldp_off;  // scratch: L*D panel, same shape
  int64_t d_off;    // this front's D^-1 (2 per pivot, FP64, reference layout)
  int ld, m, n, p, w;
  int fidx;         // slot in the per-step arrays (blk, bdinv, lperm, npass)
  int var_off;      // this front's row -> pivot-order variable list
  int pad;
};

struct RowTask {
  int f;   // index into the LdltFront array of the launch
  int r0;  // first row of the tile
};

struct LdltStep {
  double* blk;      // per slot: LDLT_BW x (LDLT_BW+1) factored diagonal block (lower)
  double* bdinv;    // per slot: 2*LDLT_BW inverted D entries
  int* lperm;       // per slot: LDLT_BW local permutation
  int* npass_raw;   // per slot: first failing column from the apply test
  int* npass;       // per slot: passed pivots after the split-2x2 adjustment
  int* var;         // all fronts' variable lists
  double* dall;     // all fronts' D^-1
  unsigned* status;
  double u, small;
  int action;
};

template <typename T>
void launch_ldlt_diag(T* arena, const LdltFront* fr, int nf, LdltStep st, cudaStream_t s);
template <typename T>
void launch_ldlt_apply(const T* arena, T* scratch, const LdltFront* fr, const RowTask* rt,
                       int nt, LdltStep st, cudaStream_t s);
template <typename T>
void launch_ldlt_commit(T* arena, T* scratch, const LdltFront* fr, const RowTask* rt, int nt,
                        LdltStep st, cudaStream_t s);
// Threshold partial pivoting on columns [p, n) of each front; writes the
// number of eliminated columns (p + eliminated) to out_nelim[fidx].
template <typename T>
void launch_ldlt_tpp(T* arena, const LdltFront* fr, int nf, LdltStep st, double u_eff,
                     int* out_nelim, cudaStream_t s);
// L*D of rows [n, m), columns [0, nelim) into scratch (indexed by front row,
// ld = m) where LdltFront.p carries nelim and ldp_off the destination.
template <typename T>
void launch_ldlt_calc_ld(const T* arena, T* scratch, const LdltFront* fr, const RowTask* rt,
                         int nt, LdltStep st, cudaStream_t s);
// x[var[k]] = D^-1 x[var[k]] over the eliminated pivots of each front.
template <typename ACC>
void launch_solve_diag(const FrontDesc* fr, int nf, const int* var, const double* dall,
                       const int64_t* d_off, ACC* x, int n, int nrhs, cudaStream_t s);

}  // namespace sylver_gb300
