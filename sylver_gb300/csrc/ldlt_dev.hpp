// Device-side descriptors and launchers of the threshold-pivoted LDL^T path.
#pragma once

#include "device.hpp"

namespace sylver_gb300 {

constexpr int LDLT_BW = 32;   // block width of the a-posteriori pivoting
constexpr int LDLT_RT = 128;  // rows per CTA tile in apply / commit / calc_ld

// One front of a level (fixed for the level; everything that pivoting
// changes lives in the per-slot state arrays of LdltStep).
struct LdltFront {
  int64_t off;      // front (0,0) in the arena; ld x m column-major, lower used
  int64_t pan_off;  // scratch: apply output, LDLT_BW columns indexed by front row (ld = m)
  int64_t ldp_off;  // scratch: L*D of the passed columns, same shape
  int64_t mv_off;   // scratch: m x n copy used to move failed columns behind the others
  int64_t d_off;    // this front's D^-1 (2 per pivot, FP64, reference layout)
  int ld, m, n;
  int fidx;         // slot in the per-level state arrays
  int var_off;      // this front's row -> pivot-order variable list
  int mvvar_off;    // int scratch (n entries) for the variable list during a move
  int nblk;         // a-posteriori block steps (0: threshold partial pivoting only)
  int p;            // calc_ld: number of eliminated columns
};

// CTA of a launch -> front (index into the launch's LdltFront array), the
// CTA's index within that front's slice and the slice size.  A kernel whose
// work depends on pivoting strides over its front's work in steps of count.
struct CtaMap {
  int f, local, count, pad;
};

// State of block step k.  Slots advance independently: p (columns
// eliminated by the block steps so far, which is also where block k starts)
// and nf (columns that failed, kept at the end of the fully-summed range)
// are read from *_cur and written to *_next; p_final gets p after a front's
// last block step.
struct LdltStep {
  double* blk;       // per slot: LDLT_BW x (LDLT_BW+1) factored diagonal block
  double* bdinv;     // per slot: 2*LDLT_BW inverted D entries
  int* lperm;        // per slot: LDLT_BW local permutation
  int* ndiag;        // per slot: pivots the diagonal block factorization took
  int* npass_raw;    // per slot: least failing pivot of the a-posteriori test
  int* npass;        // per slot: passed pivots after dropping a split 2x2
  const int* p_cur;
  const int* nf_cur;
  int* p_next;
  int* nf_next;
  int* p_final;
  int* var;          // all fronts' variable lists
  int* mvvar;        // int scratch
  double* dall;      // all fronts' D^-1
  unsigned* status;
  double u, small;
  int action;
  int k;             // block step
};

// Block step k, in this order on one stream: diagonal block (one CTA per
// front with nblk > k), rows below (apply + threshold test), commit (L,
// restore failed columns, L*D, D, state), move of the failed columns behind
// the unprocessed ones (copy, then write), trailing update of the
// fully-summed columns.  Each takes its own CTA map.
template <typename T>
void launch_app_diag(T* arena, T* scratch, const LdltFront* fr, const CtaMap* cm, int ncta,
                     LdltStep st, cudaStream_t s);
template <typename T>
void launch_app_apply(const T* arena, T* scratch, const LdltFront* fr, const CtaMap* cm, int ncta,
                      LdltStep st, cudaStream_t s);
template <typename T>
void launch_app_commit(T* arena, T* scratch, const LdltFront* fr, const CtaMap* cm, int ncta,
                       LdltStep st, cudaStream_t s);
template <typename T>
void launch_app_move(T* arena, T* scratch, const LdltFront* fr, const CtaMap* cm, int ncta,
                     LdltStep st, cudaStream_t s);
template <typename T>
void launch_app_update(T* arena, const T* scratch, const LdltFront* fr, const CtaMap* cm,
                       int ncta, LdltStep st, cudaStream_t s);
// Threshold partial pivoting on columns [pstart[fidx], n) of each front (all
// rows below); writes the number of eliminated columns to out_nelim[fidx].
template <typename T>
void launch_ldlt_tpp(T* arena, const LdltFront* fr, int nf, LdltStep st, double u_eff,
                     const int* pstart, int* out_nelim, cudaStream_t s);
// L*D of rows [n, m), columns [0, nelim) into scratch (indexed by front row,
// ld = m) where LdltFront.p carries nelim and ldp_off the destination.
template <typename T>
void launch_ldlt_calc_ld(const T* arena, T* scratch, const LdltFront* fr, const CtaMap* cm,
                         int ncta, LdltStep st, cudaStream_t s);
// x[var[k]] = D^-1 x[var[k]] over the eliminated pivots of each front.
template <typename ACC>
void launch_solve_diag(const FrontDesc* fr, int nf, const int* var, const double* dall,
                       const int64_t* d_off, ACC* x, int n, int nrhs, cudaStream_t s);

}  // namespace sylver_gb300
