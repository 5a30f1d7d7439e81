// Shared device-side definitions: task descriptors of the level schedule,
// status bits written by kernels, and the launcher entry points of each
// kernel translation unit.
#pragma once

#include <cuda_runtime.h>
#if defined(__CUDACC__)
#include <cuda_bf16.h>
#endif
#include <cstdint>
#include <stdexcept>
#include <string>

namespace sylver_gb300 {

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& s) : std::runtime_error(s) {}
};

#define SG_CUDA(call)                                                              \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      throw ::sylver_gb300::CudaError(std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Status bits accumulated (atomicOr) by kernels into one device word.
enum : unsigned {
  ST_NOT_POSDEF = 1u,     // non-positive / NaN pivot in a Cholesky front
  ST_ZERO_PIVOT = 2u,     // LDL^T eliminated a zero pivot (action = true)
  ST_SINGULAR = 4u,       // LDL^T zero pivot with action = false
  ST_OVERFLOW = 8u,       // a front outgrew its planned storage
  ST_BAD_INDEX = 16u,     // an index map pointed outside its front
  ST_TIMEOUT = 32u,       // a bounded wait inside a kernel gave up
};

#if defined(__CUDACC__)
// Asynchronous global -> shared copy of one element (cp.async, 4/8 bytes):
// every copy a thread issued lands once it passes cp_async_wait_all(); a
// __syncthreads() afterwards makes them visible to the whole CTA.  Lets a
// thread keep many loads in flight instead of one per loop iteration.
template <typename T>
__device__ __forceinline__ void cp_async(T* smem, const T* gmem) {
  static_assert(sizeof(T) == 4 || sizeof(T) == 8, "cp.async element size");
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}
// 16-byte asynchronous copy global -> shared (both addresses 16-byte
// aligned), and the commit / wait of groups of copies (the wait returns once
// at most N of the thread's committed groups are still in flight).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// Programmatic dependent launch (kernels launched with launch_pdl): the
// trigger lets the next launch of the stream start at once; the wait blocks
// until the previous grid has completed and its writes are visible.  Every
// kernel launched with launch_pdl waits in each CTA before its first read of
// data an earlier launch wrote, so a grid completes only after its
// predecessor did.
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
#endif

// Launch with programmatic stream serialization (see pdl_wait).
template <typename... KArgs, typename... Args>
void launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  SG_CUDA(cudaLaunchKernelEx(&cfg, kern, args...));
}

// ---------------------------------------------------------------------------
// Task descriptors (one per CTA unless stated).

// Dense front stored column-major, full m x m square at arena[off], leading
// dimension ld; only the lower triangle is meaningful.
struct FrontDesc {
  int64_t off;
  int ld, m, n;   // rows, fully-summed columns
  int rl;         // offset of the front's pivot-order row list (0-based ints)
  int pad;
};

// Zeroing before assembly: columns [j0, j1) of a front, rows j .. m - 1 of
// column j (the lower triangle; nothing reads the upper one).
struct ZeroTask {
  int64_t off;
  int ld, m, j0, j1;
};

// Whole small front factorized by one CTA in shared memory.
struct SmallTask {
  int64_t off;
  int ld, m, n, pad;
};

// Panel step: Cholesky of the w x w diagonal block at (k0,k0) (one task per
// front) or the triangular solve of rows [r0, r1) of columns [k0, k0+w).
struct PanelTask {
  int64_t off;
  int ld, k0, w, r0, r1, pad;
};

// Tile update C(i,j) -= sum_k A(i,k) B(j,k) with
//   C(i,j) = arena[c_off + j*ldc + i], B(j,k) = arena[b_off + k*ldb + j],
//   A(i,k) = abuf[a_off + k*lda + i]  (abuf is the arena itself for Cholesky,
//   an L*D panel for LDL^T),
// rows [row0, min(row0+TM,rowEnd)), cols [col0, min(col0+TN,colEnd)), only
// i >= j written, inner index k in [k0, k1).
struct UpdTask {
  int64_t c_off, a_off, b_off;
  int ldc, lda, ldb, row0, col0, rowEnd, colEnd, k0, k1, pad;
};

// Blocked FP32 Cholesky of large fronts (kernels_blocked.cu): panels of at
// most BLK_W columns (a multiple of BLK_B by schedule choice).
constexpr int BLK_B = 64;
constexpr int BLK_W = 256;
// k per pipeline stage of the tensor-core update (BF16 elements); stacked
// panel pitches are multiples of it
constexpr int TC_KCHUNK = 64;
// Panel [c, c + bw) of a front (pend = c + bw); xi indexes the panel's
// 16 x 16 sub-block inverses (BLK_B * BLK_B floats) in the launch's
// scratch.  For the panel kernel r0 is the first of the CTA's 64 rows
// (>= pend), and base >= 0 is the stacked tensor-core panel row of front row
// pend, where the kernel writes the rows it solves (transposed, split into
// three BF16 planes) for the later tensor-core updates, at K columns
// [c mod pitch, + panel width) of planes with pitch K columns; base < 0: no
// later update reads the panel.  cbbase >= 0: the front's contribution
// rows (>= n) are also written, at K columns [c, c + panel width) clipped to
// n rounded up to 64, to the contribution-block operand planes (pitch
// cbpitch), stacked row cbbase for front row n.
struct BlkTask {
  int64_t off;
  int ld, m, c, bw, pend, r0, xi, base;
  int n, cbbase, cbpitch;
};

#if defined(__CUDACC__)
// FP32 -> x0 + x1 + x2, three BF16 parts (round to nearest at each step; both
// remainders are exact in FP32): the operand split of the 3xBF16
// tensor-core update.  Returned as raw 16-bit patterns.
__device__ __forceinline__ void bf16x3_split(float v, uint16_t& b0, uint16_t& b1,
                                             uint16_t& b2) {
  const __nv_bfloat16 h0 = __float2bfloat16_rn(v);
  const float r1 = v - __bfloat162float(h0);
  const __nv_bfloat16 h1 = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(h1);
  const __nv_bfloat16 h2 = __float2bfloat16_rn(r2);
  b0 = __bfloat16_as_ushort(h0);
  b1 = __bfloat16_as_ushort(h1);
  b2 = __bfloat16_as_ushort(h2);
}
#endif

// Extend-add of one child contribution column into its parent; the entry
// (i, j), i >= j, of the child block lands at (max, min) of the mapped rows
// (maps are monotone for Cholesky, not once delayed columns move up).
struct ChildDesc {
  int64_t cb_off;   // child CB (0,0) in the arena
  int64_t p_off;    // parent front (0,0)
  int ld_c, ld_p, mc, map_off;
};
struct EaItem {
  int child;  // index into ChildDesc array
  int col;    // CB column
};

// ---------------------------------------------------------------------------
// Launchers (kernels_factor.cu)

template <typename T>
void prepare_factor_kernels();
template <typename T>
void launch_zero_lower(T* arena, const ZeroTask* t, int ntask, cudaStream_t s);
// arena[off, off + len) <- 0 for each span (off, len multiples of 64 elements)
struct ZeroSpan {
  int64_t off, len;
};
template <typename T>
void launch_zero_spans(T* arena, const ZeroSpan* t, int ntask, cudaStream_t s);
// dst[d, d + len) <- src[o, o + len) for each span (multiples of 4 elements,
// 16-byte aligned)
struct CopySpan {
  int64_t src, dst, len;
};
template <typename T>
void launch_copy_spans(T* dst, const T* src, const CopySpan* t, int ntask, cudaStream_t s);
template <typename T>
void launch_init_a(T* arena, const double* val, const int64_t* src, const int64_t* dst,
                   int64_t count, bool atomic, cudaStream_t s);
// Groups g of items [grp[g], grp[g + 1]) that land in one parent column, in
// child order; one warp per group, no atomics (maps must keep row order).
template <typename T>
void launch_extend_add_grouped(T* arena, const ChildDesc* cd, const EaItem* items,
                               const int* grp, const int* maps, int ngroups, cudaStream_t s);
// Assembly of whole front columns in one pass: columns [j0, j1) of the front
// at off (m rows, leading dimension ld); column j's original entries are
// arow/asrc[acp[cbase + j], acp[cbase + j + 1]) (distinct rows >= j) and the
// children's CB columns that land in it are items[gptr[cbase + j],
// gptr[cbase + j + 1]) in child order (at most 32, maps that keep row order).
struct AsmTask {
  int64_t off;
  int ld, m, j0, j1, cbase, pad;
};
template <typename T>
void launch_assemble(T* arena, const double* val, const AsmTask* t, int ntask, const int* acp,
                     const int* arow, const int64_t* asrc, const int* gptr, const EaItem* items,
                     const ChildDesc* cd, const int* maps, cudaStream_t s);
// atomic = false: at most one child per parent in this launch (see kernel).
template <typename T>
void launch_extend_add(T* arena, const ChildDesc* cd, const EaItem* items, const int* maps,
                       int nitems, cudaStream_t s, bool atomic = true);
template <typename T>
void launch_small_chol(T* arena, const SmallTask* t, int ntask, int maxm, unsigned* status,
                       cudaStream_t s);
template <typename T>
void launch_diag_chol(T* arena, const PanelTask* t, int ntask, unsigned* status,
                      cudaStream_t s);
template <typename T>
void launch_panel_trsm(T* arena, const PanelTask* t, int ntask, cudaStream_t s);
template <typename T>
void launch_update(T* arena, const T* abuf, const UpdTask* t, int ntask, cudaStream_t s);

// Launchers (kernels_blocked.cu), FP32 only.  xinv holds one 64 x 64
// inverse per diagonal-block task of the launch.
void prepare_blocked_kernels();
void launch_blk_diag(float* arena, const BlkTask* t, int ntask, float* xinv, unsigned* status,
                     cudaStream_t s);
// pw: the panel width (shared-memory layout), pitch: K columns of the planes;
// cbplanes / cbpstride: the contribution-block operand planes.
void launch_blk_panel(float* arena, const BlkTask* t, int ntask, const float* xinv,
                      uint16_t* planes, int64_t pstride, int pw, int pitch, uint16_t* cbplanes,
                      int64_t cbpstride, cudaStream_t s);

template <typename T> struct Tiles;
template <> struct Tiles<double> {
  static constexpr int TM = 64, TN = 64, NB = 32, RT = 128, SMALL_M = 96;
};
template <> struct Tiles<float> {
  static constexpr int TM = 128, TN = 128, NB = 64, RT = 128, SMALL_M = 128;
};

// ---------------------------------------------------------------------------
// Launchers (kernels_solve.cu).  ACC is the solve's accumulation type.
// scr_off[f] is the first scratch row of front f; its slab is m x nrhs.

template <typename T, typename ACC>
void launch_solve_fwd(const T* arena, const FrontDesc* fr, int nfronts, const int* rlist,
                      ACC* x, int n, int nrhs, ACC* scratch, const int64_t* scr_off,
                      bool unit_diag, cudaStream_t s);
// Small fronts (at most maxn pivot rows), one CTA each, pivot rows only:
// forward y = L11^-1 x(pivots); backward z = L11^-T (x(pivots) - tacc), tacc
// cleared.  The contribution rows are the LS_RECT_FWD / LS_RECT_BWD launches.
template <typename T, typename ACC>
void launch_small_tri(bool fwd, const T* arena, const FrontDesc* fr, int nfronts,
                      const int* rlist, ACC* x, ACC* tacc, int n, int nrhs, int maxn,
                      bool unit_diag, cudaStream_t s);

// Large-front blocked sweeps (block width 64).  Task f indexes the level's
// FrontDesc array; c0/bw give the diagonal block, r0 the first row of a tile.
struct LTask {
  int f, c0, bw, r0;
  int ntiles;  // backward step: row tiles of this front in the launch
  int pad;
};
enum LsKind {
  LS_GATHER_FWD, LS_GATHER_BWD, LS_SCATTER_FWD, LS_SCATTER_BWD,
  LS_FWD_DIAG2, LS_FWD_UPD2, LS_BWD_RED2, LS_BWD_DIAG2,
  LS_RECT_BWD,  // contribution rows' share of every pivot row, before the level (backward)
  LS_RECT_FWD,  // contribution rows' update from all pivot rows, after the level (forward)
  LS_SMALL_TRI,  // the level's small fronts (launch_small_tri)
  LS_CHAIN_FWD,  // the large fronts' block steps of a level as one dataflow launch (launch_chain)
  LS_CHAIN_BWD
};
// One task of a dataflow sweep (launch_chain, FP32 factors): the large
// fronts' block steps of one level in one launch.  CTAs take tasks in list
// order (an atomic ticket); the list is a topological order of the
// dependencies, so a task waits only on tasks taken earlier by running CTAs.
// Before reading data an earlier task writes, a task waits until counters
// [w0, w0 + nw) are all >= need0 and counter w1 (if >= 0) is >= need1; when
// done it adds one to counter sig.  Counter 0 of a level is the ticket.
// With the products P_ib = L_ib X_b (formed after the factorization) no
// diagonal mat-vec sits on the chain of block steps:
//   DF_UPD_FWD   x_i -= P_ib x_b, rows [r0, r0 + 32) below block b, once x_b
//                is final (the rows of block b + 1 first: the chain)
//   DF_DIAG_FWD  y_b = X_b x_b (x_b final), output rows [sub*16, +16)
//   DF_DIAG_BWD  u_b = X_b^T x_b for every block, first
//   DF_RED_BWD   z_j = u_j - t_j for rows [r0, r0 + 32) of block j, then
//                t_b += P_jb^T z_j (sub = 1: b = j - 1, the task that also
//                stores z_j in the xs slab)
//   DF_FIN_BWD   z_0 = u_0 - t_0, rows [r0, r0 + 32)
// P_ib sits at pofs in LsArgs::pmat, column-major with leading dimension ldp
// (rows from the first row below the block).
enum DfKind { DF_DIAG_FWD, DF_UPD_FWD, DF_RED_BWD, DF_DIAG_BWD, DF_FIN_BWD };
struct DfTask {
  int kind, f, c0, bw, r0, sub;
  int w0, nw, need0, w1, need1, sig;
  int ldp, pad;
  int64_t pofs;
};
// Formation of P_ib = L_ib X_b: rows [r0, r0 + 64) (from c1, the first row
// below the block [c0, c1)) of front f's block, into pmat + pofs (ld ldp).
struct PTask {
  int f, c0, c1, r0, ldp, pad;
  int64_t pofs;
};
constexpr int LSOLVE_BW = 64;    // inverted diagonal sub-blocks
constexpr int LSOLVE_BW2 = 256;  // columns per solve step (diagonal block with an explicit inverse)
constexpr int LSOLVE_TW = 256;   // columns of the L tiles of the update and reduction tasks
constexpr int LSOLVE_UPD_ROWS = 32;  // rows per forward-update CTA
constexpr int LSOLVE_RED_ROWS = 64;  // rows per backward-reduction CTA
constexpr int RECT_FWD_T = 128;      // threads of an LS_RECT_FWD task (two contribution rows each)
constexpr int RECT_FWD_COLS = 128;   // pivot columns per LS_RECT_FWD task (partial sums add atomically)
constexpr int RECT_BWD_COLS = 128;   // pivot columns per LS_RECT_BWD task
constexpr int RECT_BWD_T = 128;      // threads of an LS_RECT_BWD task (two columns each, two row halves)
constexpr int RECT_BWD_ROWS = 256;   // contribution rows per LS_RECT_BWD task
// Large fronts are swept block by block over their fully-summed rows only.
// The contribution rows (>= n) of every front of a level are one separate
// launch per direction: forward after the pivot rows are solved (x(cb) -=
// L21 y, LS_RECT_FWD), backward before them (tacc(pivots) = L21^T x(cb),
// LS_RECT_BWD; the pivot rows' gather subtracts and clears it).
// Buffers of the large-front sweeps, per level: xs/ys slabs (scratch, ys),
// explicit inverses of the 64x64 diagonal blocks (inv + inv_off[f] + block
// index), tt: two 256 x 32 accumulators per front (backward steps alternate
// between them; the backward gather clears both), entry (column k, right-hand
// side r) at r * 256 + k, so that a warp's atomic additions for 32
// consecutive columns fall in one cache line.
template <typename T, typename ACC>
struct LsArgs {
  const T* arena;
  const FrontDesc* fr;
  const int* rlist;
  ACC* x;
  int n, nrhs;
  ACC* scratch;
  ACC* ys;
  const int64_t* scr_off;
  const T* inv;
  const int64_t* inv_off;
  ACC* tt;
  const T* inv2;            // LSOLVE_BW2-square inverses of the solve-step diagonal blocks
  const int64_t* inv2_off;  // per front of the level
  const T* inv2t;           // the same inverses transposed (row-major)
  // contribution rows' share of the backward reduction, laid out like x
  // (n x nrhs, column stride n); zero between backward sweeps
  ACC* tacc;
  // dataflow sweeps (null otherwise): the level's counters, per front of
  // the level its counter range (offset, count) and the offset of its
  // per-block backward accumulators in tt (256 x 32 per 256-column block);
  // the gathers clear both
  int* dfc;
  const int2* dfo;
  const int64_t* ttoff;
  // dataflow sweeps (FP32): the products P_ib = L_ib X_b; pmode: the
  // backward sweep leaves z in the xs slab for the scatter
  const T* pmat;
  int pmode;
};
// Inverse of each solve-step diagonal block (LSOLVE_BW2 columns) from its
// 64x64 inverses: task (front f, c0, bw), output at inv2 + inv2_off[f] +
// (c0/LSOLVE_BW2)*LSOLVE_BW2^2 (column-major) and, transposed, at the same
// offset of inv2t.
template <typename T>
void prepare_solve_kernels();
template <typename T>
void launch_inv_block(const T* arena, const FrontDesc* fr, const LTask* tasks, int ntask,
                      const T* inv64, const int64_t* inv_off, T* inv2, T* inv2t,
                      const int64_t* inv2_off, cudaStream_t s);
template <typename T, typename ACC>
void launch_lsolve(int kind, const LTask* tasks, int ntask, LsArgs<T, ACC> a, int aux,
                   cudaStream_t s);
// Dataflow sweep over the large fronts of one level (a.dfc: its counters,
// zeroed by the gather before it): persistent CTAs, at most one per task.
// A wait that runs past its bound sets ST_TIMEOUT in *err and the task goes
// on (its result is then wrong, and the caller reports the error).
void launch_chain(bool bwd, const DfTask* tasks, int ntask, LsArgs<float, float> a, unsigned* err,
                  cudaStream_t s);
// P_ib = L_ib X_b for every task (FP32; X from inv2t, row-major).
void launch_form_p(const float* arena, const FrontDesc* fr, const PTask* tasks, int ntask,
                   const float* inv2t, const int64_t* inv2_off, float* pmat, cudaStream_t s);
// Explicit inverse of each diagonal block: task (front f, c0, bw), output at
// inv + inv_off[f] + (c0/64)*64*64, column-major 64 x 64, identity padded.
template <typename T>
void launch_inv_diag(const T* arena, const FrontDesc* fr, const LTask* tasks, int ntask,
                     T* inv, const int64_t* inv_off, bool unit, cudaStream_t s);

// xp[perm[i]] = x[i] * scale[i] (scale null: 1), per right-hand side.
template <typename ACC>
void launch_permute_in(const double* x, int ldx, ACC* xp, const int* perm, const double* scale,
                       int n, int nrhs, cudaStream_t s);
// x[i] (+)= xp[perm[i]] * scale[i] (scale null: 1), per right-hand side.
template <typename ACC>
void launch_permute_out_add(const ACC* xp, const int* perm, const double* scale, double* x,
                            int ldx, int n, int nrhs, bool add, cudaStream_t s);
// val[k] = (scale[row[k]] * val[k]) * scale[col[k]] for entries with row >= 0.
void launch_scale_vals(double* val, const int* row, const int* col, const double* scale,
                       int64_t count, cudaStream_t s);

// r = b - A x for a full CSR matrix (user order), FP64.
void launch_residual(const int64_t* rowptr, const int* col, const double* aval, int n,
                     const double* x, int ldx, const double* b, int ldb, double* r, int nrhs,
                     cudaStream_t s);
// norms[3*r+0] = max|res|, [3r+1] = max|x|, [3r+2] = max|b|  (atomic max).
void launch_maxnorms(const double* res, const double* x, int ldx, const double* b, int ldb,
                     int n, int nrhs, double* norms, cudaStream_t s);
// out = max_i sum_j |a_ij| (atomic max into *out).
void launch_rownorm_inf(const int64_t* rowptr, const double* aval, int n, double* out,
                        cudaStream_t s);
// clean values: cval[k] = sum val[src[srcptr[k]..srcptr[k+1])]; then full
// CSR values aval[e] = cval[eidx[e]].
void launch_gather_clean(const double* val, const int64_t* srcptr, const int64_t* src,
                         int64_t nclean, double* cval, cudaStream_t s);
void launch_gather(const double* cval, const int64_t* idx, int64_t count, double* out,
                   cudaStream_t s);
void launch_axpy_inplace(double* x, int ldx, const double* d, int n, int nrhs, cudaStream_t s);

// LDL^T launchers (kernels_ldlt.cu) are declared in ldlt.hpp.

}  // namespace sylver_gb300
