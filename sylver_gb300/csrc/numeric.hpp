// Host runtime of the GPU numeric phase: analysis handle (akeep), factor
// handle (fkeep), device memory, the level schedule and the solve driver.
//
// Replaces the reference's NumericTree / NumericTreePosdef objects
// (src/NumericTree.hxx:54-181, src/NumericTreePosdef.hxx:42-128) and the
// Fortran orchestration of factorize/solve (src/spldlt_factorize_mod.F90).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "analyse.hpp"
#include "device.hpp"
#include "tc.hpp"

namespace sylver_gb300 {

// Owned device allocation.
struct DevMem {
  void* p = nullptr;
  size_t bytes = 0;
  DevMem() = default;
  DevMem(const DevMem&) = delete;
  DevMem& operator=(const DevMem&) = delete;
  ~DevMem() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  void ensure(size_t nbytes) {
    if (nbytes <= bytes && p) return;
    release();
    if (nbytes == 0) return;
    SG_CUDA(cudaMalloc(&p, nbytes));
    bytes = nbytes;
  }
  template <typename T> T* as() const { return static_cast<T*>(p); }
  template <typename T> void upload(const std::vector<T>& v, cudaStream_t s) {
    ensure(std::max<size_t>(1, v.size()) * sizeof(T));
    if (!v.empty()) SG_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T),
                                            cudaMemcpyHostToDevice, s));
  }
};

// Kernel-path choices of the schedule (never the arithmetic).  Read when a
// factorization is planned; 0 selects the built-in default.
struct Schedule {
  int small_front_rows = 0;  // Cholesky: fronts with <= rows factorised whole by one CTA
  int tc_min_cb_rows = 0;    // FP32 Cholesky: CB rows for the tensor-core update (<0: never)
  int solve_large_cols = 0;  // fronts with >= eliminated columns use the blocked solve
  int ldlt_tpp_cols = 0;     // LDL^T: fronts with <= fully-summed columns use TPP only
  int fs_panel_cols = 0;     // FP32 Cholesky: outer panel width of the blocked large-front
                             // path (multiple of 64, <= 256; <0: 64-column SIMT steps)
  int fs_panel_group = 0;    // FP32 Cholesky: outer panels per trailing fully-summed update
  int front_memory = 0;      // front storage economy: 1 always, < 0 never, 0 when needed
  int solve_dataflow = 0;    // large-front solve sweeps (FP32): one dataflow launch per
                             // level (Cholesky >= 0, LDL^T > 0) or one launch per block step
  static Schedule& current();
  // default 96 rows: measured faster than the FP32 cap of 128 on 40^3, 56^3 and
  // 80^3 log-normal 27-point matrices (schedule sweeps of the learned scheduler)
  int small_rows(int compiled_max) const {
    return std::min(small_front_rows > 0 ? small_front_rows : 96, compiled_max);
  }
  int tc_rows() const { return tc_min_cb_rows == 0 ? 64 : tc_min_cb_rows; }
  int solve_cols() const { return solve_large_cols > 0 ? solve_large_cols : 96; }
  // 0: legacy SIMT panel steps, else the outer panel width
  int panel_cols() const {
    if (fs_panel_cols < 0) return 0;
    if (fs_panel_cols == 0) return 64;
    return std::max(BLK_B, std::min(BLK_W, fs_panel_cols / BLK_B * BLK_B));
  }
  int panel_group() const { return fs_panel_group > 0 ? std::min(fs_panel_group, 8) : 4; }
};

// Process-wide device context: device 0, one non-blocking stream.
struct Runtime {
  int device = -1;
  cudaStream_t stream = nullptr;
  bool ok = false;
  std::string err;
  static Runtime& get();
  bool init();  // returns false (and sets err) when no CUDA device is usable
};

struct AKeep {
  int n = 0;
  bool check = false;
  int flag = 0;
  int matrix_outrange = 0, matrix_dup = 0, matrix_missing_diag = 0;
  AnalyseResult clean;
  SymbolicTree st;
  // full symmetric CSR (user order) used by residual computations:
  // value of entry e = clean value fidx[e]
  std::vector<int64_t> frow;
  std::vector<int> fcol;
  std::vector<int64_t> fidx;
  void build_full_csr();
  // entries of the caller's val array the analysis refers to (computed once;
  // a scan of every map, too slow to repeat per factorization)
  int64_t nnz_val() const;
  mutable int64_t nz_val_ = -1;
  // per entry of the caller's val array: its row and column variable (user
  // order, 0-based; -1 for entries the analysis does not use), for the
  // scaling S A S.  Built on the first scaled factorization.
  std::vector<int> vrow, vcol;
  void build_val_rowcol();
  // scaling saved by the matching-based ordering (options.ordering = 2),
  // user order; used by factorize with options.scaling = 3
  std::vector<double> mscale;
};

// One kernel launch of the factor schedule.
struct Op {
  enum Kind { MEMSET, INIT, EA, SMALL, PANEL, UPD, DIAG, INV, SPLIT, TCUPD, BDIAG, BPANEL, EAG, ASM } kind;
  int64_t a = 0, b = 0;  // task range [a, b)
  int aux = 0;           // SMALL: max front rows; SPLIT/TCUPD: tensor-core level
};

struct Level {
  int f0 = 0, f1 = 0;  // fronts [f0, f1) of the level-ordered front table
};

// Solve schedule over a level-ordered front table.  Per level, the pivot
// rows of the small fronts (one CTA each, on chip) and of the large fronts
// (blocked multi-CTA sweeps) are solved; the contribution rows of all fronts
// of the level are one row-parallel launch per direction (forward after the
// pivot rows, backward before them).
struct SolvePlan {
  struct SOp {
    int kind;      // LsKind
    int64_t a, b;  // task range
    int aux = 0;   // LS_RECT_FWD: widest task's columns, rounded up to 16
  };
  struct Lv {
    int f0 = 0, nsmall = 0, nfront = 0;
    int small_maxn = 0;  // most pivot rows of the level's small fronts
    int64_t dfc_base = 0, dfc_count = 0;  // dataflow sweeps: the level's counters in dfcnt
    std::vector<SOp> fwd, bwd;
  };
  // Dataflow sweeps (LS_CHAIN_FWD / LS_CHAIN_BWD, task ranges in hdf) instead
  // of one launch per block step; set before build_tasks, which keeps it for
  // FP32 factors only.
  bool dataflow = true;
  std::vector<DfTask> hdf;
  std::vector<int2> hdfo;         // per level-ordered front: its counters (offset, count)
  std::vector<int64_t> httoff;    // per level-ordered front: its backward accumulators in tt
  int64_t dfc_elems = 0, df_tt_elems = 0;
  DevMem dftasks, dfo, ttoff, dfcnt, dferr;
  // the dataflow sweeps use P_ib = L_ib X_b, formed after each factorization
  // with the inverses (hpt: its tasks, p_elems floats)
  std::vector<PTask> hpt;
  int64_t p_elems = 0;
  DevMem ptasks, pmat;
  // error bits a dataflow sweep raised since the last call (ST_TIMEOUT), read
  // into *h by an asynchronous copy on s that the caller synchronizes
  void fetch_error(unsigned* h, cudaStream_t s);
  std::vector<Lv> lv;
  std::vector<LTask> htasks;
  std::vector<LTask> hinv;       // diagonal blocks to invert (f = level-ordered index)
  std::vector<int64_t> hinv_off; // per level-ordered front: offset of its inverses
  int64_t inv_elems = 0;
  std::vector<LTask> hinv2;       // 256-column diagonal blocks (f = level-ordered index)
  std::vector<int64_t> hinv2_off;
  int64_t inv2_elems = 0;
  DevMem tasks, tt, ys, inv, invt, inv_off, inv2, inv2t, invt2, inv2_off, tacc;
  int max_large = 0;
  // Invert every diagonal block of the large fronts (after a factorization).
  template <typename T>
  void compute_inverses(const T* arena, const FrontDesc* dfr, bool unit, cudaStream_t s);
  // Reorder each level small-first (perm[k] = old position of new k) and
  // build the task lists; hfr must already be in that order on entry to
  // build_tasks.
  static std::vector<int> small_first(const std::vector<FrontDesc>& hfr,
                                      const std::vector<Level>& levels);
  // elem: bytes of the factor's entries (the dataflow diagonal tasks' rows)
  void build_tasks(const std::vector<FrontDesc>& hfr, const std::vector<Level>& levels,
                   int elem, cudaStream_t s);
  void ensure_tt(size_t elem, int64_t scratch_elems, int n);
  template <typename T, typename ACC>
  void run(bool fwd, const T* arena, const FrontDesc* dfr, const int* rlist, ACC* x, int n,
           int nrhs, ACC* scratch, const int64_t* dscr, bool unit, cudaStream_t s);
  // Profiling (sylver_gb300_profile_solve): when set, run() records an event
  // after every launch, tagged with its kind (0 small fronts forward, 1 small
  // fronts backward, 2 + LsKind for the large-front launches).
  std::vector<std::pair<int, cudaEvent_t>>* prof = nullptr;
  void mark(int kind, cudaStream_t s);
};

struct FKeep {
  AKeep* ak = nullptr;
  bool posdef = true;
  int precision = 0;  // 0 FP64, 1 FP32
  double ir_tol = 1e-14;
  int ir_max_iter = 0;
  bool use_graph = true;
  // pivoting options (src/sylver_datatypes_mod.F90:57-72)
  double u = 0.01;
  double small_piv = 1e-20;
  bool action = true;
  // scaling S (user order, FP64 on the device): the factorization is of
  // S A S (init_a_block, src/kernels/assemble.hxx:162-180); solves apply S on
  // the way in and out by job (src/spldlt_factorize_mod.F90:945-1050)
  bool has_scale = false;
  DevMem dscale, dvrow, dvcol;
  void set_scale(const double* scale_host, cudaStream_t s);  // null: none
  void apply_scale(cudaStream_t s);  // val <- S val S in place (no-op without S)

  // tensor-core updates (FP32 Cholesky): stacked transposed operands, split
  // into three BF16 planes
  bool use_tc = true;
  struct TcLevel {
    int pitch;
    int64_t rows, max_rows;  // stacked panel rows; most rows of one split
    bool cb = false;         // operands in the contribution-block planes
  };
  std::vector<TcLevel> tclev;
  std::vector<CUtensorMap> tmaps;   // three per tensor-core launch (one per BF16 plane)
  DevMem tcsplit, tctask, tcplanes, tcerr;
  int64_t plane_stride = 0;        // elements between the BF16 planes
  DevMem cbplanes;                 // contribution-block operands written by the panel kernel
  int64_t cb_stride = 0;
  // blocked large-front path (FP32): diagonal-block and panel tasks, and the
  // 64 x 64 inverses of one diagonal-block launch
  DevMem blkdiag, blkpanel, blkinv;
  int64_t blkinv_count = 0;
  int blk_pw = 0;                  // outer panel width of the blocked path (0: unused)

  // host plan
  std::vector<int> order;            // level-ordered front indices
  std::vector<Level> levels;
  std::vector<int64_t> off;          // per front (original index)
  std::vector<int> ld;
  int64_t arena_elems = 0;
  std::vector<FrontDesc> hfr;        // level-ordered solve descriptors
  std::vector<int64_t> hscr;         // level-ordered scratch row offsets
  int64_t scratch_rows = 0;
  std::vector<Op> ops;
  std::vector<double> op_flops;      // algorithmic flops per op (update launches)
  std::vector<int> op_level;         // level of each op (-1: whole-factor set-up / inverses)
  bool init_atomic = false;
  int64_t ninit = 0;
  // fronts assembled column by column in one pass per level (k_assemble)
  // instead of zeroing + original entries + extend-add
  bool one_pass = false;
  // Cholesky: front blocks placed with contribution blocks given back (when
  // all blocks would take more than half of the device memory)
  bool reuse_blocks = false;

  // device data
  DevMem arena, val, cval, faval, frow, fcol, fidx, srcptr, src, status, anorm;
  // LDL^T with the factor columns copied out of the front blocks (set when
  // the fronts' blocks would not fit with only their contribution blocks
  // given back): the solves read the compact store instead of the arena
  DevMem fstore;
  bool fcopy = false;
  const void* factor_base() const { return fcopy ? fstore.p : arena.p; }
  size_t factor_bytes() const { return fcopy ? fstore.bytes : arena.bytes; }
  DevMem amap_src, amap_dst, cdesc, eaitems, eamaps, eagroups, small, panel, upd, diagt, zerot;
  DevMem asmt, asm_acp, asm_arow, asm_asrc, asm_gptr;
  int nzero = 0;
  DevMem dfr, dscr, rlist0, perm0;
  DevMem xp, scratch, bcopy, resid, norms;
  cudaGraphExec_t graph = nullptr;
  double anorm_h = 0.0;

  // statistics
  long launches = 0;
  double factor_ms = 0.0;
  int last_ir_iters = 0;
  double last_bwd_err = 0.0;
  std::vector<double> ir_hist;  // backward error after each solve of the last refinement
  int flag = 0;
  int num_neg = 0, num_two = 0, num_delay = 0, num_zero = 0, rank = 0;
  int maxfront = 0;
  int64_t num_factor = 0, num_flops = 0;
  int not_first_pass = 0, not_second_pass = 0;

  // LDL^T state (ldlt.cpp)
  std::shared_ptr<struct LdltState> ldlt;
  SolvePlan splan;

  // captured solve sweeps, keyed by job, right-hand sides and buffers
  struct SolveGraph {
    int job, nrhs;
    const void *x, *scratch, *tt;
    cudaGraphExec_t exec;
  };
  std::vector<SolveGraph> sgraphs;
  void clear_solve_graphs();
  // Run `body` (a launch sequence on stream s) through a cached graph.
  template <typename F>
  void replay(int job, int nrhs, const void* x, cudaStream_t s, F&& body) {
    for (auto& g : sgraphs)
      if (g.job == job && g.nrhs == nrhs && g.x == x && g.scratch == scratch.p &&
          g.tt == splan.tt.p) {
        SG_CUDA(cudaGraphLaunch(g.exec, s));
        return;
      }
    cudaGraph_t gr;
    SG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      body();
    } catch (...) {
      // leave the stream out of capture mode before reporting the error
      if (cudaStreamEndCapture(s, &gr) == cudaSuccess && gr) cudaGraphDestroy(gr);
      throw;
    }
    SG_CUDA(cudaStreamEndCapture(s, &gr));
    cudaGraphExec_t ex;
    SG_CUDA(cudaGraphInstantiate(&ex, gr, 0));
    cudaGraphDestroy(gr);
    sgraphs.push_back({job, nrhs, x, scratch.p, splan.tt.p, ex});
    SG_CUDA(cudaGraphLaunch(ex, s));
  }

  ~FKeep();
  void plan_cholesky();
  void upload_static(cudaStream_t s);
  // Factorize from device values (val_dev: original val layout, nnz entries).
  int factorize(const double* val_dev, cudaStream_t s);
  // Solve in place on device; x is ldx x nrhs in user order.
  int solve(int job, int nrhs, double* x_dev, int ldx, cudaStream_t s);
  // Solve with x already in pivot order (the tree-level seam), FP64 only.
  int solve_raw(int job, int nrhs, double* x_dev, int ldx, cudaStream_t s);
  // Per-kind timing of the factor schedule (see sylver_gb300_profile_factor);
  // level_ms (optional, one entry per level) receives the time per level.
  int profile(const double* val_dev, double* ms, long* launches, double* flops, cudaStream_t s,
              double* level_ms = nullptr);
  // Per-kind timing of one forward + backward sweep (see sylver_gb300_profile_solve).
  int profile_solve(int nrhs, double* ms, long* launches, cudaStream_t s);

 public:
  template <typename T> void run_ops(cudaStream_t s);
  template <typename T> void solve_pivot_order(int job, void* xp, int nrhs, cudaStream_t s);
  int64_t nnz_orig() const;
};

}  // namespace sylver_gb300
