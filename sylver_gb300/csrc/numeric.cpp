// Host runtime: level schedule planning, device memory, CUDA-graph replay of
// the factorization and the solve / iterative-refinement driver.
//
// The reference walks fronts in postorder and inserts StarPU tasks per tile
// (src/NumericTreePosdef.hxx:133-353, src/NumericTree.hxx:186-406).  Here the
// fronts are grouped by height in the assembly tree ("levels"); every launch
// covers all fronts of a level, so independent subtrees share kernels and the
// whole posdef factorization is one captured CUDA graph.
#include "numeric.hpp"
#include "arena_alloc.hpp"
#include "ldlt.hpp"
#include "../../include/sylver_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <climits>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <type_traits>

namespace sylver_gb300 {

Runtime& Runtime::get() {
  static Runtime rt;
  return rt;
}

Schedule& Schedule::current() {
  static Schedule s;
  return s;
}

bool Runtime::init() {
  if (ok) return true;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    err = std::string("no CUDA device: ") + cudaGetErrorString(e);
    cudaGetLastError();
    return false;
  }
  e = cudaSetDevice(0);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    err = cudaGetErrorString(e);
    return false;
  }
  device = 0;
  try {
    prepare_factor_kernels<float>();
    prepare_factor_kernels<double>();
    prepare_tc_kernels();
    prepare_blocked_kernels();
    prepare_solve_kernels<float>();
    prepare_solve_kernels<double>();
  } catch (const std::exception& ex) {
    err = ex.what();
    fprintf(stderr, "sylver_gb300: device set-up failed: %s\n", err.c_str());
    return false;
  }
  ok = true;
  return true;
}

void AKeep::build_full_csr() {
  const int nn = n;
  std::vector<int64_t> cnt(nn + 1, 0);
  for (int c = 0; c < nn; ++c)
    for (int64_t k = clean.cptr[c]; k < clean.cptr[c + 1]; ++k) {
      int r = clean.crow[k];
      cnt[r + 1]++;
      if (r != c) cnt[c + 1]++;
    }
  frow.assign(nn + 1, 0);
  for (int i = 0; i < nn; ++i) frow[i + 1] = frow[i] + cnt[i + 1];
  fcol.assign(frow[nn], 0);
  fidx.assign(frow[nn], 0);
  std::vector<int64_t> pos(frow.begin(), frow.end() - 1);
  for (int c = 0; c < nn; ++c)
    for (int64_t k = clean.cptr[c]; k < clean.cptr[c + 1]; ++k) {
      int r = clean.crow[k];
      fcol[pos[r]] = c;
      fidx[pos[r]++] = k;
      if (r != c) {
        fcol[pos[c]] = r;
        fidx[pos[c]++] = k;
      }
    }
}

void FKeep::clear_solve_graphs() {
  for (auto& g : sgraphs) cudaGraphExecDestroy(g.exec);
  sgraphs.clear();
}

FKeep::~FKeep() {
  if (graph) cudaGraphExecDestroy(graph);
  clear_solve_graphs();
}

int64_t AKeep::nnz_val() const {
  if (nz_val_ >= 0) return nz_val_;
  int64_t mx = 0;
  for (int64_t s : clean.src) mx = std::max(mx, s + 1);
  const auto& nl = st.nlist;
  for (size_t k = 0; k < nl.size(); k += 2) mx = std::max<int64_t>(mx, nl[k]);
  nz_val_ = mx;
  return mx;
}

int64_t FKeep::nnz_orig() const { return ak->nnz_val(); }

void AKeep::build_val_rowcol() {
  const int64_t nz = nnz_val();
  if ((int64_t)vrow.size() == nz) return;
  vrow.assign(nz, -1);
  vcol.assign(nz, -1);
  if (!clean.crow.empty()) {
    for (int c = 0; c < n; ++c)
      for (int64_t k = clean.cptr[c]; k < clean.cptr[c + 1]; ++k)
        for (int64_t q = clean.srcptr[k]; q < clean.srcptr[k + 1]; ++q) {
          vrow[clean.src[q]] = clean.crow[k];
          vcol[clean.src[q]] = c;
        }
    return;
  }
  // tree-level seam: val is indexed by nlist sources, the variables are the
  // rlist values (entry dest of a front is row dest % nrow, column dest / nrow)
  for (int f = 0; f < st.nnodes; ++f) {
    const int64_t r0 = st.rptr[f] - 1;
    const int64_t nrow = st.rptr[f + 1] - st.rptr[f];
    for (int64_t k = st.nptr[f] - 1; k < st.nptr[f + 1] - 1; ++k) {
      const int64_t srcv = st.nlist[2 * k] - 1, dst = st.nlist[2 * k + 1] - 1;
      vrow[srcv] = st.rlist[r0 + dst % nrow] - 1;
      vcol[srcv] = st.rlist[r0 + dst / nrow] - 1;
    }
  }
}

void FKeep::set_scale(const double* scale_host, cudaStream_t s) {
  has_scale = scale_host != nullptr && ak->n > 0;
  if (!has_scale) return;
  ak->build_val_rowcol();
  if (dvrow.bytes < ak->vrow.size() * sizeof(int) || !dvrow.p) {
    dvrow.upload(ak->vrow, s);
    dvcol.upload(ak->vcol, s);
  }
  dscale.ensure((size_t)ak->n * sizeof(double));
  SG_CUDA(cudaMemcpyAsync(dscale.p, scale_host, (size_t)ak->n * sizeof(double),
                          cudaMemcpyHostToDevice, s));
}

void FKeep::apply_scale(cudaStream_t s) {
  if (!has_scale) return;
  launch_scale_vals(val.as<double>(), dvrow.as<int>(), dvcol.as<int>(), dscale.as<double>(),
                    nnz_orig(), s);
}

namespace {
// fronts that get the blocked multi-CTA solve
inline bool is_large(const FrontDesc& d) {
  return d.n >= Schedule::current().solve_cols() || (int64_t)d.m * d.n >= (1 << 16);
}
inline int round_up(int v, int a) { return (v + a - 1) / a * a; }
inline int64_t round_up64(int64_t v, int64_t a) { return (v + a - 1) / a * a; }
}  // namespace

// ---------------------------------------------------------------------------
// Static plan for Cholesky: every front size is known after analysis, so the
// arena, every task list and the launch sequence are fixed here.

void FKeep::plan_cholesky() {
  const SymbolicTree& st = ak->st;
  const int ns = st.nnodes;
  const bool f32 = precision == 1;
  const int TM = f32 ? Tiles<float>::TM : Tiles<double>::TM;
  const int NB = f32 ? Tiles<float>::NB : Tiles<double>::NB;
  const int RT = f32 ? Tiles<float>::RT : Tiles<double>::RT;
  const Schedule& sched = Schedule::current();
  const int SMALL_M = sched.small_rows(f32 ? Tiles<float>::SMALL_M : Tiles<double>::SMALL_M);
  const int TC_ROWS = sched.tc_rows();

  order.resize(ns);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return st.level[a] < st.level[b]; });
  levels.assign(st.nlevels, Level());
  {
    std::vector<int> cnt(st.nlevels + 1, 0);
    for (int s = 0; s < ns; ++s) cnt[st.level[s] + 1]++;
    for (int l = 0; l < st.nlevels; ++l) {
      cnt[l + 1] += cnt[l];
      levels[l].f0 = cnt[l];
      levels[l].f1 = cnt[l + 1];
    }
  }
  // front blocks: one after another when they all fit in half of the device
  // memory; otherwise placed level by level with the contribution blocks a
  // level assembled given back before the next level is placed (the schedule
  // runs the levels in order on one stream, so each level's assembly, which
  // writes every entry of its fronts' lower triangles, comes after the
  // previous level read those blocks)
  off.assign(ns, 0);
  ld.assign(ns, 0);
  int64_t blocks = 0;
  for (int s = 0; s < ns; ++s)
    blocks += ArenaAlloc::round64((int64_t)round_up(std::max(st.nrow[s], 1), 4) * st.nrow[s]);
  size_t freeb = 0, totb = 0;
  SG_CUDA(cudaMemGetInfo(&freeb, &totb));
  const int fmem = sched.front_memory;
  reuse_blocks = fmem > 0 || (fmem == 0 && (double)blocks * (f32 ? sizeof(float) : sizeof(double)) >
                                               0.5 * (double)totb);
  {
    ArenaAlloc al;
    std::vector<int> pend;
    for (const Level& L : levels) {
      for (int c : pend) {
        int64_t a, b;
        cb_span(off[c], ld[c], st.nrow[c], st.ncol[c], &a, &b);
        al.release(a, b);
      }
      pend.clear();
      for (int k = L.f0; k < L.f1; ++k) {
        const int s = order[k], m = st.nrow[s];
        ld[s] = round_up(std::max(m, 1), 4);
        off[s] = al.alloc((int64_t)ld[s] * m);
        if (reuse_blocks)
          for (int c : st.children[s]) pend.push_back(c);
      }
    }
    arena_elems = std::max<int64_t>(al.high_water(), 1);
  }
  // zeroing (or one-pass assembly) tasks: each front's lower triangle in
  // column ranges of about 64K entries, level by level (zlv[l] = first task
  // of level l); colbase[k] = first column of level-ordered front k in the
  // per-column tables of the one-pass assembly
  std::vector<ZeroTask> zt;
  std::vector<AsmTask> at;
  std::vector<int64_t> zlv(levels.size() + 1, 0), ilv(levels.size() + 1, 0);
  std::vector<int64_t> colbase(ns + 1, 0);
  for (int k = 0; k < ns; ++k) colbase[k + 1] = colbase[k] + st.nrow[order[k]];
  for (size_t l = 0; l < levels.size(); ++l) {
    zlv[l] = (int64_t)zt.size();
    for (int k = levels[l].f0; k < levels[l].f1; ++k) {
      const int s = order[k], m = st.nrow[s];
      int j0 = 0;
      while (j0 < m) {
        int64_t acc = 0;
        int j1 = j0;
        while (j1 < m && acc < 65536) acc += m - j1++;
        zt.push_back({off[s], ld[s], m, j0, j1});
        at.push_back({off[s], ld[s], m, j0, j1, (int)colbase[k], 0});
        j0 = j1;
      }
    }
  }
  zlv[levels.size()] = (int64_t)zt.size();
  nzero = (int)zt.size();

  // A -> arena map, level by level (ilv[l] = first entry of level l)
  std::vector<int64_t> asrc, adst;
  asrc.reserve(st.nlist.size() / 2);
  adst.reserve(st.nlist.size() / 2);
  init_atomic = false;
  for (size_t l = 0; l < levels.size(); ++l) {
    ilv[l] = (int64_t)asrc.size();
    for (int kk = levels[l].f0; kk < levels[l].f1; ++kk) {
      const int s = order[kk];
      int nrow = st.nrow[s];
      int64_t prev = -1;
      for (int64_t k = st.nptr[s] - 1; k < st.nptr[s + 1] - 1; ++k) {
        int64_t src = st.nlist[2 * k] - 1, dest = st.nlist[2 * k + 1] - 1;
        int64_t c = dest / nrow, r = dest % nrow;
        asrc.push_back(src);
        adst.push_back(off[s] + c * ld[s] + r);
        if (dest == prev) init_atomic = true;
        prev = dest;
      }
    }
  }
  ninit = (int64_t)asrc.size();
  ilv[levels.size()] = ninit;

  // One-pass assembly (k_assemble) when every column's original entries
  // have distinct rows in the lower triangle, every child's rows land in
  // increasing parent rows and no front has more than 32 children with a
  // contribution block; otherwise zeroing + k_init_a + extend-add.
  std::vector<int> acp, arow, gptr;
  std::vector<int64_t> asrc_c;
  one_pass = !init_atomic && colbase[ns] < INT_MAX && ninit < INT_MAX;
  if (one_pass) {
    std::vector<int> mark(st.n, -1);
    for (int s = 0; s < ns && one_pass; ++s) {
      for (int64_t q = st.rptr[s] - 1; q < st.rptr[s + 1] - 1; ++q)
        mark[st.rlist[q] - 1] = (int)(q - (st.rptr[s] - 1));
      int nch = 0;
      for (int c : st.children[s]) {
        const int mc = st.nrow[c] - st.ncol[c];
        if (mc <= 0) continue;
        ++nch;
        const int64_t b = st.rptr[c] - 1 + st.ncol[c];
        for (int i = 1; i < mc && one_pass; ++i)
          if (mark[st.rlist[b + i] - 1] <= mark[st.rlist[b + i - 1] - 1]) one_pass = false;
      }
      if (nch > 32) one_pass = false;
    }
  }
  if (one_pass) {
    acp.assign(colbase[ns] + 1, 0);
    arow.resize(ninit);
    asrc_c.resize(ninit);
    std::vector<std::pair<int64_t, int64_t>> ent;  // (front entry c * nrow + r, source)
    for (int k = 0; k < ns && one_pass; ++k) {
      const int s = order[k], nrow = st.nrow[s];
      ent.clear();
      for (int64_t q = st.nptr[s] - 1; q < st.nptr[s + 1] - 1; ++q)
        ent.push_back({st.nlist[2 * q + 1] - 1, st.nlist[2 * q] - 1});
      std::stable_sort(ent.begin(), ent.end(),
                       [](const auto& x, const auto& y) { return x.first < y.first; });
      int64_t e = acp[colbase[k]];
      int jn = 0;  // next column whose start is unset
      for (size_t q = 0; q < ent.size(); ++q) {
        const int c = (int)(ent[q].first / nrow), r = (int)(ent[q].first % nrow);
        if (r < c || (q > 0 && ent[q].first == ent[q - 1].first)) {
          one_pass = false;
          break;
        }
        while (jn <= c) acp[colbase[k] + jn++] = (int)e;
        arow[e] = r;
        asrc_c[e] = ent[q].second;
        ++e;
      }
      while (jn <= nrow) acp[colbase[k] + jn++] = (int)e;
    }
  }
  if (one_pass) gptr.assign(colbase[ns] + 1, 0);

  // rlist (0-based) and solve descriptors in level order, small fronts first
  std::vector<int> rl0(st.rlist.size());
  for (size_t k = 0; k < st.rlist.size(); ++k) rl0[k] = st.rlist[k] - 1;
  hfr.resize(ns);
  hscr.resize(ns);
  for (int k = 0; k < ns; ++k) {
    int s = order[k];
    hfr[k] = FrontDesc{off[s], ld[s], st.nrow[s], st.ncol[s], (int)(st.rptr[s] - 1), 0};
  }
  {
    std::vector<int> pm = SolvePlan::small_first(hfr, levels);
    std::vector<FrontDesc> t(ns);
    for (int k = 0; k < ns; ++k) t[k] = hfr[pm[k]];
    hfr.swap(t);
  }
  scratch_rows = 0;
  for (auto& L : levels) {
    int64_t acc = 0;
    for (int k = L.f0; k < L.f1; ++k) {
      hscr[k] = acc;
      acc += hfr[k].m;
    }
    scratch_rows = std::max(scratch_rows, acc);
  }

  // per-level launches
  std::vector<ChildDesc> cds;
  std::vector<EaItem> items;
  std::vector<int> eagrp;  // first item of each extend-add group (grouped levels)
  std::vector<int> maps;
  std::vector<SmallTask> smalls;
  std::vector<PanelTask> panels, diags;
  std::vector<UpdTask> upds;
  std::vector<TcSplit> tcs;
  std::vector<TcTask> tct;
  std::vector<double> tc_flops;
  std::vector<std::pair<size_t, double>> tcop_flops;  // (op index, flops) of grouped updates
  std::vector<BlkTask> blkd, blkp;
  tclev.clear();
  blkinv_count = 0;
  const int PW = (f32 && use_tc) ? sched.panel_cols() : 0;
  blk_pw = PW;
  std::vector<int> pos(st.n, -1);
  ops.clear();
  op_level.clear();
  for (auto& L : levels) {
    // one-pass assembly of the level's fronts; otherwise the front blocks
    // <- 0, then the original entries (every level's at once before the
    // first when no block is reused), then the extend-add below
    const size_t l = &L - levels.data();
    const size_t l1 = reuse_blocks ? l + 1 : levels.size();
    if (one_pass) {
      if (zlv[l + 1] > zlv[l]) ops.push_back({Op::ASM, zlv[l], zlv[l + 1], 0});
    } else if (reuse_blocks || l == 0) {
      if (zlv[l1] > zlv[l]) ops.push_back({Op::MEMSET, zlv[l], zlv[l1], 0});
      if (ilv[l1] > ilv[l]) ops.push_back({Op::INIT, ilv[l], ilv[l1], 0});
    }
    // extend-add of children into this level's fronts, in child order and
    // without atomics (the factors are bitwise reproducible): one warp per
    // parent column adds the children's columns that land there one after
    // another (one launch per level); should a child's row map not keep row
    // order, one launch per child rank (the r-th child of every front)
    std::vector<std::vector<EaItem>> by_rank;
    struct Dest {
      int p, pc, rank;
      EaItem it;
    };
    std::vector<Dest> dests;
    bool ordered = true;
    for (int k = L.f0; k < L.f1; ++k) {
      int p = order[k];
      for (int64_t q = st.rptr[p] - 1; q < st.rptr[p + 1] - 1; ++q)
        pos[st.rlist[q] - 1] = (int)(q - (st.rptr[p] - 1));
      int rank = 0;
      for (int c : st.children[p]) {
        int mc = st.nrow[c] - st.ncol[c];
        if (mc <= 0) continue;
        ChildDesc cd;
        cd.cb_off = off[c] + (int64_t)st.ncol[c] * ld[c] + st.ncol[c];
        cd.p_off = off[p];
        cd.ld_c = ld[c];
        cd.ld_p = ld[p];
        cd.mc = mc;
        cd.map_off = (int)maps.size();
        for (int i = 0; i < mc; ++i) maps.push_back(pos[st.rlist[st.rptr[c] - 1 + st.ncol[c] + i] - 1]);
        int ci = (int)cds.size();
        cds.push_back(cd);
        if ((int)by_rank.size() <= rank) by_rank.resize(rank + 1);
        for (int j = 0; j < mc; ++j) {
          by_rank[rank].push_back({ci, j});
          dests.push_back({k, maps[cd.map_off + j], rank, {ci, j}});
          if (j > 0 && maps[cd.map_off + j] <= maps[cd.map_off + j - 1]) ordered = false;
        }
        ++rank;
      }
    }
    if (one_pass) {
      // the level's items grouped by parent column in child order, and each
      // column's item range (the assembly op above reads them)
      std::stable_sort(dests.begin(), dests.end(), [](const Dest& x, const Dest& y) {
        return x.p != y.p ? x.p < y.p : (x.pc != y.pc ? x.pc < y.pc : x.rank < y.rank);
      });
      size_t q = 0;
      for (int k = L.f0; k < L.f1; ++k) {
        const int m = st.nrow[order[k]];
        for (int j = 0; j < m; ++j) {
          gptr[colbase[k] + j] = (int)items.size();
          while (q < dests.size() && dests[q].p == k && dests[q].pc == j)
            items.push_back(dests[q++].it);
        }
      }
      if (q != dests.size() || !ordered)
        throw std::runtime_error("one-pass assembly: child rows out of order");
    } else if (ordered && !dests.empty()) {
      std::stable_sort(dests.begin(), dests.end(), [](const Dest& x, const Dest& y) {
        return x.p != y.p ? x.p < y.p : (x.pc != y.pc ? x.pc < y.pc : x.rank < y.rank);
      });
      const int64_t g0 = (int64_t)eagrp.size();
      for (size_t q = 0; q < dests.size(); ++q) {
        if (q == 0 || dests[q].p != dests[q - 1].p || dests[q].pc != dests[q - 1].pc)
          eagrp.push_back((int)items.size());
        items.push_back(dests[q].it);
      }
      ops.push_back({Op::EAG, g0, (int64_t)eagrp.size(), 0});
    } else {
      for (const auto& rk : by_rank) {
        const int64_t i0 = (int64_t)items.size();
        items.insert(items.end(), rk.begin(), rk.end());
        ops.push_back({Op::EA, i0, (int64_t)items.size(), 0});
      }
    }
    // small fronts: one CTA each
    int64_t s0 = (int64_t)smalls.size();
    int maxm = 0;
    std::vector<int> large;
    for (int k = L.f0; k < L.f1; ++k) {
      int s = order[k];
      if (st.nrow[s] <= SMALL_M) {
        smalls.push_back({off[s], ld[s], st.nrow[s], st.ncol[s], 0});
        maxm = std::max(maxm, st.nrow[s]);
      } else {
        large.push_back(s);
      }
    }
    if ((int64_t)smalls.size() > s0) ops.push_back({Op::SMALL, s0, (int64_t)smalls.size(), maxm});
    // contribution blocks updated on the tensor cores (FP32, 3xBF16, blocks
    // of at least TC_ROWS rows): their rows are stacked in the operand
    // planes (pitch: n rounded up to 64, the most of the level), row cbb[s]
    // for front row n; the blocked path's panel kernel writes them
    std::vector<int> tcf;
    std::vector<int> cbb(ns, -1);
    int cb_pitch = 0;
    int64_t cb_rows = 0, cb_mx = 0;
    for (int s : large) {
      const int m = st.nrow[s], n = st.ncol[s];
      if (m > n && f32 && use_tc && TC_ROWS > 0 && m - n >= TC_ROWS) {
        tcf.push_back(s);
        cbb[s] = (int)cb_rows;
        cb_rows += m - n;
        cb_mx = std::max<int64_t>(cb_mx, m - n);
        cb_pitch = std::max(cb_pitch, (n + TC_KCHUNK - 1) / TC_KCHUNK * TC_KCHUNK);
      }
    }
    // large fronts: panel steps over the fully-summed columns, batched
    int maxsteps = 0;
    if (PW > 0) {
      // blocked path: outer panels of PW columns in groups of G.  After
      // each panel but the group's last, the group's remaining columns get
      // that panel's update on the tensor cores (K = PW); after the group
      // the trailing fully-summed columns get the whole group's (K = G PW),
      // which reads and writes the trailing columns once per group.
      const int G = sched.panel_group();
      const int GW = G * PW;
      int maxn = 0;
      for (int s : large) maxn = std::max(maxn, st.ncol[s]);
      for (int g0 = 0; g0 < maxn; g0 += GW) {
        // rows [g0 + PW, m) of fronts with fully-summed columns past the
        // group's first panel are stacked (transposed, 3xBF16 split, K
        // columns [g PW, (g + 1) PW) written by the group's panel g)
        const int q = g0 + PW;
        std::vector<int> base(ns, -1);
        int64_t rows = 0, mxr = 0;
        for (int s : large)
          if (q < st.ncol[s]) {
            base[s] = (int)rows;
            mxr = std::max<int64_t>(mxr, st.nrow[s] - q);
            rows += st.nrow[s] - q;
          }
        const int lvl = rows > 0 ? (int)tclev.size() : -1;
        if (rows > 0) {
          tclev.push_back({GW, rows, mxr});
          tc_flops.push_back(0.0);  // per-op figures in tcop_flops
        }
        // update of columns [c, ce) x rows [c, m) of every front with
        // c < min(ce, n), by K columns [kc0, kc0 + nk) chunks of the group
        auto tc_update = [&](int coff, int cend_off, int kc0, int nk) {
          double fl = 0.0;
          const int64_t tk0 = (int64_t)tct.size();
          for (int s : large) {
            if (base[s] < 0) continue;
            const int m = st.nrow[s], n = st.ncol[s];
            const int c = g0 + coff, ce = std::min(n, cend_off < 0 ? n : g0 + cend_off);
            if (c >= ce) continue;
            for (int col0 = c; col0 < ce; col0 += 128)
              for (int row0 = col0; row0 < m; row0 += 128)
                tct.push_back({off[s], ld[s], row0, col0, m, ce, base[s] + row0 - q,
                               base[s] + col0 - q, nk, kc0});
            // lower-triangle entries of rows [c, m) x cols [c, ce), times 2K
            const double cnt = (double)(ce - c) * m - (0.5 * ce * (ce - 1.0) - 0.5 * c * (c - 1.0));
            fl += 2.0 * nk * TC_KCHUNK * cnt;
          }
          if ((int64_t)tct.size() > tk0) {
            tcop_flops.push_back({ops.size(), fl});
            ops.push_back({Op::TCUPD, tk0, (int64_t)tct.size(), lvl});
          }
        };
        for (int g = 0; g < G; ++g) {
          const int k0 = g0 + g * PW;
          if (k0 >= maxn) break;
          // the panel's diagonal block (one CTA per front), then the rows
          // below it (one CTA per 64 rows)
          const int64_t d0 = (int64_t)blkd.size(), p0 = (int64_t)blkp.size();
          for (int s : large) {
            const int m = st.nrow[s], n = st.ncol[s];
            if (k0 >= n) continue;
            const int pend = std::min(k0 + PW, n);
            const int xi = (int)((int64_t)blkd.size() - d0);
            // stacked row of row pend: only when a later update of this
            // group reads the panel (columns remain past it)
            const int pb = (pend < n) ? base[s] + (pend - q) : -1;
            blkd.push_back({off[s], ld[s], m, k0, pend - k0, pend, 0, xi, -1, n, -1, 0});
            for (int r0 = pend; r0 < m; r0 += 64)
              blkp.push_back({off[s], ld[s], m, k0, pend - k0, pend, r0, xi, pb, n,
                              r0 + 64 > n ? cbb[s] : -1, cb_pitch});
          }
          if ((int64_t)blkd.size() > d0) {
            ops.push_back({Op::BDIAG, d0, (int64_t)blkd.size(), 0});
            blkinv_count = std::max(blkinv_count, (int64_t)blkd.size() - d0);
          }
          if ((int64_t)blkp.size() > p0) ops.push_back({Op::BPANEL, p0, (int64_t)blkp.size(), GW});
          if (lvl < 0) continue;
          // the group's next panels, by this one
          if (g + 1 < G) tc_update((g + 1) * PW, GW, g * (PW / TC_KCHUNK), PW / TC_KCHUNK);
        }
        // the trailing fully-summed columns, by the whole group
        if (lvl >= 0) tc_update(GW, -1, 0, GW / TC_KCHUNK);
      }
    } else {
      for (int s : large) maxsteps = std::max(maxsteps, (st.ncol[s] + NB - 1) / NB);
    }
    for (int step = 0; step < maxsteps; ++step) {
      int64_t p0 = (int64_t)panels.size(), u0 = (int64_t)upds.size();
      int64_t d0 = (int64_t)diags.size();
      for (int s : large) {
        int m = st.nrow[s], n = st.ncol[s];
        int k0 = step * NB;
        if (k0 >= n) continue;
        int w = std::min(NB, n - k0);
        diags.push_back({off[s], ld[s], k0, w, k0, k0 + w, 0});
        for (int r0 = k0 + w; r0 < m; r0 += RT)
          panels.push_back({off[s], ld[s], k0, w, r0, std::min(r0 + RT, m), 0});
        int o = k0 + w;
        if (o < n) {
          for (int cj = 0; o + cj * TM < n; ++cj)
            for (int ri = cj; o + ri * TM < m; ++ri)
              upds.push_back({off[s], off[s], off[s], ld[s], ld[s], ld[s], o + ri * TM,
                              o + cj * TM, m, n, k0, k0 + w, 0});
        }
      }
      if ((int64_t)diags.size() > d0) ops.push_back({Op::DIAG, d0, (int64_t)diags.size(), 0});
      if ((int64_t)panels.size() > p0) ops.push_back({Op::PANEL, p0, (int64_t)panels.size(), 0});
      if ((int64_t)upds.size() > u0) ops.push_back({Op::UPD, u0, (int64_t)upds.size(), 0});
    }
    // contribution blocks: one Schur-complement update with K = n, on the
    // tensor cores (FP32, 3xBF16) for blocks of at least 64 rows
    int64_t u0 = (int64_t)upds.size();
    for (int s : large) {
      int m = st.nrow[s], n = st.ncol[s];
      if (m <= n || cbb[s] >= 0) continue;
      for (int cj = 0; n + cj * TM < m; ++cj)
        for (int ri = cj; n + ri * TM < m; ++ri)
          upds.push_back({off[s], off[s], off[s], ld[s], ld[s], ld[s], n + ri * TM,
                          n + cj * TM, m, m, 0, n, 0});
    }
    if ((int64_t)upds.size() > u0) ops.push_back({Op::UPD, u0, (int64_t)upds.size(), 0});
    if (!tcf.empty()) {
      const int pitch = cb_pitch;
      int64_t rows = 0, mx = cb_mx;
      int64_t sp0 = (int64_t)tcs.size(), tk0 = (int64_t)tct.size();
      for (int s : tcf) {
        int m = st.nrow[s], n = st.ncol[s];
        // without the blocked path a transposed split copy makes the operands
        if (PW == 0) tcs.push_back({off[s], ld[s], m, n, n, (int)rows, 0});
        for (int cj = 0; cj * 128 < m - n; ++cj)
          for (int ri = cj; ri * 128 < m - n; ++ri)
            tct.push_back({off[s], ld[s], n + ri * 128, n + cj * 128, m, m,
                           (int)rows + ri * 128, (int)rows + cj * 128,
                           (n + TC_KCHUNK - 1) / TC_KCHUNK});
        rows += m - n;
      }
      int lvl = (int)tclev.size();
      tclev.push_back({pitch, rows, mx, PW > 0});
      double fl = 0.0;  // lower triangle (diagonal included) x 2K
      for (int s : tcf) {
        double mc = st.nrow[s] - st.ncol[s];
        fl += mc * (mc + 1.0) * st.ncol[s];
      }
      tc_flops.push_back(fl);
      if (PW == 0) ops.push_back({Op::SPLIT, sp0, (int64_t)tcs.size(), lvl});
      ops.push_back({Op::TCUPD, tk0, (int64_t)tct.size(), lvl});
    }
    op_level.resize(ops.size(), (int)(&L - levels.data()));
  }

  ops.push_back({Op::INV, 0, 0, 0});
  op_level.resize(ops.size(), -1);
  // algorithmic flops of update launches: lower-triangle entries x 2K
  op_flops.assign(ops.size(), 0.0);
  for (const auto& tf : tcop_flops) op_flops[tf.first] = tf.second;
  for (size_t q = 0; q < ops.size(); ++q) {
    if (ops[q].kind == Op::TCUPD) {
      if (op_flops[q] == 0.0) op_flops[q] = tc_flops[ops[q].aux];
      continue;
    }
    if (ops[q].kind != Op::UPD) continue;
    double f = 0.0;
    for (int64_t k = ops[q].a; k < ops[q].b; ++k) {
      const UpdTask& t = upds[k];
      int r1 = std::min(t.row0 + TM, t.rowEnd), c1 = std::min(t.col0 + TM, t.colEnd);
      double pairs = 0.0;
      for (int c = t.col0; c < c1; ++c) pairs += std::max(0, r1 - std::max(c, t.row0));
      f += 2.0 * pairs * (t.k1 - t.k0);
    }
    op_flops[q] = f;
  }
  cudaStream_t s = Runtime::get().stream;
  if (one_pass) {
    gptr[colbase[ns]] = (int)items.size();
    asmt.upload(at, s);
    asm_acp.upload(acp, s);
    asm_arow.upload(arow, s);
    asm_asrc.upload(asrc_c, s);
    asm_gptr.upload(gptr, s);
  } else {
    zerot.upload(zt, s);
    amap_src.upload(asrc, s);
    amap_dst.upload(adst, s);
  }
  cdesc.upload(cds, s);
  eaitems.upload(items, s);
  eamaps.upload(maps, s);
  eagrp.push_back((int)items.size());  // end of the last group
  eagroups.upload(eagrp, s);
  small.upload(smalls, s);
  panel.upload(panels, s);
  diagt.upload(diags, s);
  tcsplit.upload(tcs, s);
  tctask.upload(tct, s);
  blkdiag.upload(blkd, s);
  blkpanel.upload(blkp, s);
  upd.upload(upds, s);
  dfr.upload(hfr, s);
  dscr.upload(hscr, s);
  splan.dataflow = sched.solve_dataflow >= 0;
  splan.build_tasks(hfr, levels, precision == 1 ? 4 : 8, s);
  rlist0.upload(rl0, s);
  std::vector<int> p0(st.n);
  for (int i = 0; i < st.n; ++i) p0[i] = st.perm[i];
  perm0.upload(p0, s);
  maxfront = st.maxfront;
  num_factor = st.num_factor;
  num_flops = st.num_flops;
}

void FKeep::upload_static(cudaStream_t s) {
  AKeep& a = *ak;
  frow.upload(a.frow, s);
  fcol.upload(a.fcol, s);
  fidx.upload(a.fidx, s);
  srcptr.upload(a.clean.srcptr, s);
  src.upload(a.clean.src, s);
  cval.ensure(std::max<size_t>(1, a.clean.crow.size()) * sizeof(double));
  faval.ensure(std::max<size_t>(1, a.fcol.size()) * sizeof(double));
  status.ensure(sizeof(unsigned));
  anorm.ensure(sizeof(double));
  // (LDL^T sizes its arena at factor time, when it knows whether the
  // factor columns go to the compact store)
  if (!ldlt) arena.ensure((size_t)arena_elems * (precision == 1 ? sizeof(float) : sizeof(double)));
  if (posdef) {
    // the inverses are formed inside the captured factor graph: allocate now
    const size_t es = precision == 1 ? sizeof(float) : sizeof(double);
    splan.inv.ensure((size_t)std::max<int64_t>(splan.inv_elems, 1) * es);
    splan.inv2.ensure((size_t)std::max<int64_t>(splan.inv2_elems, 1) * es);
    splan.inv2t.ensure((size_t)std::max<int64_t>(splan.inv2_elems, 1) * es);
    if (splan.dataflow && splan.p_elems > 0) splan.pmat.ensure((size_t)splan.p_elems * sizeof(float));
  }
  tcerr.ensure(sizeof(unsigned));
  if (blkinv_count > 0) blkinv.ensure((size_t)blkinv_count * BLK_B * BLK_B * sizeof(float));
  if (!tclev.empty()) {
    int64_t cap = 0, cbcap = 0;
    for (auto& L : tclev) (L.cb ? cbcap : cap) = std::max(L.cb ? cbcap : cap, L.rows * L.pitch);
    // three BF16 planes of cap elements each (plane stride rounded to 64
    // elements keeps every plane 128-byte aligned)
    plane_stride = (std::max<int64_t>(cap, 1) + 63) / 64 * 64;
    tcplanes.ensure((size_t)3 * plane_stride * sizeof(uint16_t));
    cb_stride = (std::max<int64_t>(cbcap, 1) + 63) / 64 * 64;
    cbplanes.ensure((size_t)3 * cb_stride * sizeof(uint16_t));
    tmaps.resize(3 * tclev.size());
    for (size_t l = 0; l < tclev.size(); ++l)
      for (int q = 0; q < 3; ++q) {
        const uint16_t* pl = tclev[l].cb ? cbplanes.as<uint16_t>() + q * cb_stride
                                         : tcplanes.as<uint16_t>() + q * plane_stride;
        make_panel_map(&tmaps[3 * l + q], pl, tclev[l].rows, tclev[l].pitch);
      }
  }
}

template <typename T>
void FKeep::run_ops(cudaStream_t s) {
  T* A = arena.as<T>();
  unsigned* stp = status.as<unsigned>();
  for (const Op& op : ops) {
    int64_t cnt = op.b - op.a;
    switch (op.kind) {
      case Op::MEMSET:
        launch_zero_lower<T>(A, zerot.as<ZeroTask>() + op.a, (int)cnt, s);
        break;
      case Op::INIT:
        launch_init_a<T>(A, val.as<double>(), amap_src.as<int64_t>() + op.a,
                         amap_dst.as<int64_t>() + op.a, cnt, init_atomic, s);
        break;
      case Op::ASM:
        launch_assemble<T>(A, val.as<double>(), asmt.as<AsmTask>() + op.a, (int)cnt,
                           asm_acp.as<int>(), asm_arow.as<int>(), asm_asrc.as<int64_t>(),
                           asm_gptr.as<int>(), eaitems.as<EaItem>(), cdesc.as<ChildDesc>(),
                           eamaps.as<int>(), s);
        break;
      case Op::EA:
        launch_extend_add<T>(A, cdesc.as<ChildDesc>(), eaitems.as<EaItem>() + op.a,
                             eamaps.as<int>(), (int)cnt, s, false);
        break;
      case Op::EAG:
        launch_extend_add_grouped<T>(A, cdesc.as<ChildDesc>(), eaitems.as<EaItem>(),
                                     eagroups.as<int>() + op.a, eamaps.as<int>(), (int)cnt, s);
        break;
      case Op::SMALL:
        launch_small_chol<T>(A, small.as<SmallTask>() + op.a, (int)cnt, op.aux, stp, s);
        break;
      case Op::DIAG:
        launch_diag_chol<T>(A, diagt.as<PanelTask>() + op.a, (int)cnt, stp, s);
        break;
      case Op::PANEL:
        launch_panel_trsm<T>(A, panel.as<PanelTask>() + op.a, (int)cnt, s);
        break;
      case Op::UPD:
        launch_update<T>(A, A, upd.as<UpdTask>() + op.a, (int)cnt, s);
        break;
      case Op::INV:
        splan.compute_inverses<T>(A, dfr.as<FrontDesc>(), false, s);
        break;
      case Op::SPLIT:
        if constexpr (std::is_same<T, float>::value)
          launch_split_t(A, tcsplit.as<TcSplit>() + op.a, (int)cnt, tclev[op.aux].max_rows,
                         tcplanes.as<uint16_t>(), plane_stride, tclev[op.aux].pitch, s);
        break;
      case Op::BDIAG:
        if constexpr (std::is_same<T, float>::value)
          launch_blk_diag(A, blkdiag.as<BlkTask>() + op.a, (int)cnt, blkinv.as<float>(), stp, s);
        break;
      case Op::BPANEL:
        if constexpr (std::is_same<T, float>::value)
          launch_blk_panel(A, blkpanel.as<BlkTask>() + op.a, (int)cnt, blkinv.as<float>(),
                           tcplanes.as<uint16_t>(), plane_stride, blk_pw, op.aux,
                           cbplanes.as<uint16_t>(), cb_stride, s);
        break;
      case Op::TCUPD:
        if constexpr (std::is_same<T, float>::value)
          launch_update_tc(&tmaps[3 * op.aux], A, tctask.as<TcTask>() + op.a, (int)cnt,
                           tcerr.as<unsigned>(), s);
        break;
    }
  }
}

int FKeep::factorize(const double* val_dev, cudaStream_t s) {
  AKeep& a = *ak;
  const int64_t nclean = (int64_t)a.clean.crow.size();
  // values: clean (duplicates summed) then full CSR for residuals
  launch_gather_clean(val_dev, srcptr.as<int64_t>(), src.as<int64_t>(), nclean,
                      cval.as<double>(), s);
  launch_gather(cval.as<double>(), fidx.as<int64_t>(), (int64_t)a.fcol.size(),
                faval.as<double>(), s);
  SG_CUDA(cudaMemsetAsync(anorm.p, 0, sizeof(double), s));
  launch_rownorm_inf(frow.as<int64_t>(), faval.as<double>(), a.n, anorm.as<double>(), s);
  SG_CUDA(cudaMemsetAsync(status.p, 0, sizeof(unsigned), s));
  SG_CUDA(cudaMemsetAsync(tcerr.p, 0, sizeof(unsigned), s));
  // the factor schedule reads val through the fkeep-owned buffer so that the
  // captured graph stays valid across calls
  if (val_dev != val.as<double>()) {
    int64_t nz = nnz_orig();
    val.ensure(std::max<int64_t>(nz, 1) * sizeof(double));
    if (nz) SG_CUDA(cudaMemcpyAsync(val.p, val_dev, nz * sizeof(double),
                                    cudaMemcpyDeviceToDevice, s));
  }
  apply_scale(s);
  cudaEvent_t e0, e1;
  SG_CUDA(cudaEventCreate(&e0));
  SG_CUDA(cudaEventCreate(&e1));
  SG_CUDA(cudaEventRecord(e0, s));
  if (use_graph) {
    if (!graph) {
      cudaGraph_t g;
      SG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      if (precision == 1) run_ops<float>(s);
      else run_ops<double>(s);
      SG_CUDA(cudaStreamEndCapture(s, &g));
      SG_CUDA(cudaGraphInstantiate(&graph, g, 0));
      cudaGraphDestroy(g);
    }
    SG_CUDA(cudaGraphLaunch(graph, s));
  } else {
    if (precision == 1) run_ops<float>(s);
    else run_ops<double>(s);
  }
  SG_CUDA(cudaEventRecord(e1, s));
  launches = (long)ops.size();
  unsigned st = 0, tce = 0;
  SG_CUDA(cudaMemcpyAsync(&st, status.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaMemcpyAsync(&tce, tcerr.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaMemcpyAsync(&anorm_h, anorm.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  factor_ms = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  flag = 0;
  if (tce) throw CudaError("tensor-core update: a bounded wait timed out");
  if (posdef) {
    rank = (st & ST_NOT_POSDEF) ? 0 : ak->n;
    if (st & ST_NOT_POSDEF) flag = -6;
  }
  return flag;
}

int FKeep::profile(const double* val_dev, double* ms, long* nl, double* flops, cudaStream_t s,
                   double* level_ms) {
  for (int k = 0; k < 12; ++k) {
    ms[k] = 0.0;
    nl[k] = 0;
    flops[k] = 0.0;
  }
  if (!posdef) return -98;
  if (val_dev && val_dev != val.as<double>()) {
    int64_t nz = nnz_orig();
    SG_CUDA(cudaMemcpyAsync(val.p, val_dev, nz * sizeof(double), cudaMemcpyDeviceToDevice, s));
  }
  apply_scale(s);
  SG_CUDA(cudaMemsetAsync(status.p, 0, sizeof(unsigned), s));
  std::vector<cudaEvent_t> ev(ops.size() + 1);
  for (auto& e : ev) SG_CUDA(cudaEventCreate(&e));
  SG_CUDA(cudaEventRecord(ev[0], s));
  std::vector<Op> all = ops;
  for (size_t q = 0; q < all.size(); ++q) {
    ops = {all[q]};
    if (precision == 1) run_ops<float>(s);
    else run_ops<double>(s);
    SG_CUDA(cudaEventRecord(ev[q + 1], s));
  }
  ops = all;
  SG_CUDA(cudaStreamSynchronize(s));
  for (size_t q = 0; q < all.size(); ++q) {
    float t = 0.f;
    cudaEventElapsedTime(&t, ev[q], ev[q + 1]);
    // grouped extend-add and one-pass assembly both count as extend-add
    int k = (all[q].kind == Op::EAG || all[q].kind == Op::ASM) ? (int)Op::EA : (int)all[q].kind;
    ms[k] += t;
    nl[k] += 1;
    flops[k] += op_flops.empty() ? 0.0 : op_flops[q];
    if (level_ms && q < op_level.size() && op_level[q] >= 0) level_ms[op_level[q]] += t;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return 0;
}

// ---------------------------------------------------------------------------

std::vector<int> SolvePlan::small_first(const std::vector<FrontDesc>& hfr,
                                        const std::vector<Level>& levels) {
  std::vector<int> pm(hfr.size());
  std::iota(pm.begin(), pm.end(), 0);
  for (const Level& L : levels)
    std::stable_sort(pm.begin() + L.f0, pm.begin() + L.f1, [&](int a, int b) {
      return is_large(hfr[a]) < is_large(hfr[b]);
    });
  return pm;
}

void SolvePlan::build_tasks(const std::vector<FrontDesc>& hfr, const std::vector<Level>& levels,
                            int elem, cudaStream_t s) {
  const int LB = LSOLVE_BW;
  lv.clear();
  htasks.clear();
  hdf.clear();
  hdfo.assign(hfr.size(), make_int2(0, 0));
  httoff.assign(hfr.size(), 0);
  dfc_elems = 0;
  df_tt_elems = 0;
  // the dataflow sweeps need the FP32 products P_ib (FP64: per-step launches)
  if (elem != 4) dataflow = false;
  hpt.clear();
  p_elems = 0;
  // rows per dataflow diagonal task (DfRows in kernels_solve.cu)
  const int DFR = 16, NSUB = LSOLVE_BW2 / DFR;
  hinv.clear();
  hinv_off.assign(hfr.size(), 0);
  inv_elems = 0;
  hinv2.clear();
  hinv2_off.assign(hfr.size(), 0);
  inv2_elems = 0;
  max_large = 0;
  for (const Level& L : levels) {
    Lv v;
    v.f0 = L.f0;
    v.nfront = L.f1 - L.f0;
    v.nsmall = 0;
    while (v.nsmall < v.nfront && !is_large(hfr[L.f0 + v.nsmall])) v.nsmall++;
    for (int f = 0; f < v.nsmall; ++f) v.small_maxn = std::max(v.small_maxn, hfr[L.f0 + f].n);
    max_large = std::max(max_large, v.nfront);
    auto push = [&](std::vector<SOp>& ops, int kind, int64_t a) {
      int64_t b = (int64_t)htasks.size();
      if (b > a) ops.push_back({kind, a, b});
    };
    // contribution rows of every front of the level, one launch per
    // direction: forward after all pivot rows are solved, backward before
    // (tiles start on a row divisible by 4, for 16-byte copies of L; the
    // kernels skip the first tile's rows below n)
    auto rect = [&](std::vector<SOp>& ops, bool fwd) {
      int64_t a = (int64_t)htasks.size();
      const int cw = fwd ? RECT_FWD_COLS : RECT_BWD_COLS;
      const int rh = fwd ? 2 * RECT_FWD_T : RECT_BWD_ROWS;
      int wmax = 0;
      for (int f = 0; f < v.nfront; ++f) {
        const FrontDesc& d = hfr[L.f0 + f];
        if (d.m <= d.n) continue;
        for (int c0 = 0; c0 < d.n; c0 += cw) {
          const int bw = std::min(cw, d.n - c0);
          wmax = std::max(wmax, bw);
          for (int r0 = d.n & ~3; r0 < d.m; r0 += rh) htasks.push_back({f, c0, bw, r0, 0, 0});
        }
      }
      push(ops, fwd ? LS_RECT_FWD : LS_RECT_BWD, a);
      if (!ops.empty() && ops.back().kind == (fwd ? LS_RECT_FWD : LS_RECT_BWD))
        ops.back().aux = round_up(wmax, 16);
    };
    rect(v.bwd, false);
    if (v.nsmall > 0) {
      v.fwd.push_back({LS_SMALL_TRI, 0, 0});
      v.bwd.push_back({LS_SMALL_TRI, 0, 0});
    }
    if (v.nsmall < v.nfront) {
      int maxb = 0;
      for (int f = v.nsmall; f < v.nfront; ++f) {
        const FrontDesc& d = hfr[L.f0 + f];
        int nb = (d.n + LB - 1) / LB;
        maxb = std::max(maxb, nb);
        hinv_off[L.f0 + f] = inv_elems;
        for (int b = 0; b < nb; ++b)
          hinv.push_back({L.f0 + f, b * LB, std::min(LB, d.n - b * LB), 0, 0, 0});
        // inverses are stored per 256-column block (four 64-blocks each)
        const int nb2 = (d.n + LSOLVE_BW2 - 1) / LSOLVE_BW2;
        inv_elems += (int64_t)nb2 * (LSOLVE_BW2 / LB) * LB * LB;
        hinv2_off[L.f0 + f] = inv2_elems;
        for (int b = 0; b < nb2; ++b)
          hinv2.push_back({L.f0 + f, b * LSOLVE_BW2,
                           std::min(LSOLVE_BW2, d.n - b * LSOLVE_BW2), 0, 0, 0});
        inv2_elems += (int64_t)nb2 * LSOLVE_BW2 * LSOLVE_BW2;
      }
      auto rows = [&](std::vector<SOp>& ops, int kind) {
        int64_t a = (int64_t)htasks.size();
        for (int f = v.nsmall; f < v.nfront; ++f)
          for (int r0 = 0; r0 < hfr[L.f0 + f].n; r0 += 256) htasks.push_back({f, 0, 0, r0, 0, 0});
        push(ops, kind, a);
      };
      rows(v.fwd, LS_GATHER_FWD);
      const int LB2 = LSOLVE_BW2;
      int maxb2 = 0;
      for (int f = v.nsmall; f < v.nfront; ++f)
        maxb2 = std::max(maxb2, (hfr[L.f0 + f].n + LB2 - 1) / LB2);
      // block steps over the fully-summed rows (< n) below the block
      auto step = [&](std::vector<SOp>& ops, int kind, int b, bool diag) {
        int64_t a = (int64_t)htasks.size();
        for (int f = v.nsmall; f < v.nfront; ++f) {
          const FrontDesc& d = hfr[L.f0 + f];
          int c0 = b * LB2;
          if (c0 >= d.n) continue;
          int bw = std::min(LB2, d.n - c0), c1 = c0 + bw;
          if (diag) htasks.push_back({f, c0, bw, 0, 0, 0});
          else if (kind == LS_FWD_UPD2)
            for (int r0 = c1; r0 < d.n; r0 += LSOLVE_UPD_ROWS) htasks.push_back({f, c0, bw, r0, 0, 0});
          else  // reductions in column tiles of LSOLVE_TW (one accumulator row per column)
            for (int h0 = c0; h0 < c1; h0 += LSOLVE_TW)
              for (int r0 = c1; r0 < d.n; r0 += LSOLVE_RED_ROWS)
                htasks.push_back({f, h0, std::min(LSOLVE_TW, c1 - h0), r0, 0, 0});
        }
        push(ops, kind, a);
      };
      if (dataflow) {
        // counters of the level: [0] ticket, then per front: row tiles of 32
        // (forward: updates applied), per block: a sink (the tasks nothing
        // waits for count there), reductions added and diagonal tasks done
        // (backward)
        constexpr int RT = LSOLVE_UPD_ROWS, BR = 32;  // rows per update / reduction task
        v.dfc_base = dfc_elems;
        int cnt = 1;
        int64_t tto = 0;
        std::vector<int> o(v.nfront, 0), nrt(v.nfront, 0), nbk(v.nfront, 0);
        for (int f = v.nsmall; f < v.nfront; ++f) {
          const int n = hfr[L.f0 + f].n;
          nrt[f] = (n + RT - 1) / RT;
          nbk[f] = (n + LB2 - 1) / LB2;
          o[f] = cnt;
          hdfo[L.f0 + f] = make_int2(cnt, nrt[f] + 3 * nbk[f]);
          cnt += nrt[f] + 3 * nbk[f];
          httoff[L.f0 + f] = tto;
          tto += (int64_t)nbk[f] * LB2 * 32;
        }
        dfc_elems += cnt;
        v.dfc_count = cnt;
        df_tt_elems = std::max(df_tt_elems, tto);
        auto bw_of = [&](int f, int b) { return std::min(LB2, hfr[L.f0 + f].n - b * LB2); };
        auto ready = [&](int f, int b) { return o[f] + nrt[f] + b; };           // forward
        auto nred_ctr = [&](int f, int b) { return o[f] + nrt[f] + nbk[f] + b; };
        auto zdone = [&](int f, int b) { return o[f] + nrt[f] + 2 * nbk[f] + b; };
        auto nred_of = [&](int f, int j) {  // reductions into block j: 32-row pieces below it
          int c = 0;
          for (int jj = j + 1; jj < nbk[f]; ++jj) c += (bw_of(f, jj) + BR - 1) / BR;
          return c;
        };
        // P_ib for every block with rows below it (ld: rows rounded up to 4)
        std::vector<std::vector<std::pair<int64_t, int>>> pb(v.nfront);
        for (int f = v.nsmall; f < v.nfront; ++f) {
          const int n = hfr[L.f0 + f].n;
          for (int b = 0; b + 1 < nbk[f]; ++b) {
            const int c1 = (b + 1) * LB2, ldp = round_up(n - c1, 4);
            pb[f].push_back({p_elems, ldp});
            for (int r0 = c1; r0 < n; r0 += 64)
              hpt.push_back({L.f0 + f, b * LB2, c1, r0, ldp, 0, p_elems});
            p_elems += (int64_t)ldp * LB2;
          }
        }
        // forward: x_i -= P_ib x_b once x_b is final (the next block's rows
        // first: the chain); y_b = X_b x_b off the chain
        int64_t a = (int64_t)hdf.size();
        for (int b = 0; b < maxb2; ++b) {
          for (int pass = 0; pass < 2; ++pass)
            for (int f = v.nsmall; f < v.nfront; ++f) {
              if (b + 1 >= nbk[f]) continue;
              const int t0 = b * LB2 / RT, nt = LB2 / RT, tn = (b + 2) * LB2 / RT;
              const int lo = pass == 0 ? (b + 1) * LB2 / RT : tn, hi = pass == 0 ? tn : nrt[f];
              for (int rt = lo; rt < std::min(hi, nrt[f]); ++rt)
                hdf.push_back({DF_UPD_FWD, f, b * LB2, LB2, rt * RT, 0, o[f] + t0, b > 0 ? nt : 0,
                               b, o[f] + rt, b, o[f] + rt, pb[f][b].second, 0, pb[f][b].first});
            }
          for (int f = v.nsmall; f < v.nfront; ++f) {
            if (b >= nbk[f]) continue;
            const int t0 = b * LB2 / RT, nt = (bw_of(f, b) + RT - 1) / RT;
            for (int q = 0; q < NSUB; ++q)
              hdf.push_back({DF_DIAG_FWD, f, b * LB2, bw_of(f, b), 0, q, o[f] + t0, b > 0 ? nt : 0,
                             b, -1, 0, ready(f, 0), 0, 0, 0});
          }
        }
        v.fwd.push_back({LS_CHAIN_FWD, a, (int64_t)hdf.size()});
        rows(v.fwd, LS_SCATTER_FWD);
        rows(v.bwd, LS_GATHER_BWD);
        // backward: u_b = X_b^T x_b for every block; then from the last
        // block: z_j = u_j - t_j and t_b += P_jb^T z_j (the block before
        // first: the chain; its tasks store z_j); z_0 = u_0 - t_0
        a = (int64_t)hdf.size();
        for (int f = v.nsmall; f < v.nfront; ++f)
          for (int b = 0; b < nbk[f]; ++b)
            for (int q = 0; q < NSUB; ++q)
              hdf.push_back({DF_DIAG_BWD, f, b * LB2, bw_of(f, b), 0, q, 0, 0, 0, -1, 0,
                             zdone(f, b), 0, 0, 0});
        for (int j = maxb2 - 1; j >= 1; --j)
          for (int b = j - 1; b >= 0; --b)
            for (int f = v.nsmall; f < v.nfront; ++f) {
              if (j >= nbk[f]) continue;
              const int r1 = j * LB2 + bw_of(f, j);
              for (int r0 = j * LB2; r0 < r1; r0 += BR)
                hdf.push_back({DF_RED_BWD, f, b * LB2, LB2, r0, b == j - 1 ? 1 : 0,
                               nred_ctr(f, j), 1, nred_of(f, j), zdone(f, j), NSUB,
                               nred_ctr(f, b), pb[f][b].second, 0, pb[f][b].first});
            }
        for (int f = v.nsmall; f < v.nfront; ++f)
          for (int r0 = 0; r0 < bw_of(f, 0); r0 += BR)
            hdf.push_back({DF_FIN_BWD, f, 0, bw_of(f, 0), r0, 0, nred_ctr(f, 0), 1,
                           nred_of(f, 0), zdone(f, 0), NSUB, ready(f, 0), 0, 0, 0});
        v.bwd.push_back({LS_CHAIN_BWD, a, (int64_t)hdf.size()});
        rows(v.bwd, LS_SCATTER_BWD);
      } else {
        for (int b = 0; b < maxb2; ++b) {
          step(v.fwd, LS_FWD_DIAG2, b, true);
          step(v.fwd, LS_FWD_UPD2, b, false);
        }
        rows(v.fwd, LS_SCATTER_FWD);
        rows(v.bwd, LS_GATHER_BWD);
        for (int b = maxb2 - 1; b >= 0; --b) {
          step(v.bwd, LS_BWD_RED2, b, false);
          step(v.bwd, LS_BWD_DIAG2, b, true);
        }
        rows(v.bwd, LS_SCATTER_BWD);
      }
    }
    rect(v.fwd, true);
    lv.push_back(std::move(v));
  }
  tasks.upload(htasks, s);
  if (dataflow) {
    // Each sweep's list must be a topological order: run it in list order on
    // the host, every wait already met when its task comes up (then a CTA
    // only ever waits for tasks running CTAs took before it), every counter
    // inside the level's range.
    for (const Lv& v : lv)
      for (int dir = 0; dir < 2; ++dir)
        for (const SOp& op : dir ? v.bwd : v.fwd) {
          if (op.kind != LS_CHAIN_FWD && op.kind != LS_CHAIN_BWD) continue;
          const int64_t lim = v.dfc_count;
          std::vector<int> c((size_t)lim, 0);
          for (int64_t q = op.a; q < op.b; ++q) {
            const DfTask& t = hdf[q];
            auto in = [&](int i) { return i > 0 && i < lim; };
            bool ok = in(t.sig) && t.nw < 32 && (t.nw == 0 || (in(t.w0) && in(t.w0 + t.nw - 1))) &&
                      (t.w1 < 0 || in(t.w1));
            for (int i = 0; ok && i < t.nw; ++i) ok = c[t.w0 + i] >= t.need0;
            if (ok && t.w1 >= 0) ok = c[t.w1] >= t.need1;
            if (!ok) throw std::runtime_error("dataflow solve: task list out of order");
            c[t.sig]++;
          }
        }
    dftasks.upload(hdf, s);
    ptasks.upload(hpt, s);
    dfo.upload(hdfo, s);
    ttoff.upload(httoff, s);
    dfcnt.ensure((size_t)std::max<int64_t>(dfc_elems, 1) * sizeof(int));
    if (!dferr.p) {
      dferr.ensure(sizeof(unsigned));
      SG_CUDA(cudaMemsetAsync(dferr.p, 0, sizeof(unsigned), s));
    }
  }
  invt.upload(hinv, s);
  inv_off.upload(hinv_off, s);
  invt2.upload(hinv2, s);
  inv2_off.upload(hinv2_off, s);
}

template <typename T>
void SolvePlan::compute_inverses(const T* arena, const FrontDesc* dfr, bool unit, cudaStream_t s) {
  inv.ensure((size_t)std::max<int64_t>(inv_elems, 1) * sizeof(T));
  inv2.ensure((size_t)std::max<int64_t>(inv2_elems, 1) * sizeof(T));
  inv2t.ensure((size_t)std::max<int64_t>(inv2_elems, 1) * sizeof(T));
  launch_inv_diag<T>(arena, dfr, invt.as<LTask>(), (int)hinv.size(), inv.as<T>(),
                     inv_off.as<int64_t>(), unit, s);
  launch_inv_block<T>(arena, dfr, invt2.as<LTask>(), (int)hinv2.size(), inv.as<T>(),
                   inv_off.as<int64_t>(), inv2.as<T>(), inv2t.as<T>(), inv2_off.as<int64_t>(),
                   s);
  if constexpr (std::is_same<T, float>::value) {
    if (dataflow && !hpt.empty()) {
      pmat.ensure((size_t)p_elems * sizeof(float));
      launch_form_p(arena, dfr, ptasks.as<PTask>(), (int)hpt.size(), inv2t.as<float>(),
                    inv2_off.as<int64_t>(), pmat.as<float>(), s);
    }
  }
}
template void SolvePlan::compute_inverses<float>(const float*, const FrontDesc*, bool,
                                                 cudaStream_t);
template void SolvePlan::compute_inverses<double>(const double*, const FrontDesc*, bool,
                                                  cudaStream_t);

void SolvePlan::fetch_error(unsigned* h, cudaStream_t s) {
  *h = 0;
  if (!dataflow || !dferr.p) return;
  SG_CUDA(cudaMemcpyAsync(h, dferr.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaMemsetAsync(dferr.p, 0, sizeof(unsigned), s));
}

void SolvePlan::ensure_tt(size_t elem, int64_t scratch_elems, int n) {
  const void* before = tt.p;
  tt.ensure((size_t)std::max<int64_t>((int64_t)std::max(max_large, 1) * 2 * LSOLVE_BW2 * 32,
                                      df_tt_elems) * elem);
  // the backward steps leave the accumulators zero; a new buffer starts zero
  if (tt.p != before) SG_CUDA(cudaMemset(tt.p, 0, tt.bytes));
  ys.ensure((size_t)std::max<int64_t>(scratch_elems, 1) * elem);
  // contribution rows' share of the pivot rows, laid out like x (32
  // right-hand sides); each backward sweep's consumers clear what they read
  const void* tbefore = tacc.p;
  tacc.ensure((size_t)std::max(n, 1) * 32 * elem);
  if (tacc.p != tbefore) SG_CUDA(cudaMemset(tacc.p, 0, tacc.bytes));
}

template <typename T, typename ACC>
void SolvePlan::run(bool fwd, const T* arena, const FrontDesc* dfr, const int* rlist, ACC* x,
                    int n, int nrhs, ACC* scratch, const int64_t* dscr, bool unit,
                    cudaStream_t s) {
  auto level = [&](const Lv& v) {
    const FrontDesc* fr = dfr + v.f0;
    const int64_t* sc = dscr + v.f0;
    LsArgs<T, ACC> a{arena, fr, rlist, x, n, nrhs, scratch, ys.as<ACC>(), sc, inv.as<T>(),
                     inv_off.as<int64_t>() + v.f0, tt.as<ACC>(), inv2.as<T>(),
                     inv2_off.as<int64_t>() + v.f0, inv2t.as<T>(), tacc.as<ACC>(),
                     dataflow ? dfcnt.as<int>() + v.dfc_base : nullptr,
                     dataflow ? dfo.as<int2>() + v.f0 : nullptr,
                     dataflow ? ttoff.as<int64_t>() + v.f0 : nullptr,
                     dataflow ? static_cast<const T*>(pmat.p) : nullptr, dataflow ? 1 : 0};
    const std::vector<SOp>& ops = fwd ? v.fwd : v.bwd;
    for (size_t k = 0; k < ops.size(); ++k) {
      const SOp& op = ops[k];
      if (op.kind == LS_CHAIN_FWD || op.kind == LS_CHAIN_BWD) {
        if constexpr (std::is_same<T, float>::value && std::is_same<ACC, float>::value)
          launch_chain(op.kind == LS_CHAIN_BWD, dftasks.as<DfTask>() + op.a, (int)(op.b - op.a),
                       a, dferr.as<unsigned>(), s);
        if (prof) mark(2 + op.kind, s);
        continue;
      }
      if (op.kind == LS_SMALL_TRI) {
        launch_small_tri<T, ACC>(fwd, arena, fr, v.nsmall, rlist, x, tacc.as<ACC>(), n, nrhs,
                                 v.small_maxn, unit, s);
        if (prof) mark(fwd ? 0 : 1, s);
        continue;
      }
      launch_lsolve<T, ACC>(op.kind, tasks.as<LTask>() + op.a, (int)(op.b - op.a), a, op.aux, s);
      if (prof) mark(2 + op.kind, s);
    }
  };
  if (fwd)
    for (const Lv& v : lv) level(v);
  else
    for (int l = (int)lv.size() - 1; l >= 0; --l) level(lv[l]);
}

void SolvePlan::mark(int kind, cudaStream_t s) {
  cudaEvent_t e;
  SG_CUDA(cudaEventCreate(&e));
  SG_CUDA(cudaEventRecord(e, s));
  prof->push_back({kind, e});
}

int FKeep::profile_solve(int nrhs, double* ms, long* nl, cudaStream_t s) {
  for (int k = 0; k < 16; ++k) {
    ms[k] = 0.0;
    nl[k] = 0;
  }
  if (ldlt || nrhs < 1 || nrhs > 32) return -98;
  const int n = ak->n;
  const size_t es = precision == 1 ? sizeof(float) : sizeof(double);
  xp.ensure(std::max<size_t>((size_t)n * nrhs * es, 1));
  SG_CUDA(cudaMemsetAsync(xp.p, 0, (size_t)n * nrhs * es, s));
  scratch.ensure(std::max<int64_t>(scratch_rows * nrhs, 1) * es);
  splan.ensure_tt(es, scratch_rows * nrhs, n);
  std::vector<std::pair<int, cudaEvent_t>> ev;
  splan.prof = &ev;
  try {
    splan.mark(-1, s);
    for (int dir = 0; dir < 2; ++dir) {
      if (precision == 1)
        splan.run<float, float>(dir == 0, arena.as<float>(), dfr.as<FrontDesc>(),
                                rlist0.as<int>(), xp.as<float>(), n, nrhs, scratch.as<float>(),
                                dscr.as<int64_t>(), false, s);
      else
        splan.run<double, double>(dir == 0, arena.as<double>(), dfr.as<FrontDesc>(),
                                  rlist0.as<int>(), xp.as<double>(), n, nrhs,
                                  scratch.as<double>(), dscr.as<int64_t>(), false, s);
    }
    SG_CUDA(cudaStreamSynchronize(s));
  } catch (...) {
    splan.prof = nullptr;
    for (auto& e : ev) cudaEventDestroy(e.second);
    throw;
  }
  splan.prof = nullptr;
  for (size_t q = 1; q < ev.size(); ++q) {
    float t = 0.f;
    cudaEventElapsedTime(&t, ev[q - 1].second, ev[q].second);
    const int k = ev[q].first;
    if (k >= 0 && k < 16) {
      ms[k] += t;
      nl[k] += 1;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e.second);
  return 0;
}

template void SolvePlan::run<float, float>(bool, const float*, const FrontDesc*, const int*,
                                           float*, int, int, float*, const int64_t*, bool,
                                           cudaStream_t);
template void SolvePlan::run<double, double>(bool, const double*, const FrontDesc*, const int*,
                                             double*, int, int, double*, const int64_t*, bool,
                                             cudaStream_t);

template <typename T>
void FKeep::solve_pivot_order(int job, void* xpv, int nrhs, cudaStream_t s) {
  using ACC = T;
  ACC* xpd = static_cast<ACC*>(xpv);
  const int n = ak->n;
  const T* A = arena.as<T>();
  scratch.ensure(std::max<int64_t>(scratch_rows * std::min(nrhs, 32), 1) * sizeof(ACC));
  bool fwd = job == 0 || job == 1;
  bool bwd = job == 0 || job == 3 || job == 4;
  splan.ensure_tt(sizeof(ACC), scratch_rows * std::min(nrhs, 32), n);
  replay(job, nrhs, xpd, s, [&]() {
    for (int r0 = 0; r0 < nrhs; r0 += 32) {
      int nr = std::min(32, nrhs - r0);
      ACC* xr = xpd + (int64_t)r0 * n;
      if (fwd) splan.run<T, ACC>(true, A, dfr.as<FrontDesc>(), rlist0.as<int>(), xr, n, nr,
                                 scratch.as<ACC>(), dscr.as<int64_t>(), !posdef, s);
      if (bwd) splan.run<T, ACC>(false, A, dfr.as<FrontDesc>(), rlist0.as<int>(), xr, n, nr,
                                 scratch.as<ACC>(), dscr.as<int64_t>(), !posdef, s);
    }
  });
}

int FKeep::solve_raw(int job, int nrhs, double* x, int ldx, cudaStream_t s) {
  if (precision != 0) return -98;
  const int n = ak->n;
  xp.ensure((size_t)n * nrhs * sizeof(double));
  for (int r = 0; r < nrhs; ++r)
    SG_CUDA(cudaMemcpyAsync(xp.as<double>() + (size_t)r * n, x + (size_t)r * ldx,
                            n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  if (ldlt) ldlt_solve_pivot_order(*this, job, xp.as<double>(), nrhs, s);
  else solve_pivot_order<double>(job, xp.p, nrhs, s);
  for (int r = 0; r < nrhs; ++r)
    SG_CUDA(cudaMemcpyAsync(x + (size_t)r * ldx, xp.as<double>() + (size_t)r * n,
                            n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  unsigned dferr_h = 0;
  splan.fetch_error(&dferr_h, s);
  SG_CUDA(cudaStreamSynchronize(s));
  return dferr_h ? SYLVER_ERROR_CUDA_UNKNOWN : 0;
}

int FKeep::solve(int job, int nrhs, double* x, int ldx, cudaStream_t s) {
  const int n = ak->n;
  if (n == 0) return 0;
  const bool f32 = precision == 1;
  const size_t acc_sz = f32 ? sizeof(float) : sizeof(double);
  xp.ensure((size_t)n * nrhs * acc_sz);
  const int* perm = perm0.as<int>();
  last_ir_iters = 0;
  last_bwd_err = -1.0;
  ir_hist.clear();
  // S on the way in for jobs 0/1 and on the way out for jobs 0/3/4
  // (src/spldlt_factorize_mod.F90:945-955, :1040-1050)
  const double* sc = has_scale ? dscale.as<double>() : nullptr;
  auto one_solve = [&](const double* rhs, int ldr, double* out, int ldo, bool add, int jb) {
    const double* sin = (jb == 0 || jb == 1) ? sc : nullptr;
    const double* sout = (jb == 0 || jb == 3 || jb == 4) ? sc : nullptr;
    if (f32) {
      launch_permute_in<float>(rhs, ldr, xp.as<float>(), perm, sin, n, nrhs, s);
      if (ldlt) ldlt_solve_pivot_order(*this, jb, xp.as<float>(), nrhs, s);
      else solve_pivot_order<float>(jb, xp.p, nrhs, s);
      launch_permute_out_add<float>(xp.as<float>(), perm, sout, out, ldo, n, nrhs, add, s);
    } else {
      launch_permute_in<double>(rhs, ldr, xp.as<double>(), perm, sin, n, nrhs, s);
      if (ldlt) ldlt_solve_pivot_order(*this, jb, xp.as<double>(), nrhs, s);
      else solve_pivot_order<double>(jb, xp.p, nrhs, s);
      launch_permute_out_add<double>(xp.as<double>(), perm, sout, out, ldo, n, nrhs, add, s);
    }
  };
  const bool refine = job == 0 && (f32 || ir_max_iter > 0);
  unsigned dferr_h = 0;  // a dataflow sweep's bounded wait gave up: the result is wrong
  if (!refine) {
    one_solve(x, ldx, x, ldx, false, job);
    splan.fetch_error(&dferr_h, s);
    SG_CUDA(cudaStreamSynchronize(s));
    return dferr_h ? SYLVER_ERROR_CUDA_UNKNOWN : 0;
  }
  // iterative refinement: x0 = solve(b); repeat r = b - A x (FP64), check
  // the scaled backward error, x += solve(r)
  bcopy.ensure((size_t)n * nrhs * sizeof(double));
  resid.ensure((size_t)n * nrhs * sizeof(double));
  norms.ensure((size_t)3 * nrhs * sizeof(double));
  for (int r = 0; r < nrhs; ++r)
    SG_CUDA(cudaMemcpyAsync(bcopy.as<double>() + (size_t)r * n, x + (size_t)r * ldx,
                            n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  one_solve(bcopy.as<double>(), n, x, ldx, false, 0);
  const int maxit = std::max(ir_max_iter, 1);
  std::vector<double> hn(3 * nrhs);
  for (int it = 0;; ++it) {
    launch_residual(frow.as<int64_t>(), fcol.as<int>(), faval.as<double>(), n, x, ldx,
                    bcopy.as<double>(), n, resid.as<double>(), nrhs, s);
    SG_CUDA(cudaMemsetAsync(norms.p, 0, 3 * nrhs * sizeof(double), s));
    launch_maxnorms(resid.as<double>(), x, ldx, bcopy.as<double>(), n, n, nrhs,
                    norms.as<double>(), s);
    SG_CUDA(cudaMemcpyAsync(hn.data(), norms.p, 3 * nrhs * sizeof(double),
                            cudaMemcpyDeviceToHost, s));
    splan.fetch_error(&dferr_h, s);
    SG_CUDA(cudaStreamSynchronize(s));
    if (dferr_h) return SYLVER_ERROR_CUDA_UNKNOWN;
    double worst = 0.0;
    for (int r = 0; r < nrhs; ++r) {
      double den = anorm_h * hn[3 * r + 1] + hn[3 * r + 2];
      double be = den > 0 ? hn[3 * r] / den : 0.0;
      if (!(be == be)) be = INFINITY;
      worst = std::max(worst, be);
    }
    last_bwd_err = worst;
    ir_hist.push_back(worst);
    last_ir_iters = it;
    if (worst <= ir_tol) break;
    if (it >= maxit) return SYLVER_GB300_WARNING_IR_NOT_CONVERGED;
    one_solve(resid.as<double>(), n, x, ldx, true, 0);
  }
  return 0;
}

}  // namespace sylver_gb300
