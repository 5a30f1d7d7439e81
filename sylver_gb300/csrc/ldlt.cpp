// Host driver of the threshold-pivoted LDL^T factorization.
//
// Replaces the reference's indefinite numeric tree (src/NumericTree.hxx:54-181,
// :186-406), front allocation with delays (src/NumericFront.hxx:73-145),
// assembly of delayed columns (src/kernels/assemble.hxx:926-1093), the APP
// driver (src/factor_indef.hxx:1338-1474, :1484-1646), the failed-pivot TPP
// pass (src/factor_failed.hxx:29-157) and the inertia reduction
// (src/NumericTree.hxx:143-178).
//
// Fronts are processed level by level (height in the assembly tree).  Front
// sizes depend on how many columns the children delayed, so each level is
// planned on the host once its children are done: that is the one host
// synchronisation per level.  Inside a level everything runs on the device:
// a front with n fully-summed columns takes ceil(n / 32) block steps
// whatever fails (each step processes the next 32 columns not yet tried),
// so the launch sequence is known in advance; where a block starts, how many
// of its pivots pass and how many columns failed so far live in device state
// that the kernels read.  Per step: diagonal block -> rows below (solve +
// threshold test) -> commit (L, restore failed columns, L*D, D) -> trailing
// update -> move of the failed columns behind the unprocessed ones.  Then
// threshold partial pivoting on the failed columns, a relaxed pass at the
// roots, and the contribution-block update once the host knows how many
// columns each front eliminated.  Children's contributions are added in a
// fixed order (one launch per child rank), so the factors are deterministic.
#include "ldlt.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <type_traits>

#include "arena_alloc.hpp"
#include "ldlt_dev.hpp"
#include "tc.hpp"

namespace sylver_gb300 {

struct LdltState {
  // per front (original index)
  std::vector<int> m, n, nelim, ld, var_off;
  std::vector<int64_t> off, d_off;
  std::vector<std::vector<int>> var;  // host copy after factorization
  int64_t var_used = 0, d_used = 0;
  // front blocks in the arena: contribution blocks are given back once the
  // parent's level has assembled them (`pending`: the fronts whose blocks
  // the last level read)
  ArenaAlloc alloc;
  std::vector<int> pending;
  // arena high-water marks from the symbolic sizes: contribution blocks
  // given back (in place) or whole blocks given back with the factor
  // columns copied out; elements of factor columns (symbolic)
  int64_t hw_inplace = 0, hw_copyout = 0, fsym = 0;
  bool copyout = false;
  std::vector<int64_t> foff;  // copy-out: offset of each front's factor columns
  int64_t fused = 0;
  DevMem cspans;
  DevMem dvar, dall, blk, bdinv, lperm, state, mvvar;
  DevMem fr, fr2, cmap, cmap2, up, sc, sc2;  // per-level descriptors + scratch
  DevMem tcsplit, tctask, tcplanes;          // FP32 contribution blocks on the tensor cores
  DevMem ea_cd, ea_items, ea_maps, am_src, am_dst, zspans;
  // solve
  DevMem sfr, sscr, sdoff;
  std::vector<FrontDesc> hsfr;
  std::vector<int64_t> hsscr, hsdoff;
  int64_t scratch_rows = 0;
};

namespace {

inline int round_up(int v, int a) { return (v + a - 1) / a * a; }

// threshold of the relaxed pass at the roots (keeps only the small-pivot test)
constexpr double kRootU = 1e-300;
inline int64_t round_up64(int64_t v, int64_t a) { return (v + a - 1) / a * a; }

// grow a device buffer keeping its contents
void grow(DevMem& d, size_t bytes, cudaStream_t s) {
  if (bytes <= d.bytes && d.p) return;
  size_t nb = std::max(bytes, d.bytes + d.bytes / 2);
  void* np = nullptr;
  SG_CUDA(cudaMalloc(&np, nb));
  if (d.p && d.bytes) SG_CUDA(cudaMemcpyAsync(np, d.p, d.bytes, cudaMemcpyDeviceToDevice, s));
  SG_CUDA(cudaStreamSynchronize(s));
  d.release();
  d.p = np;
  d.bytes = nb;
}

template <typename V>
void put(DevMem& d, const std::vector<V>& v, cudaStream_t s) {
  d.ensure(std::max<size_t>(1, v.size()) * sizeof(V));
  if (!v.empty())
    SG_CUDA(cudaMemcpyAsync(d.p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice, s));
}

}  // namespace

void plan_ldlt(FKeep& fk) {
  // level order as for Cholesky; sizes are decided at factor time
  const SymbolicTree& st = fk.ak->st;
  const int ns = st.nnodes;
  fk.order.resize(ns);
  std::iota(fk.order.begin(), fk.order.end(), 0);
  std::stable_sort(fk.order.begin(), fk.order.end(),
                   [&](int a, int b) { return st.level[a] < st.level[b]; });
  fk.levels.assign(st.nlevels, Level());
  std::vector<int> cnt(st.nlevels + 1, 0);
  for (int s = 0; s < ns; ++s) cnt[st.level[s] + 1]++;
  for (int l = 0; l < st.nlevels; ++l) {
    cnt[l + 1] += cnt[l];
    fk.levels[l].f0 = cnt[l];
    fk.levels[l].f1 = cnt[l + 1];
  }
  fk.ldlt = std::make_shared<LdltState>();
  std::vector<int> p0(st.n);
  for (int i = 0; i < st.n; ++i) p0[i] = st.perm[i];
  fk.perm0.upload(p0, Runtime::get().stream);
  fk.num_flops = st.num_flops;
  // arena: the high-water mark of the front blocks with contribution blocks
  // given back after the parent's level (symbolic sizes, no delays), plus
  // headroom for delays; it grows when a level needs more.  The same with
  // whole blocks given back (factor columns copied out) for fronts that
  // would not fit that way.
  LdltState& L = *fk.ldlt;
  for (int whole = 0; whole < 2; ++whole) {
    ArenaAlloc sim;
    std::vector<int64_t> soff(ns, 0);
    std::vector<int> pend;
    for (const Level& lev : fk.levels) {
      for (int c : pend) {
        const int64_t ldc = round_up(std::max(st.nrow[c], 1), 4);
        int64_t a = soff[c], b = soff[c] + ArenaAlloc::round64(ldc * st.nrow[c]);
        if (!whole) cb_span(soff[c], ldc, st.nrow[c], st.ncol[c], &a, &b);
        sim.release(a, b);
      }
      pend.clear();
      for (int k = lev.f0; k < lev.f1; ++k) {
        const int s = fk.order[k];
        const int64_t lds = round_up(std::max(st.nrow[s], 1), 4);
        soff[s] = sim.alloc(lds * st.nrow[s]);
        for (int c : st.children[s]) pend.push_back(c);
        if (whole) L.fsym += ArenaAlloc::round64(lds * st.ncol[s]);
      }
    }
    (whole ? L.hw_copyout : L.hw_inplace) = sim.high_water();
  }
  fk.arena_elems = L.hw_inplace + L.hw_inplace / 8 + 1024;
}

namespace {

// CTA slices of one launch: for each front (index into the level's LdltFront
// array) `count` CTAs.
void add_slice(std::vector<CtaMap>& v, int f, int count) {
  count = std::max(count, 1);
  for (int c = 0; c < count; ++c) v.push_back({f, c, count, 0});
}

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

}  // namespace

template <typename T>
static int factorize_ldlt_t(FKeep& fk, cudaStream_t s) {
  const SymbolicTree& st = fk.ak->st;
  LdltState& L = *fk.ldlt;
  const int ns = st.nnodes;
  const int TM = Tiles<T>::TM;
  L.m.assign(ns, 0);
  L.n.assign(ns, 0);
  L.nelim.assign(ns, 0);
  L.ld.assign(ns, 0);
  L.var_off.assign(ns, 0);
  L.off.assign(ns, 0);
  L.d_off.assign(ns, 0);
  L.var.assign(ns, {});
  L.var_used = L.d_used = 0;
  L.alloc.reset();
  L.pending.clear();
  // fronts kept in place unless their blocks would take more than half of
  // the device memory that way; then the factor columns are copied out to a
  // compact store after each level and whole blocks are given back
  {
    size_t freeb = 0, totb = 0;
    SG_CUDA(cudaMemGetInfo(&freeb, &totb));
    const double avail = (double)freeb + (double)fk.arena.bytes + (double)fk.fstore.bytes;
    const int fsch = Schedule::current().front_memory;
    L.copyout = fsch > 0 ||
                (fsch == 0 && (double)(L.hw_inplace + L.hw_inplace / 8) * sizeof(T) > 0.5 * avail);
    fk.fcopy = L.copyout;
    if (L.copyout) {
      fk.arena_elems = L.hw_copyout + L.hw_copyout / 8 + 1024;
      const int64_t fe = L.fsym + L.fsym / 4 + 1024;
      if (fk.fstore.bytes < (size_t)fe * sizeof(T)) {
        fk.fstore.release();
        fk.fstore.ensure((size_t)fe * sizeof(T));
      }
      L.foff.assign(ns, 0);
      L.fused = 0;
    } else {
      fk.fstore.release();
      fk.arena_elems = std::max(fk.arena_elems, L.hw_inplace + L.hw_inplace / 8 + 1024);
    }
  }
  if (L.copyout && fk.arena.bytes > (size_t)fk.arena_elems * sizeof(T) * 2) fk.arena.release();
  fk.arena.ensure((size_t)fk.arena_elems * sizeof(T));
  unsigned* status = fk.status.as<unsigned>();
  SG_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned), s));
  SG_CUDA(cudaMemsetAsync(fk.tcerr.p, 0, sizeof(unsigned), s));
  long launches = 0;
  std::vector<int> pos(st.n, -1);
  const int tpp_cols = Schedule::current().ldlt_tpp_cols;
  fk.not_first_pass = fk.not_second_pass = 0;
  fk.num_delay = 0;

  for (const Level& lev : fk.levels) {
    std::vector<int> F(fk.order.begin() + lev.f0, fk.order.begin() + lev.f1);
    const int nslot = (int)F.size();
    // ---- sizes, variable lists, storage: the contribution blocks the last
    // level assembled are given back first (that level has completed: its
    // host synchronisation), then this level's fronts are placed
    for (int c : L.pending) {
      int64_t a = L.off[c], b = L.off[c] + round_up64((int64_t)L.ld[c] * L.m[c], 64);
      if (!L.copyout) cb_span(L.off[c], L.ld[c], L.m[c], L.nelim[c], &a, &b);
      L.alloc.release(a, b);
    }
    L.pending.clear();
    std::vector<ZeroSpan> zsp;
    std::vector<int> hvar_lvl;
    for (int s2 : F) {
      int sncol = st.ncol[s2], snrow = st.nrow[s2];
      int ndin = 0;
      for (int c : st.children[s2]) ndin += L.n[c] - L.nelim[c];
      L.n[s2] = sncol + ndin;
      L.m[s2] = snrow + ndin;
      L.ld[s2] = round_up(std::max(L.m[s2], 1), 4);
      const int64_t blk = round_up64((int64_t)L.ld[s2] * L.m[s2], 64);
      L.off[s2] = L.alloc.alloc(blk);
      for (int64_t z = 0; z < blk; z += (int64_t)1 << 20)
        zsp.push_back({L.off[s2] + z, std::min<int64_t>((int64_t)1 << 20, blk - z)});
      for (int c : st.children[s2]) L.pending.push_back(c);
      L.d_off[s2] = L.d_used;
      L.d_used += 2 * (int64_t)std::max(L.n[s2], 1);
      L.var_off[s2] = (int)L.var_used;
      L.var_used += L.m[s2];
      auto& v = L.var[s2];
      v.clear();
      const int* rl = &st.rlist[st.rptr[s2] - 1];
      for (int i = 0; i < sncol; ++i) v.push_back(rl[i] - 1);
      for (int c : st.children[s2])
        for (int jj = L.nelim[c]; jj < L.n[c]; ++jj) v.push_back(L.var[c][jj]);
      for (int i = sncol; i < snrow; ++i) v.push_back(rl[i] - 1);
      hvar_lvl.insert(hvar_lvl.end(), v.begin(), v.end());
      fk.maxfront = std::max(fk.maxfront, L.m[s2]);
    }
    if (L.alloc.top() > fk.arena_elems) {
      int64_t ne = std::max(L.alloc.top(), fk.arena_elems + fk.arena_elems / 4);
      grow(fk.arena, (size_t)ne * sizeof(T), s);
      fk.arena_elems = ne;
    }
    grow(L.dvar, (size_t)std::max<int64_t>(L.var_used, 1) * sizeof(int), s);
    grow(L.dall, (size_t)std::max<int64_t>(L.d_used, 1) * sizeof(double), s);
    T* A = fk.arena.as<T>();
    int* dvar = L.dvar.as<int>();
    if (!hvar_lvl.empty())
      SG_CUDA(cudaMemcpyAsync(dvar + L.var_off[F[0]], hvar_lvl.data(),
                              hvar_lvl.size() * sizeof(int), cudaMemcpyHostToDevice, s));
    put(L.zspans, zsp, s);
    launch_zero_spans<T>(A, L.zspans.as<ZeroSpan>(), (int)zsp.size(), s);
    SG_CUDA(cudaMemsetAsync(L.dall.as<double>() + L.d_off[F[0]], 0,
                            (size_t)(L.d_used - L.d_off[F[0]]) * sizeof(double), s));
    // ---- original entries (rows below the own columns shift by ndelay_in)
    {
      std::vector<int64_t> asrc, adst;
      bool atomic = false;
      for (int s2 : F) {
        int snrow = st.nrow[s2], sncol = st.ncol[s2], ndin = L.n[s2] - sncol;
        int64_t prev = -1;
        for (int64_t k = st.nptr[s2] - 1; k < st.nptr[s2 + 1] - 1; ++k) {
          int64_t src = st.nlist[2 * k] - 1, dest = st.nlist[2 * k + 1] - 1;
          int64_t c = dest / snrow, r = dest % snrow;
          if (r >= sncol) r += ndin;
          asrc.push_back(src);
          adst.push_back(L.off[s2] + c * L.ld[s2] + r);
          if (dest == prev) atomic = true;
          prev = dest;
        }
      }
      put(L.am_src, asrc, s);
      put(L.am_dst, adst, s);
      launch_init_a<T>(A, fk.val.as<double>(), L.am_src.as<int64_t>(), L.am_dst.as<int64_t>(),
                       (int64_t)asrc.size(), atomic, s);
      launches++;
    }
    // ---- children: delayed columns and contribution blocks, one launch per
    // child rank (the r-th child of every front), children in increasing
    // index order, so every parent entry sums its terms in a fixed order
    {
      int maxkids = 0;
      for (int p2 : F) maxkids = std::max(maxkids, (int)st.children[p2].size());
      std::vector<ChildDesc> cds;
      std::vector<EaItem> items;
      std::vector<int> maps;
      std::vector<int64_t> rank_item0(maxkids + 1, 0);
      std::vector<std::vector<int>> pmaps(F.size());
      for (size_t k = 0; k < F.size(); ++k) {
        int p2 = F[k];
        for (int i = 0; i < L.m[p2]; ++i) pos[L.var[p2][i]] = i;
        auto& pm = pmaps[k];
        for (int c : st.children[p2])
          for (int i = L.nelim[c]; i < L.m[c]; ++i) pm.push_back(pos[L.var[c][i]]);
      }
      for (int r = 0; r < maxkids; ++r) {
        rank_item0[r] = (int64_t)items.size();
        for (size_t k = 0; k < F.size(); ++k) {
          int p2 = F[k];
          const auto& kids = st.children[p2];
          if (r >= (int)kids.size()) continue;
          int moff = 0;
          for (int rr = 0; rr < r; ++rr) moff += L.m[kids[rr]] - L.nelim[kids[rr]];
          int c = kids[r];
          int mc = L.m[c] - L.nelim[c];
          if (mc <= 0) continue;
          ChildDesc cd;
          cd.cb_off = L.off[c] + (int64_t)L.nelim[c] * L.ld[c] + L.nelim[c];
          cd.p_off = L.off[p2];
          cd.ld_c = L.ld[c];
          cd.ld_p = L.ld[p2];
          cd.mc = mc;
          cd.map_off = (int)maps.size();
          maps.insert(maps.end(), pmaps[k].begin() + moff, pmaps[k].begin() + moff + mc);
          int ci = (int)cds.size();
          cds.push_back(cd);
          for (int jj = 0; jj < mc; ++jj) items.push_back({ci, jj});
        }
      }
      rank_item0[maxkids] = (int64_t)items.size();
      if (!items.empty()) {
        put(L.ea_cd, cds, s);
        put(L.ea_items, items, s);
        put(L.ea_maps, maps, s);
        for (int r = 0; r < maxkids; ++r) {
          int cnt = (int)(rank_item0[r + 1] - rank_item0[r]);
          if (cnt <= 0) continue;
          launch_extend_add<T>(A, L.ea_cd.as<ChildDesc>(),
                               L.ea_items.as<EaItem>() + rank_item0[r], L.ea_maps.as<int>(),
                               cnt, s, /*atomic=*/false);
          launches++;
        }
      }
    }
    // ---- level descriptors and scratch
    std::vector<LdltFront> fr(nslot);
    int64_t scr = 0, ivar = 0;
    int maxblk = 0;
    for (int q = 0; q < nslot; ++q) {
      int s2 = F[q];
      LdltFront& f = fr[q];
      f.off = L.off[s2];
      f.ld = L.ld[s2];
      f.m = L.m[s2];
      f.n = L.n[s2];
      f.fidx = q;
      f.var_off = L.var_off[s2];
      f.d_off = L.d_off[s2];
      f.nblk = (f.n == 0 || f.n <= tpp_cols) ? 0 : ceil_div(f.n, LDLT_BW);
      f.p = 0;
      f.pan_off = scr;
      scr += (int64_t)f.m * LDLT_BW;
      f.ldp_off = scr;
      scr += (int64_t)f.m * LDLT_BW;
      f.mv_off = scr;
      scr += f.nblk > 0 ? (int64_t)f.m * f.n : 0;
      scr = round_up64(scr, 32);
      f.mvvar_off = (int)ivar;
      ivar += f.n;
      maxblk = std::max(maxblk, f.nblk);
    }
    if (L.sc.bytes < (size_t)std::max<int64_t>(scr, 1) * sizeof(T))
      L.sc.ensure((size_t)std::max<int64_t>(scr, 1) * sizeof(T));
    L.mvvar.ensure((size_t)std::max<int64_t>(ivar, 1) * sizeof(int));
    put(L.fr, fr, s);
    // per-step CTA maps: diag, apply, commit, update, move
    std::vector<CtaMap> maps;
    struct StepMaps { int64_t o[5]; int n[5]; };
    std::vector<StepMaps> sm(maxblk);
    for (int k = 0; k < maxblk; ++k) {
      for (int kind = 0; kind < 5; ++kind) {
        sm[k].o[kind] = (int64_t)maps.size();
        for (int q = 0; q < nslot; ++q) {
          const LdltFront& f = fr[q];
          if (f.nblk <= k) continue;
          const int w = std::min(LDLT_BW, f.n - LDLT_BW * k);
          const int p0 = LDLT_BW * k;  // block start when nothing failed so far
          int cnt = 1;
          if (kind == 1) cnt = ceil_div(std::max(f.m - p0 - w, 1), LDLT_RT);
          if (kind == 2) cnt = ceil_div(f.m - p0, LDLT_RT);
          if (kind == 3) {
            const int o = std::min(p0 + w, f.n - 1);
            const int R = ceil_div(f.m - o, TM), C = ceil_div(f.n - o, TM);
            cnt = C * R - C * (C - 1) / 2;
          }
          if (kind == 4) cnt = ceil_div(f.n, 8);
          add_slice(maps, q, cnt);
        }
        sm[k].n[kind] = (int)((int64_t)maps.size() - sm[k].o[kind]);
      }
    }
    put(L.cmap, maps, s);
    // per-slot step buffers and state (p/nf ping-pong, p_final)
    L.blk.ensure((size_t)std::max(nslot, 1) * LDLT_BW * (LDLT_BW + 1) * sizeof(double));
    L.bdinv.ensure((size_t)std::max(nslot, 1) * 2 * LDLT_BW * sizeof(double));
    L.lperm.ensure((size_t)std::max(nslot, 1) * LDLT_BW * sizeof(int));
    L.state.ensure((size_t)std::max(nslot, 1) * 10 * sizeof(int));
    SG_CUDA(cudaMemsetAsync(L.state.p, 0, (size_t)std::max(nslot, 1) * 10 * sizeof(int), s));
    int* stt = L.state.as<int>();
    int* Pbuf[2] = {stt, stt + nslot};
    int* NFbuf[2] = {stt + 2 * nslot, stt + 3 * nslot};
    int* p_final = stt + 4 * nslot;
    int* ndiag = stt + 5 * nslot;
    int* npass_raw = stt + 6 * nslot;
    int* npass = stt + 7 * nslot;
    int* tpp1 = stt + 8 * nslot;
    int* tpp2 = stt + 9 * nslot;
    LdltStep stp{L.blk.as<double>(), L.bdinv.as<double>(), L.lperm.as<int>(), ndiag, npass_raw,
                 npass, nullptr, nullptr, nullptr, nullptr, p_final, dvar, L.mvvar.as<int>(),
                 L.dall.as<double>(), status, fk.u, fk.small_piv, fk.action ? 1 : 0, 0};
    const LdltFront* dfr = L.fr.as<LdltFront>();
    const CtaMap* dcm = L.cmap.as<CtaMap>();
    T* sc = L.sc.as<T>();
    // ---- a-posteriori block steps
    for (int k = 0; k < maxblk; ++k) {
      stp.k = k;
      stp.p_cur = Pbuf[k & 1];
      stp.nf_cur = NFbuf[k & 1];
      stp.p_next = Pbuf[(k + 1) & 1];
      stp.nf_next = NFbuf[(k + 1) & 1];
      launch_app_diag<T>(A, sc, dfr, dcm + sm[k].o[0], sm[k].n[0], stp, s);
      launch_app_apply<T>(A, sc, dfr, dcm + sm[k].o[1], sm[k].n[1], stp, s);
      launch_app_commit<T>(A, sc, dfr, dcm + sm[k].o[2], sm[k].n[2], stp, s);
      launch_app_update<T>(A, sc, dfr, dcm + sm[k].o[3], sm[k].n[3], stp, s);
      launch_app_move<T>(A, sc, dfr, dcm + sm[k].o[4], sm[k].n[4], stp, s);
      launches += 6;
    }
    // ---- threshold partial pivoting on what the block steps did not take;
    // at a root nothing can take delays, so a second pass keeps only the
    // small-pivot test (plain partial pivoting)
    launch_ldlt_tpp<T>(A, dfr, nslot, stp, fk.u, p_final, tpp1, s);
    SG_CUDA(cudaMemcpyAsync(tpp2, tpp1, nslot * sizeof(int), cudaMemcpyDeviceToDevice, s));
    std::vector<LdltFront> roots;
    for (int q = 0; q < nslot; ++q)
      if (st.sparent[F[q]] - 1 >= ns) roots.push_back(fr[q]);
    if (!roots.empty()) {
      put(L.fr2, roots, s);
      launch_ldlt_tpp<T>(A, L.fr2.as<LdltFront>(), (int)roots.size(), stp, kRootU, tpp1, tpp2,
                         s);
      launches++;
    }
    launches += 1;
    // ---- the level's one host synchronisation: eliminated counts and the
    // (pivoted) variable lists for the parents' maps
    std::vector<int> h(3 * nslot);
    SG_CUDA(cudaMemcpyAsync(h.data(), p_final, nslot * sizeof(int), cudaMemcpyDeviceToHost, s));
    SG_CUDA(cudaMemcpyAsync(h.data() + nslot, tpp1, 2 * nslot * sizeof(int),
                            cudaMemcpyDeviceToHost, s));
    if (!hvar_lvl.empty())
      SG_CUDA(cudaMemcpyAsync(hvar_lvl.data(), dvar + L.var_off[F[0]],
                              hvar_lvl.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
    SG_CUDA(cudaStreamSynchronize(s));
    {
      size_t o = 0;
      for (int s2 : F) {
        std::copy(hvar_lvl.begin() + o, hvar_lvl.begin() + o + L.m[s2], L.var[s2].begin());
        o += L.m[s2];
      }
    }
    for (int q = 0; q < nslot; ++q) {
      const int s2 = F[q], nn = L.n[s2];
      const int pf = h[q], t1 = h[nslot + q], t2 = h[2 * nslot + q];
      L.nelim[s2] = t2;
      // src/factor_failed.hxx:58-59, :115-120 (pivot_method tpp for fronts
      // that skip the block steps)
      if (fr[q].nblk > 0) {
        fk.not_first_pass += nn - pf;
        if (pf < nn) fk.not_second_pass += nn - t1;
      } else {
        fk.not_first_pass += nn - t1;
      }
      fk.num_delay += nn - t2;
    }
    // ---- copy-out: the level's factor columns to the compact store (the
    // blocks are given back whole once the parents have assembled them)
    if (L.copyout) {
      std::vector<CopySpan> cs;
      for (int s2 : F) {
        const int64_t len = (int64_t)L.ld[s2] * L.nelim[s2];
        L.foff[s2] = L.fused;
        L.fused += round_up64(len, 64);
        for (int64_t z = 0; z < len; z += (int64_t)1 << 20)
          cs.push_back({L.off[s2] + z, L.foff[s2] + z, std::min<int64_t>((int64_t)1 << 20, len - z)});
      }
      if ((size_t)L.fused * sizeof(T) > fk.fstore.bytes)
        grow(fk.fstore, (size_t)L.fused * sizeof(T), s);
      put(L.cspans, cs, s);
      launch_copy_spans<T>(fk.fstore.as<T>(), fk.arena.as<T>(), L.cspans.as<CopySpan>(),
                           (int)cs.size(), s);
    }
    // ---- contribution blocks: CB -= (L D) L^T over all eliminated columns
    // (form_contrib).  FP32 fronts with enough contribution rows run it on the
    // tensor cores: L and L*D of the contribution rows are split into 3xBF16
    // K-major planes (L*D rows stacked after L rows) and every 128 x 128 tile
    // takes its A rows from L*D and its B rows from L; the rest use SIMT tiles.
    {
      std::vector<LdltFront> cfr;
      std::vector<CtaMap> cm;
      std::vector<UpdTask> ut;
      std::vector<TcSplit> spl, spd;
      std::vector<TcTask> tct;
      int64_t cscr = 0, tcrows = 0, max_rows = 0;
      int pitch = 0;
      const bool tc_ok = std::is_same<T, float>::value && fk.use_tc;
      const int tc_min = Schedule::current().tc_rows();
      for (int q = 0; q < nslot; ++q) {
        int s2 = F[q];
        int m = L.m[s2], n = L.n[s2], ne = L.nelim[s2];
        if (m <= n || ne == 0) continue;
        LdltFront f = fr[q];
        f.p = ne;
        f.ldp_off = cscr;
        cscr += (int64_t)m * ne;
        int kf = (int)cfr.size();
        cfr.push_back(f);
        add_slice(cm, kf, ceil_div(m - n, LDLT_RT));
        const int mc = m - n;
        if (tc_ok && tc_min > 0 && mc >= tc_min) {
          pitch = std::max(pitch, (ne + TC_KCHUNK - 1) / TC_KCHUNK * TC_KCHUNK);
          const int64_t bl = tcrows, bd = tcrows + mc;
          tcrows += 2 * (int64_t)mc;
          max_rows = std::max<int64_t>(max_rows, mc);
          spl.push_back({f.off, f.ld, m, n, ne, (int)bl, 0});
          spd.push_back({f.ldp_off, m, m, n, ne, (int)bd, 0});
          const int nk = (ne + TC_KCHUNK - 1) / TC_KCHUNK;
          for (int cj = 0; n + cj * 128 < m; ++cj)
            for (int ri = cj; n + ri * 128 < m; ++ri)
              tct.push_back({f.off, f.ld, n + ri * 128, n + cj * 128, m, m,
                             (int)(bd + ri * 128), (int)(bl + cj * 128), nk, 0});
        } else {
          for (int cj = 0; n + cj * TM < m; ++cj)
            for (int ri = cj; n + ri * TM < m; ++ri)
              ut.push_back({f.off, f.ldp_off, f.off, f.ld, m, f.ld, n + ri * TM, n + cj * TM, m,
                            m, 0, ne, 0});
        }
      }
      if (!cfr.empty()) {
        if (L.sc2.bytes < (size_t)std::max<int64_t>(cscr, 1) * sizeof(T))
          L.sc2.ensure((size_t)std::max<int64_t>(cscr, 1) * sizeof(T));
        put(L.fr2, cfr, s);
        put(L.cmap2, cm, s);
        launch_ldlt_calc_ld<T>(A, L.sc2.as<T>(), L.fr2.as<LdltFront>(), L.cmap2.as<CtaMap>(),
                               (int)cm.size(), stp, s);
        launches++;
        if (!ut.empty()) {
          put(L.up, ut, s);
          launch_update<T>(A, L.sc2.as<T>(), L.up.as<UpdTask>(), (int)ut.size(), s);
          launches++;
        }
        if constexpr (std::is_same<T, float>::value) {
          if (!tct.empty()) {
            // planes of tcrows x pitch BF16 each, 128-byte aligned
            const int64_t pstride = (tcrows * pitch + 63) / 64 * 64;
            if (L.tcplanes.bytes < (size_t)3 * pstride * sizeof(uint16_t))
              L.tcplanes.ensure((size_t)3 * pstride * sizeof(uint16_t));
            uint16_t* planes = L.tcplanes.as<uint16_t>();
            std::vector<TcSplit> all(spl);
            all.insert(all.end(), spd.begin(), spd.end());
            put(L.tcsplit, all, s);
            put(L.tctask, tct, s);
            launch_split_t(A, L.tcsplit.as<TcSplit>(), (int)spl.size(), max_rows, planes,
                           pstride, pitch, s);
            launch_split_t(L.sc2.as<float>(), L.tcsplit.as<TcSplit>() + spl.size(),
                           (int)spd.size(), max_rows, planes, pstride, pitch, s);
            CUtensorMap maps[3];
            for (int qq = 0; qq < 3; ++qq)
              make_panel_map(&maps[qq], planes + qq * pstride, tcrows, pitch);
            launch_update_tc(maps, A, L.tctask.as<TcTask>(), (int)tct.size(),
                             fk.tcerr.as<unsigned>(), s);
            launches += 3;
          }
        }
      }
    }
  }
  // ---- statistics and inertia from D (src/NumericTree.hxx:143-178)
  std::vector<double> D(std::max<int64_t>(L.d_used, 1));
  unsigned sth = 0, tce = 0;
  SG_CUDA(cudaMemcpyAsync(D.data(), L.dall.p, L.d_used * sizeof(double), cudaMemcpyDeviceToHost,
                          s));
  SG_CUDA(cudaMemcpyAsync(&sth, status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaMemcpyAsync(&tce, fk.tcerr.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaStreamSynchronize(s));
  if (tce) throw CudaError("tensor-core update: a bounded wait timed out");
  fk.launches = launches;
  fk.num_neg = fk.num_two = fk.num_zero = 0;
  fk.num_factor = 0;
  int rank = 0;
  int uneliminated = 0;
  for (int s2 = 0; s2 < ns; ++s2) {
    const double* d = &D[L.d_off[s2]];
    int ne = L.nelim[s2];
    fk.num_factor += (int64_t)ne * L.m[s2] - (int64_t)ne * (ne - 1) / 2;
    if (st.sparent[s2] - 1 >= ns) uneliminated += L.n[s2] - ne;
    for (int i = 0; i < ne;) {
      double a11 = d[2 * i], a21 = d[2 * i + 1];
      if (i + 1 == ne || std::isfinite(d[2 * i + 2])) {
        if (a11 == 0.0) fk.num_zero++;
        else rank++;
        if (a11 < 0.0) fk.num_neg++;
        i++;
      } else {
        double a22 = d[2 * i + 3];
        fk.num_two++;
        double det = a11 * a22 - a21 * a21, tr = a11 + a22;
        if (det < 0) fk.num_neg++;
        else if (tr < 0) fk.num_neg += 2;
        rank += 2;
        i += 2;
      }
    }
  }
  fk.num_zero += uneliminated;
  fk.rank = rank;
  fk.flag = 0;
  if ((sth & ST_SINGULAR) || (uneliminated && !fk.action)) fk.flag = -5;
  else if (fk.num_zero > 0) fk.flag = 7;
  // ---- solve descriptors (level order, small fronts first)
  L.hsfr.assign(ns, FrontDesc{});
  L.hsscr.assign(ns, 0);
  L.hsdoff.assign(ns, 0);
  std::vector<FrontDesc> tmp(ns);
  for (int k = 0; k < ns; ++k) {
    int s2 = fk.order[k];
    tmp[k] = FrontDesc{L.copyout ? L.foff[s2] : L.off[s2], L.ld[s2], L.m[s2], L.nelim[s2],
                       L.var_off[s2], 0};
  }
  std::vector<int> pm = SolvePlan::small_first(tmp, fk.levels);
  for (int k = 0; k < ns; ++k) {
    L.hsfr[k] = tmp[pm[k]];
    L.hsdoff[k] = L.d_off[fk.order[pm[k]]];
  }
  L.scratch_rows = 0;
  for (const Level& lev : fk.levels) {
    int64_t acc = 0;
    for (int k = lev.f0; k < lev.f1; ++k) {
      L.hsscr[k] = acc;
      acc += L.hsfr[k].m;
    }
    L.scratch_rows = std::max(L.scratch_rows, acc);
  }
  fk.clear_solve_graphs();
  put(L.sfr, L.hsfr, s);
  put(L.sscr, L.hsscr, s);
  put(L.sdoff, L.hsdoff, s);
  // per-step launches unless asked for: on the shifted 7-point 48^3 matrix (4
  // right-hand sides, five corrections) the dataflow sweeps measured slower
  // (refined solve 23.0-24.2 ms against 21.0-22.4 ms)
  fk.splan.dataflow = Schedule::current().solve_dataflow > 0;
  fk.splan.build_tasks(L.hsfr, fk.levels, (int)sizeof(T), s);
  fk.splan.compute_inverses<T>(static_cast<const T*>(fk.factor_base()), L.sfr.as<FrontDesc>(),
                              true, s);
  SG_CUDA(cudaStreamSynchronize(s));
  return fk.flag;
}

int factorize_ldlt(FKeep& fk, const double* val_dev, cudaStream_t s) {
  // values: clean copy for residuals, fkeep-owned copy for the schedule
  AKeep& a = *fk.ak;
  launch_gather_clean(val_dev, fk.srcptr.as<int64_t>(), fk.src.as<int64_t>(),
                      (int64_t)a.clean.crow.size(), fk.cval.as<double>(), s);
  launch_gather(fk.cval.as<double>(), fk.fidx.as<int64_t>(), (int64_t)a.fcol.size(),
                fk.faval.as<double>(), s);
  SG_CUDA(cudaMemsetAsync(fk.anorm.p, 0, sizeof(double), s));
  launch_rownorm_inf(fk.frow.as<int64_t>(), fk.faval.as<double>(), a.n, fk.anorm.as<double>(), s);
  if (val_dev != fk.val.as<double>()) {
    int64_t nz = fk.nnz_orig();
    fk.val.ensure(std::max<int64_t>(nz, 1) * sizeof(double));
    if (nz) SG_CUDA(cudaMemcpyAsync(fk.val.p, val_dev, nz * sizeof(double),
                                    cudaMemcpyDeviceToDevice, s));
  }
  fk.apply_scale(s);
  SG_CUDA(cudaMemcpyAsync(&fk.anorm_h, fk.anorm.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  fk.not_first_pass = fk.not_second_pass = 0;
  cudaEvent_t e0, e1;
  SG_CUDA(cudaEventCreate(&e0));
  SG_CUDA(cudaEventCreate(&e1));
  SG_CUDA(cudaEventRecord(e0, s));
  int flag = fk.precision == 1 ? factorize_ldlt_t<float>(fk, s) : factorize_ldlt_t<double>(fk, s);
  SG_CUDA(cudaEventRecord(e1, s));
  SG_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  fk.factor_ms = ms;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return flag;
}

template <typename ACC>
static void ldlt_solve_t(FKeep& fk, int job, ACC* xp, int nrhs, cudaStream_t s) {
  LdltState& L = *fk.ldlt;
  const int n = fk.ak->n;
  bool fwd = job == 0 || job == 1;
  bool diag = job == 0 || job == 2 || job == 4;
  bool bwd = job == 0 || job == 3 || job == 4;
  fk.scratch.ensure(std::max<int64_t>(L.scratch_rows * std::min(nrhs, 32), 1) * sizeof(ACC));
  const FrontDesc* fr = L.sfr.as<FrontDesc>();
  const int64_t* sc = L.sscr.as<int64_t>();
  const int64_t* dof = L.sdoff.as<int64_t>();
  const int* var = L.dvar.as<int>();
  using T = ACC;  // factors and accumulation share the factor precision
  const T* A = static_cast<const T*>(fk.factor_base());
  fk.splan.ensure_tt(sizeof(ACC), L.scratch_rows * std::min(nrhs, 32), n);
  fk.replay(job, nrhs, xp, s, [&]() {
    for (int r0 = 0; r0 < nrhs; r0 += 32) {
      int nr = std::min(32, nrhs - r0);
      ACC* xr = xp + (int64_t)r0 * n;
      if (fwd)
        fk.splan.run<T, ACC>(true, A, fr, var, xr, n, nr, fk.scratch.as<ACC>(), sc, true, s);
      if (diag)
        launch_solve_diag<ACC>(fr, (int)L.hsfr.size(), var, L.dall.as<double>(), dof, xr, n,
                               nr, s);
      if (bwd)
        fk.splan.run<T, ACC>(false, A, fr, var, xr, n, nr, fk.scratch.as<ACC>(), sc, true, s);
    }
  });
}

void ldlt_solve_pivot_order(FKeep& fk, int job, float* xp, int nrhs, cudaStream_t s) {
  ldlt_solve_t<float>(fk, job, xp, nrhs, s);
}
void ldlt_solve_pivot_order(FKeep& fk, int job, double* xp, int nrhs, cudaStream_t s) {
  ldlt_solve_t<double>(fk, job, xp, nrhs, s);
}

bool ldlt_solve_tables(const FKeep& fk, const FrontDesc** fr, const int64_t** scr,
                       const int** rows, int64_t* scratch_rows) {
  if (!fk.ldlt || fk.ldlt->hsfr.empty()) return false;
  const LdltState& L = *fk.ldlt;
  *fr = L.sfr.as<FrontDesc>();
  *scr = L.sscr.as<int64_t>();
  *rows = L.dvar.as<int>();
  *scratch_rows = L.scratch_rows;
  return true;
}

int ldlt_export_diag(const FKeep& fk, double* d, int* piv_order) {
  if (!fk.ldlt) return 0;
  const LdltState& L = *fk.ldlt;
  if (L.d_used == 0) return 0;
  std::vector<double> D(L.d_used);
  SG_CUDA(cudaMemcpy(D.data(), L.dall.p, L.d_used * sizeof(double), cudaMemcpyDeviceToHost));
  int k = 0;
  for (int s = 0; s < (int)L.nelim.size(); ++s)
    for (int i = 0; i < L.nelim[s]; ++i) {
      if (d) {
        d[2 * k] = D[L.d_off[s] + 2 * i];
        d[2 * k + 1] = D[L.d_off[s] + 2 * i + 1];
      }
      if (piv_order) piv_order[k] = L.var[s][i] + 1;
      k++;
    }
  return k;
}

int ldlt_export_fronts(const FKeep& fk, int* m, int* n, int* nelim) {
  if (!fk.ldlt) return 0;
  const LdltState& L = *fk.ldlt;
  const int ns = (int)L.nelim.size();
  for (int s = 0; s < ns; ++s) {
    if (m) m[s] = L.m[s];
    if (n) n[s] = L.n[s];
    if (nelim) nelim[s] = L.nelim[s];
  }
  return ns;
}

}  // namespace sylver_gb300
