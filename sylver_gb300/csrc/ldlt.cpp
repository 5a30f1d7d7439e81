// Host driver of the threshold-pivoted LDL^T factorization.
//
// Replaces the reference's indefinite numeric tree (src/NumericTree.hxx:54-181,
// :186-406), front allocation with delays (src/NumericFront.hxx:73-145),
// assembly of delayed columns (src/kernels/assemble.hxx:926-1093), the APP
// driver (src/factor_indef.hxx:1484-1646), the failed-pivot TPP pass
// (src/factor_failed.hxx:29-157) and the inertia reduction
// (src/NumericTree.hxx:143-178).
//
// Fronts are processed level by level (height in the assembly tree).  Front
// sizes depend on how many columns the children delayed, so each level is
// planned on the host once its children are done.  Inside a level every
// block-column step is one launch sequence over all fronts of the level:
//   diag (complete pivoting, FP64) -> apply (solve + threshold test) ->
//   host reads the passed counts -> commit -> trailing update (tile GEMM).
// Columns that no block accepts go through threshold partial pivoting; what
// still fails is delayed to the parent, whose front grows accordingly.
#include "ldlt.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "ldlt_dev.hpp"

namespace sylver_gb300 {

struct LdltState {
  // per front (original index)
  std::vector<int> m, n, nelim, ld, var_off;
  std::vector<int64_t> off, d_off;
  std::vector<std::vector<int>> var;  // host copy after factorization
  int64_t arena_used = 0, var_used = 0, d_used = 0;
  DevMem dvar, dall, blk, bdinv, lperm, npass_raw, npass, tppo;
  DevMem fr, rt, up, sc;  // per-launch descriptor buffers + scratch
  DevMem ea_cd, ea_items, ea_maps, am_src, am_dst;
  // solve
  DevMem sfr, sscr, sdoff;
  std::vector<FrontDesc> hsfr;
  std::vector<int64_t> hsscr, hsdoff;
  int64_t scratch_rows = 0;
};

namespace {

inline int round_up(int v, int a) { return (v + a - 1) / a * a; }
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
  // arena: symbolic size plus headroom for delays; grows when a level needs
  int64_t sym = 0;
  for (int s = 0; s < ns; ++s) sym += round_up64((int64_t)round_up(st.nrow[s], 4) * st.nrow[s], 64);
  fk.arena_elems = sym + sym / 8 + 1024;
}

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
  L.arena_used = L.var_used = L.d_used = 0;
  fk.arena.ensure((size_t)fk.arena_elems * sizeof(T));
  L.blk.ensure(1);
  unsigned* status = fk.status.as<unsigned>();
  SG_CUDA(cudaMemsetAsync(status, 0, sizeof(unsigned), s));
  long launches = 0;
  std::vector<int> pos(st.n, -1);
  const double u = fk.u, small = fk.small_piv;

  for (const Level& lev : fk.levels) {
    std::vector<int> F(fk.order.begin() + lev.f0, fk.order.begin() + lev.f1);
    // ---- sizes, variable lists, storage
    int64_t lvl_off0 = L.arena_used;
    std::vector<int> hvar_lvl;
    for (int s : F) {
      int sncol = st.ncol[s], snrow = st.nrow[s];
      int ndin = 0;
      for (int c : st.children[s]) ndin += L.n[c] - L.nelim[c];
      L.n[s] = sncol + ndin;
      L.m[s] = snrow + ndin;
      L.ld[s] = round_up(std::max(L.m[s], 1), 4);
      L.off[s] = L.arena_used;
      L.arena_used += round_up64((int64_t)L.ld[s] * L.m[s], 64);
      L.d_off[s] = L.d_used;
      L.d_used += 2 * (int64_t)std::max(L.n[s], 1);
      L.var_off[s] = (int)L.var_used;
      L.var_used += L.m[s];
      auto& v = L.var[s];
      v.clear();
      const int* rl = &st.rlist[st.rptr[s] - 1];
      for (int i = 0; i < sncol; ++i) v.push_back(rl[i] - 1);
      for (int c : st.children[s])
        for (int j = L.nelim[c]; j < L.n[c]; ++j) v.push_back(L.var[c][j]);
      for (int i = sncol; i < snrow; ++i) v.push_back(rl[i] - 1);
      hvar_lvl.insert(hvar_lvl.end(), v.begin(), v.end());
      fk.maxfront = std::max(fk.maxfront, L.m[s]);
    }
    if (L.arena_used > fk.arena_elems) {
      int64_t ne = std::max(L.arena_used, fk.arena_elems + fk.arena_elems / 4);
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
    SG_CUDA(cudaMemsetAsync(A + lvl_off0, 0, (size_t)(L.arena_used - lvl_off0) * sizeof(T), s));
    SG_CUDA(cudaMemsetAsync(L.dall.as<double>() + L.d_off[F[0]], 0,
                            (size_t)(L.d_used - L.d_off[F[0]]) * sizeof(double), s));
    // ---- original entries (rows below the own columns shift by ndelay_in)
    {
      std::vector<int64_t> asrc, adst;
      bool atomic = false;
      for (int s : F) {
        int snrow = st.nrow[s], sncol = st.ncol[s], ndin = L.n[s] - sncol;
        int64_t prev = -1;
        for (int64_t k = st.nptr[s] - 1; k < st.nptr[s + 1] - 1; ++k) {
          int64_t src = st.nlist[2 * k] - 1, dest = st.nlist[2 * k + 1] - 1;
          int64_t c = dest / snrow, r = dest % snrow;
          if (r >= sncol) r += ndin;
          asrc.push_back(src);
          adst.push_back(L.off[s] + c * L.ld[s] + r);
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
    // ---- children: delayed columns and contribution blocks
    {
      std::vector<ChildDesc> cds;
      std::vector<EaItem> items;
      std::vector<int> maps;
      for (int p : F) {
        for (int i = 0; i < L.m[p]; ++i) pos[L.var[p][i]] = i;
        for (int c : st.children[p]) {
          int mc = L.m[c] - L.nelim[c];
          if (mc <= 0) continue;
          ChildDesc cd;
          cd.cb_off = L.off[c] + (int64_t)L.nelim[c] * L.ld[c] + L.nelim[c];
          cd.p_off = L.off[p];
          cd.ld_c = L.ld[c];
          cd.ld_p = L.ld[p];
          cd.mc = mc;
          cd.map_off = (int)maps.size();
          for (int i = L.nelim[c]; i < L.m[c]; ++i) maps.push_back(pos[L.var[c][i]]);
          int ci = (int)cds.size();
          cds.push_back(cd);
          for (int j = 0; j < mc; ++j) items.push_back({ci, j});
        }
      }
      if (!items.empty()) {
        put(L.ea_cd, cds, s);
        put(L.ea_items, items, s);
        put(L.ea_maps, maps, s);
        launch_extend_add<T>(A, L.ea_cd.as<ChildDesc>(), L.ea_items.as<EaItem>(),
                             L.ea_maps.as<int>(), (int)items.size(), s);
        launches++;
      }
    }
    // ---- block-column steps (a posteriori pivoting)
    const int nslot = (int)F.size();
    L.blk.ensure((size_t)nslot * LDLT_BW * (LDLT_BW + 1) * sizeof(double));
    L.bdinv.ensure((size_t)nslot * 2 * LDLT_BW * sizeof(double));
    L.lperm.ensure((size_t)nslot * LDLT_BW * sizeof(int));
    L.npass_raw.ensure((size_t)nslot * sizeof(int));
    L.npass.ensure((size_t)nslot * sizeof(int));
    L.tppo.ensure((size_t)nslot * sizeof(int));
    LdltStep stp{L.blk.as<double>(), L.bdinv.as<double>(), L.lperm.as<int>(),
                 L.npass_raw.as<int>(), L.npass.as<int>(), dvar, L.dall.as<double>(), status,
                 u, small, fk.action ? 1 : 0};
    std::vector<int> p(nslot, 0);
    std::vector<char> app_done(nslot, 0);
    // small fronts may skip the block steps and go to TPP directly
    const int tpp_cols = Schedule::current().ldlt_tpp_cols;
    for (int q = 0; q < nslot; ++q) app_done[q] = L.n[F[q]] == 0 || L.n[F[q]] <= tpp_cols;
    std::vector<int> hraw, hnp;
    std::vector<double> hdv;
    for (;;) {
      std::vector<LdltFront> fr;
      std::vector<int> slot;
      int64_t scr = 0;
      for (int q = 0; q < nslot; ++q) {
        if (app_done[q]) continue;
        int s2 = F[q];
        LdltFront f{};
        f.off = L.off[s2];
        f.ld = L.ld[s2];
        f.m = L.m[s2];
        f.n = L.n[s2];
        f.p = p[q];
        f.w = std::min(LDLT_BW, L.n[s2] - p[q]);
        f.fidx = q;
        f.var_off = L.var_off[s2];
        f.d_off = L.d_off[s2];
        f.pan_off = scr;
        scr += (int64_t)f.m * LDLT_BW;
        f.ldp_off = scr;
        scr += (int64_t)f.m * LDLT_BW;
        fr.push_back(f);
        slot.push_back(q);
      }
      if (fr.empty()) break;
      L.sc.ensure((size_t)std::max<int64_t>(scr, 1) * sizeof(T));
      put(L.fr, fr, s);
      std::vector<int> init_np(nslot, LDLT_BW);
      for (auto& f : fr) init_np[f.fidx] = f.w;
      put(L.npass_raw, init_np, s);
      L.npass_raw.ensure((size_t)nslot * sizeof(int));
      stp.npass_raw = L.npass_raw.as<int>();
      // apply row tiles (rows below the block)
      std::vector<RowTask> at;
      for (int k = 0; k < (int)fr.size(); ++k)
        for (int r0 = fr[k].p + fr[k].w; r0 < fr[k].m; r0 += LDLT_RT) at.push_back({k, r0});
      launch_ldlt_diag<T>(A, L.fr.as<LdltFront>(), (int)fr.size(), stp, s);
      launches++;
      if (!at.empty()) {
        put(L.rt, at, s);
        launch_ldlt_apply<T>(A, L.sc.as<T>(), L.fr.as<LdltFront>(), L.rt.as<RowTask>(),
                             (int)at.size(), stp, s);
        launches++;
      }
      hraw.resize(nslot);
      hdv.resize((size_t)nslot * 2 * LDLT_BW);
      SG_CUDA(cudaMemcpyAsync(hraw.data(), L.npass_raw.p, nslot * sizeof(int),
                              cudaMemcpyDeviceToHost, s));
      SG_CUDA(cudaMemcpyAsync(hdv.data(), L.bdinv.p, hdv.size() * sizeof(double),
                              cudaMemcpyDeviceToHost, s));
      SG_CUDA(cudaStreamSynchronize(s));
      // drop a 2x2 pivot split by the threshold failure (Column::adjust)
      hnp.assign(nslot, 0);
      for (auto& f : fr) {
        int np = std::min(hraw[f.fidx], f.w);
        const double* d = &hdv[(size_t)f.fidx * 2 * LDLT_BW];
        if (np > 0 && std::isfinite(d[2 * (np - 1)]) && d[2 * (np - 1) + 1] != 0.0) np--;
        hnp[f.fidx] = np;
      }
      put(L.npass, hnp, s);
      stp.npass = L.npass.as<int>();
      // commit rows [p, m)
      std::vector<RowTask> ct;
      for (int k = 0; k < (int)fr.size(); ++k)
        for (int r0 = fr[k].p; r0 < fr[k].m; r0 += LDLT_RT) ct.push_back({k, r0});
      put(L.rt, ct, s);
      launch_ldlt_commit<T>(A, L.sc.as<T>(), L.fr.as<LdltFront>(), L.rt.as<RowTask>(),
                            (int)ct.size(), stp, s);
      launches++;
      // trailing update of the fully-summed part
      std::vector<UpdTask> ut;
      for (auto& f : fr) {
        int np = hnp[f.fidx];
        if (np == 0) continue;
        int o = f.p + np;
        for (int cj = 0; o + cj * TM < f.n; ++cj)
          for (int ri = cj; o + ri * TM < f.m; ++ri)
            ut.push_back({f.off, f.ldp_off, f.off + (int64_t)f.p * f.ld, f.ld, f.m, f.ld,
                          o + ri * TM, o + cj * TM, f.m, f.n, 0, np, 0});
      }
      if (!ut.empty()) {
        put(L.up, ut, s);
        launch_update<T>(A, L.sc.as<T>(), L.up.as<UpdTask>(), (int)ut.size(), s);
        launches++;
      }
      for (auto& f : fr) {
        int q = f.fidx, np = hnp[q];
        p[q] += np;
        fk.not_first_pass += 0;
        if (np == 0 || p[q] >= L.n[F[q]]) app_done[q] = 1;
      }
    }
    // ---- threshold partial pivoting on what the blocks did not accept
    for (int pass = 0; pass < 2; ++pass) {
      std::vector<LdltFront> fr;
      for (int q = 0; q < nslot; ++q) {
        int s2 = F[q];
        if (p[q] >= L.n[s2]) continue;
        bool root = st.sparent[s2] - 1 >= ns;
        if (pass == 1 && !root) continue;
        LdltFront f{};
        f.off = L.off[s2];
        f.ld = L.ld[s2];
        f.m = L.m[s2];
        f.n = L.n[s2];
        f.p = p[q];
        f.fidx = q;
        f.var_off = L.var_off[s2];
        f.d_off = L.d_off[s2];
        fr.push_back(f);
        if (pass == 0) fk.not_first_pass += L.n[s2] - p[q];
        else fk.not_second_pass += L.n[s2] - p[q];
      }
      if (fr.empty()) continue;
      put(L.fr, fr, s);
      // nothing above a root can take delays: its second pass keeps only the
      // small-pivot test (plain partial pivoting)
      double ueff = pass == 0 ? u : 1e-300;
      launch_ldlt_tpp<T>(A, L.fr.as<LdltFront>(), (int)fr.size(), stp, ueff, L.tppo.as<int>(), s);
      launches++;
      std::vector<int> out(nslot);
      SG_CUDA(cudaMemcpyAsync(out.data(), L.tppo.p, nslot * sizeof(int), cudaMemcpyDeviceToHost,
                              s));
      SG_CUDA(cudaStreamSynchronize(s));
      for (auto& f : fr) p[f.fidx] = out[f.fidx];
    }
    for (int q = 0; q < nslot; ++q) L.nelim[F[q]] = p[q];
    // ---- contribution blocks: CB -= (L D) L^T over all eliminated columns
    {
      std::vector<LdltFront> fr;
      std::vector<RowTask> rt;
      std::vector<UpdTask> ut;
      int64_t scr = 0;
      for (int q = 0; q < nslot; ++q) {
        int s2 = F[q];
        int m = L.m[s2], n = L.n[s2], ne = L.nelim[s2];
        if (m <= n || ne == 0) continue;
        LdltFront f{};
        f.off = L.off[s2];
        f.ld = L.ld[s2];
        f.m = m;
        f.n = n;
        f.p = ne;
        f.fidx = q;
        f.d_off = L.d_off[s2];
        f.ldp_off = scr;
        scr += (int64_t)m * ne;
        int k = (int)fr.size();
        fr.push_back(f);
        for (int r0 = n; r0 < m; r0 += LDLT_RT) rt.push_back({k, r0});
        for (int cj = 0; n + cj * TM < m; ++cj)
          for (int ri = cj; n + ri * TM < m; ++ri)
            ut.push_back({f.off, f.ldp_off, f.off, f.ld, m, f.ld, n + ri * TM, n + cj * TM, m, m,
                          0, ne, 0});
      }
      if (!fr.empty()) {
        L.sc.ensure((size_t)std::max<int64_t>(scr, 1) * sizeof(T));
        put(L.fr, fr, s);
        put(L.rt, rt, s);
        put(L.up, ut, s);
        launch_ldlt_calc_ld<T>(A, L.sc.as<T>(), L.fr.as<LdltFront>(), L.rt.as<RowTask>(),
                               (int)rt.size(), stp, s);
        launch_update<T>(A, L.sc.as<T>(), L.up.as<UpdTask>(), (int)ut.size(), s);
        launches += 2;
      }
    }
    // ---- bring the (pivoted) variable lists back for the parents' maps
    if (!hvar_lvl.empty()) {
      SG_CUDA(cudaMemcpyAsync(hvar_lvl.data(), dvar + L.var_off[F[0]],
                              hvar_lvl.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
      SG_CUDA(cudaStreamSynchronize(s));
      size_t o = 0;
      for (int s2 : F) {
        std::copy(hvar_lvl.begin() + o, hvar_lvl.begin() + o + L.m[s2], L.var[s2].begin());
        o += L.m[s2];
      }
    }
  }
  // ---- statistics and inertia from D (src/NumericTree.hxx:143-178)
  std::vector<double> D(std::max<int64_t>(L.d_used, 1));
  unsigned sth = 0;
  SG_CUDA(cudaMemcpyAsync(D.data(), L.dall.p, L.d_used * sizeof(double), cudaMemcpyDeviceToHost,
                          s));
  SG_CUDA(cudaMemcpyAsync(&sth, status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaStreamSynchronize(s));
  fk.launches = launches;
  fk.num_neg = fk.num_two = fk.num_zero = fk.num_delay = 0;
  fk.num_factor = 0;
  int rank = 0;
  int uneliminated = 0;
  for (int s2 = 0; s2 < ns; ++s2) {
    const double* d = &D[L.d_off[s2]];
    int ne = L.nelim[s2];
    fk.num_factor += (int64_t)ne * L.m[s2] - (int64_t)ne * (ne - 1) / 2;
    if (st.sparent[s2] - 1 < ns) fk.num_delay += L.n[s2] - ne;
    else uneliminated += L.n[s2] - ne;
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
    tmp[k] = FrontDesc{L.off[s2], L.ld[s2], L.m[s2], L.nelim[s2], L.var_off[s2], 0};
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
  fk.splan.build_tasks(L.hsfr, fk.levels, s);
  fk.splan.compute_inverses<T>(fk.arena.as<T>(), L.sfr.as<FrontDesc>(), true, s);
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
  const T* A = fk.arena.as<T>();
  fk.splan.ensure_tt(sizeof(ACC), L.scratch_rows * std::min(nrhs, 32));
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

}  // namespace sylver_gb300
