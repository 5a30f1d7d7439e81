// Threshold-pivoted LDL^T kernels: a-posteriori pivoting (APP) by block
// columns of 32, threshold partial pivoting (TPP) for what fails.  Pivot
// decisions, 2x2 inversions and the acceptance test run in FP64 whatever the
// storage type.
//
// Reference algorithm (math and control flow, not code), with the block
// size equal to the inner block size 32 (one level of blocking):
//   APP block-column loop          src/factor_indef.hxx:1338-1474 (notask),
//                                  :885-1183
//   Block::factor: block_ldlt<T,32> on a full 32x32 diagonal block,
//     ldlt_tpp_factor on a partial one (nrow() x ncol(), so the first CB
//     rows of the block row take part)  src/kernels/ldlt_app.hxx:458-560
//   apply_pivot<OP_N/OP_T> + check_threshold
//                                  src/kernels/ldlt_app.hxx:145-255, :579-601
//   Column::adjust (split 2x2)     include/sylver/kernels/Column.hxx:87-101
//   restore_if_required            src/kernels/ldlt_app.hxx:405-431
//   Block::update / calcLD         src/kernels/ldlt_app.hxx:619-718
//   permute_failed                 src/factor_indef.hxx:1190-1288
//   factor_front_indef_failed      src/factor_failed.hxx:29-157
// SPRAL's block_ldlt and ldlt_tpp_factor are not vendored; the pivot
// searches below restate the published algorithms (Duff, Hogg & Lopez,
// SISC 2020): complete pivoting with a 1x1 / 2x2 choice on a full block,
// threshold partial pivoting elsewhere.
//
// Layout difference, same elimination: the reference leaves failed columns
// in their block and applies later pivots to them through the blocks to
// their left (ApplyT / UpdateT), then permutes them to the back at the end.
// Here the commit of a block moves its failed columns behind all columns not
// yet processed, so the next block is the same set of columns as the
// reference's next block, later pivots reach the failed columns as ordinary
// rows below (same multipliers, same threshold test), and at the end they
// are already at the back, in the order the reference puts them.
//
// D^-1 uses the reference storage (src/kernels/ldlt_app.hxx:166-171):
// 1x1 [d^-1, 0], 2x2 [a, b, Inf, c] with (a b; b c) = D^-1, zero pivot [0, 0].
//
// Arithmetic order: every multiply-add of the FP64 path is an explicit
// __fma_rn / __dmul_rn and the file is compiled without FMA contraction, so
// that a CPU restatement with std::fma in the same order reproduces the
// factors bit for bit.
#include <cfloat>

#include "ldlt_dev.hpp"
#include "tile_update.cuh"

namespace sylver_gb300 {

namespace {

constexpr int BW = LDLT_BW;
constexpr int LDB = BW + 1;

__device__ __forceinline__ double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ double mul_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float mul_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double dinf() { return __longlong_as_double(0x7ff0000000000000LL); }

__device__ __forceinline__ int block_width(const LdltFront& F, int k) {
  return min(BW, F.n - BW * k);
}
// CB rows that join a partial diagonal block (the reference's block row of
// 32 rows reaches past n)
__device__ __forceinline__ int extra_rows(const LdltFront& F, int w) {
  return w == BW ? 0 : min(BW - w, F.m - F.n);
}

// Warp-wide argmax of v over lanes (first maximum: lowest index on ties);
// lanes with nothing to offer pass v = -1, idx = -1.
template <typename C>
__device__ __forceinline__ void warp_argmax(C& v, int& idx) {
  for (int o = 16; o > 0; o >>= 1) {
    C ov = __shfl_xor_sync(0xffffffffu, v, o);
    int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov > v || (ov == v && oi >= 0 && (idx < 0 || oi < idx))) {
      v = ov;
      idx = oi;
    }
  }
}

// ---------------------------------------------------------------------------
// Diagonal block of step k (one CTA per front, warp 0 pivots).
//   full block (32 columns): complete pivoting over the block, 1x1 or 2x2;
//   partial block (w < 32 columns, the front's last): threshold partial
//   pivoting over the w columns with rows = the w block rows followed by the
//   first e = min(32 - w, m - n) contribution rows.
// Output: the factored block (unit L, lower) in blk, D^-1, the local
// permutation, the number of pivots taken (ndiag, also the initial
// npass_raw), the L rows of the e extra rows into the apply panel; the block
// permutation is applied to the rows of the eliminated columns [0, p) and to
// the variable list.
template <typename T>
__global__ void __launch_bounds__(128) k_app_diag(T* __restrict__ arena, T* __restrict__ scratch,
                                                  const LdltFront* __restrict__ fr,
                                                  const CtaMap* __restrict__ cm, LdltStep st) {
  using C = T;  // block arithmetic; FP64 for the pivot tests and 2x2 inverses
  __shared__ C a[BW][LDB];  // a[j][i] = panel(i, j); i >= j, or i >= w (extra rows)
  __shared__ double dv[2 * BW];
  __shared__ int perm[BW];
  __shared__ int s_nd;
  const LdltFront F = fr[cm[blockIdx.x].f];
  const int q = F.fidx, w = block_width(F, st.k), e = extra_rows(F, w), R = w + e;
  const int p = st.p_cur[q];
  T* A = arena + F.off;
  const int ld = F.ld;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  auto prow = [&](int i) { return i < w ? p + i : F.n + (i - w); };  // panel row -> front row
  for (int idx = tid; idx < R * w; idx += blockDim.x) {
    int i = idx % R, j = idx / R;
    if (i >= j) a[j][i] = (C)A[(int64_t)(p + j) * ld + prow(i)];
  }
  if (tid < BW) perm[tid] = tid;
  if (tid < 2 * BW) dv[tid] = 0.0;
  __syncthreads();
  if (warp == 0) {
    __syncwarp();  // reconverge after the lane-dependent staging loop
    // symmetric swap of candidates x < y (lower storage), rows [0, R)
    auto swap_xy = [&](int x, int y) {
      if (x == y) return;
      if (x > y) { int t = x; x = y; y = t; }
      int kk = lane;
      if (kk < R) {
        C t;
        if (kk < x) { t = a[kk][x]; a[kk][x] = a[kk][y]; a[kk][y] = t; }
        else if (kk == x) { t = a[x][x]; a[x][x] = a[y][y]; a[y][y] = t; }
        else if (kk < y) { t = a[x][kk]; a[x][kk] = a[kk][y]; a[kk][y] = t; }
        else if (kk > y) { t = a[x][kk]; a[x][kk] = a[y][kk]; a[y][kk] = t; }
      }
      if (lane == 0) { int t = perm[x]; perm[x] = perm[y]; perm[y] = t; }
      __syncwarp();
    };
    // 1x1 pivot at s: candidate columns (s, cend), rows [j, R)
    auto elim1 = [&](int s, int cend) {
      const C di = C(1) / a[s][s];
      const int j = lane;
      if (j > s && j < cend) {
        const C lj = mul_(a[s][j], di);
        for (int i = j; i < R; ++i) a[j][i] = fma_(-a[s][i], lj, a[j][i]);
      }
      __syncwarp();
      if (lane > s && lane < R) a[s][lane] = mul_(a[s][lane], di);
      if (lane == 0) {
        a[s][s] = C(1);
        dv[2 * s] = (double)di;
        dv[2 * s + 1] = 0.0;
      }
      __syncwarp();
    };
    // 2x2 pivot at (s, s+1)
    auto elim2 = [&](int s, int cend) {
      const double a11 = a[s][s], a21 = a[s][s + 1], a22 = a[s + 1][s + 1];
      const double det = __dsub_rn(mul_(a11, a22), mul_(a21, a21));
      const double i11 = a22 / det, i12 = -a21 / det, i22 = a11 / det;
      const int j = lane;
      if (j > s + 1 && j < cend) {
        const double w1 = a[s][j], w2 = a[s + 1][j];
        const C l1 = (C)fma_(i11, w1, mul_(i12, w2)), l2 = (C)fma_(i12, w1, mul_(i22, w2));
        for (int i = j; i < R; ++i) a[j][i] = fma_(-a[s + 1][i], l2, fma_(-a[s][i], l1, a[j][i]));
      }
      __syncwarp();
      if (lane > s + 1 && lane < R) {
        const double w1 = a[s][lane], w2 = a[s + 1][lane];
        a[s][lane] = (C)fma_(i11, w1, mul_(i12, w2));
        a[s + 1][lane] = (C)fma_(i12, w1, mul_(i22, w2));
      }
      if (lane == 0) {
        a[s][s] = C(1);
        a[s][s + 1] = C(0);
        a[s + 1][s + 1] = C(1);
        dv[2 * s] = i11;
        dv[2 * s + 1] = i12;
        dv[2 * s + 2] = dinf();
        dv[2 * s + 3] = i22;
      }
      __syncwarp();
    };
    // zero pivot at s: column of L is zero
    auto elim0 = [&](int s) {
      if (lane >= s && lane < R) a[s][lane] = (lane == s) ? C(1) : C(0);
      if (lane == 0) {
        dv[2 * s] = 0.0;
        dv[2 * s + 1] = 0.0;
        atomicOr(st.status, ST_ZERO_PIVOT);
      }
      __syncwarp();
    };
    int s = 0;
    if (w == BW) {
      // ---- complete pivoting (block_ldlt)
      while (s < w) {
        C best = C(-1);
        int bi = -1, bj = -1;
        if (lane >= s && lane < w)
          for (int i = lane; i < w; ++i) {
            C v = fabs(a[lane][i]);
            if (v > best) { best = v; bi = i; bj = lane; }
          }
        for (int o = 16; o > 0; o >>= 1) {
          C ob = __shfl_xor_sync(0xffffffffu, best, o);
          int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          int oj = __shfl_xor_sync(0xffffffffu, bj, o);
          if (ob > best || (ob == best && (oj < bj || (oj == bj && oi < bi)))) {
            best = ob; bi = oi; bj = oj;
          }
        }
        const double amax = best;
        if (!(amax >= st.small)) {
          // the rest of the block is (numerically) zero: zero pivots
          for (int kk = s; kk < w; ++kk) {
            if (lane >= kk && lane < w) a[kk][lane] = (lane == kk) ? C(1) : C(0);
            if (lane == 0) { dv[2 * kk] = 0.0; dv[2 * kk + 1] = 0.0; }
          }
          if (lane == 0) atomicOr(st.status, st.action ? ST_ZERO_PIVOT : ST_SINGULAR);
          __syncwarp();
          s = w;
          break;
        }
        const int t = bi, qq = bj;  // t >= qq
        bool two = false;
        int piv = t;
        if (t != qq) {
          double dt = fabs((double)a[t][t]), dq = fabs((double)a[qq][qq]);
          if (fmax(dt, dq) >= mul_(st.u, amax)) piv = (dt >= dq) ? t : qq;
          else two = true;
        }
        if (!two) {
          swap_xy(s, piv);
          elim1(s, w);
          s += 1;
        } else {
          swap_xy(s, qq);
          swap_xy(s + 1, (t == s) ? qq : t);
          elim2(s, w);
          s += 2;
        }
      }
    } else {
      // ---- threshold partial pivoting over the w candidates (ldlt_tpp_factor)
      const double lim = 1.0 / st.u;
      while (s < w) {
        int decided = 0, piv = -1, tpiv = -1;
        for (int c = s; c < w && !decided; ++c) {
          auto colv = [&](int i, int col) -> double { return i > col ? a[col][i] : a[i][col]; };
          double v = -1.0;
          int vi = -1;
          if (lane >= s && lane < R && lane != c) { v = fabs(colv(lane, c)); vi = lane; }
          warp_argmax(v, vi);
          const double amax = fmax(v, 0.0);
          const int t = vi;
          const double acc = fabs((double)a[c][c]);
          if (amax < st.small && acc < st.small) { decided = 3; piv = c; break; }
          if (acc >= mul_(st.u, amax)) { decided = 1; piv = c; break; }
          if (t >= 0 && t < w) {
            double v1 = -1.0, v2 = -1.0;
            int d1 = -1, d2 = -1;
            if (lane >= s && lane < R && lane != c && lane != t) {
              v1 = fabs(colv(lane, c)); d1 = lane;
              v2 = fabs(colv(lane, t)); d2 = lane;
            }
            warp_argmax(v1, d1);
            warp_argmax(v2, d2);
            const double ap2 = fmax(v1, 0.0), at2 = fmax(v2, 0.0);
            const double a11 = a[c][c], a22 = a[t][t], a21 = colv(t, c);
            const double det = __dsub_rn(mul_(a11, a22), mul_(a21, a21));
            if (fabs(det) > st.small && isfinite(det)) {
              const double i11 = a22 / det, i12 = -a21 / det, i22 = a11 / det;
              if (fma_(fabs(i11), ap2, mul_(fabs(i12), at2)) <= lim &&
                  fma_(fabs(i12), ap2, mul_(fabs(i22), at2)) <= lim) {
                decided = 2; piv = c; tpiv = t;
              }
            }
          }
        }
        if (!decided) break;
        if (decided == 3) {
          if (!st.action) {
            if (lane == 0) atomicOr(st.status, ST_SINGULAR);
            break;
          }
          swap_xy(s, piv);
          elim0(s);
          s += 1;
        } else if (decided == 1) {
          swap_xy(s, piv);
          elim1(s, w);
          s += 1;
        } else {
          swap_xy(s, piv);
          swap_xy(s + 1, (tpiv == s) ? piv : tpiv);
          elim2(s, w);
          s += 2;
        }
      }
    }
    if (lane == 0) s_nd = s;
  }
  __syncthreads();
  const int nd = s_nd;
  C* blk = reinterpret_cast<C*>(st.blk) + (int64_t)q * BW * LDB;
  for (int idx = tid; idx < BW * LDB; idx += blockDim.x) blk[idx] = (&a[0][0])[idx];
  if (tid < 2 * BW) st.bdinv[q * 2 * BW + tid] = dv[tid];
  if (tid < BW) st.lperm[q * BW + tid] = perm[tid];
  if (tid == 0) {
    st.ndiag[q] = nd;
    st.npass_raw[q] = nd;
  }
  // L of the extra rows (partial block) goes where apply puts rows below
  if (e > 0) {
    T* pan = scratch + F.pan_off;
    for (int idx = tid; idx < e * nd; idx += blockDim.x) {
      int i = w + idx % e, kk = idx / e;
      pan[(int64_t)kk * F.m + prow(i)] = (T)a[kk][i];
    }
  }
  // apply the block permutation to the rows of the eliminated columns [0, p)
  // and to the variable list
  for (int c = warp; c < p; c += blockDim.x / 32) {
    T v = T(0);
    if (lane < w) v = A[(int64_t)c * ld + p + perm[lane]];
    __syncwarp();
    if (lane < w) A[(int64_t)c * ld + p + lane] = v;
  }
  if (warp == 0) {
    int* var = st.var + F.var_off + p;
    int v = (lane < w) ? var[perm[lane]] : 0;
    __syncwarp();
    if (lane < w) var[lane] = v;
  }
}

// apply D^-1 to the first nd entries of a solved row (apply_pivot OP_N)
template <typename C>
__device__ __forceinline__ void apply_dinv(C* x, const double* dv, int nd, double small) {
#pragma unroll
  for (int k = 0; k < BW;) {
    if (k >= nd) break;
    if (k + 1 < nd && isinf(dv[2 * k + 2])) {
      const double x1 = x[k], x2 = x[k + 1];
      x[k] = (C)fma_(dv[2 * k], x1, mul_(dv[2 * k + 1], x2));
      x[k + 1] = (C)fma_(dv[2 * k + 1], x1, mul_(dv[2 * k + 3], x2));
      k += 2;
    } else {
      const double d = dv[2 * k];
      if (d == 0.0) {
        const double v = x[k];
        x[k] = (C)((fabs(v) < small) ? 0.0 : dinf() * v);
      } else {
        x[k] = mul_(x[k], (C)d);
      }
      k += 1;
    }
  }
}

// rows below block step k in a compressed index: [p + w, n), then (a partial
// block's extra rows excluded) [n + e, m)
struct BelowRows {
  int lo, n, e, m;
  __device__ int count() const { return (n - lo) + (m - n - e); }
  __device__ int row(int ci) const { return ci < n - lo ? lo + ci : n + e + (ci - (n - lo)); }
};

// ---------------------------------------------------------------------------
// Rows below the diagonal block: x = a P L_kk^-T D^-1 over the ndiag pivots,
// into the apply panel; the least pivot with |x| > 1/u lowers npass_raw.
template <typename T>
__global__ void __launch_bounds__(LDLT_RT) k_app_apply(const T* __restrict__ arena,
                                                      T* __restrict__ scratch,
                                                      const LdltFront* __restrict__ fr,
                                                      const CtaMap* __restrict__ cm,
                                                      LdltStep st) {
  using C = T;
  __shared__ C L[BW][LDB];
  __shared__ double dv[2 * BW];
  __shared__ int perm[BW];
  __shared__ C xs[BW][LDLT_RT + 1];
  __shared__ int fail;
  const CtaMap c = cm[blockIdx.x];
  const LdltFront F = fr[c.f];
  const int q = F.fidx, w = block_width(F, st.k), e = extra_rows(F, w);
  const int p = st.p_cur[q], nd = st.ndiag[q];
  const T* A = arena + F.off;
  const int ld = F.ld, tid = threadIdx.x;
  const C* blk = reinterpret_cast<const C*>(st.blk) + (int64_t)q * BW * LDB;
  for (int idx = tid; idx < BW * LDB; idx += blockDim.x) (&L[0][0])[idx] = blk[idx];
  if (tid < 2 * BW) dv[tid] = st.bdinv[q * 2 * BW + tid];
  if (tid < BW) perm[tid] = st.lperm[q * BW + tid];
  if (tid == 0) fail = nd;
  __syncthreads();
  const BelowRows br{p + w, F.n, e, F.m};
  const int nrow = br.count();
  const double lim = 1.0 / st.u;
  T* pan = scratch + F.pan_off;
  for (int t0 = c.local * LDLT_RT; t0 < nrow; t0 += c.count * LDLT_RT) {
    const int ci = t0 + tid;
    if (ci < nrow) {
      const int r = br.row(ci);
      for (int k = 0; k < nd; ++k) xs[k][tid] = (C)A[(int64_t)(p + perm[k]) * ld + r];
      // x L^T = a  (unit lower L)
      for (int j = 0; j < nd; ++j) {
        const C xj = xs[j][tid];
        for (int k = j + 1; k < nd; ++k) xs[k][tid] = fma_(-xj, L[j][k], xs[k][tid]);
      }
      C x[BW];
#pragma unroll
      for (int k = 0; k < BW; ++k) x[k] = (k < nd) ? xs[k][tid] : C(0);
      apply_dinv(x, dv, nd, st.small);
      int first = nd;
#pragma unroll
      for (int k = BW - 1; k >= 0; --k)
        if (k < nd && fabs((double)x[k]) > lim) first = k;
      if (first < nd) atomicMin(&fail, first);
#pragma unroll
      for (int k = 0; k < BW; ++k)
        if (k < nd) pan[(int64_t)k * F.m + r] = (T)x[k];
    }
  }
  __syncthreads();
  if (tid == 0 && fail < nd) atomicMin(&st.npass_raw[q], fail);
}

// ---------------------------------------------------------------------------
// Commit over rows [p, m): passed columns get L (and L*D of the rows from
// p + npass on, for the trailing update), failed columns get back their
// values from before the step in the block's symmetric order (the front
// itself is the backup: nothing before the commit writes it in the block's
// columns).  The CTA with local index 0 stores D and the state.
template <typename T>
__global__ void __launch_bounds__(LDLT_RT) k_app_commit(T* __restrict__ arena,
                                                       T* __restrict__ scratch,
                                                       const LdltFront* __restrict__ fr,
                                                       const CtaMap* __restrict__ cm,
                                                       LdltStep st) {
  using C = T;
  __shared__ C L[BW][LDB];
  __shared__ double dv[2 * BW];
  __shared__ int perm[BW];
  __shared__ C orig[BW][LDLT_RT + 1];
  const CtaMap c = cm[blockIdx.x];
  const LdltFront F = fr[c.f];
  const int q = F.fidx, w = block_width(F, st.k);
  const int p = st.p_cur[q], nd = st.ndiag[q];
  T* A = arena + F.off;
  const int ld = F.ld, tid = threadIdx.x;
  const C* blk = reinterpret_cast<const C*>(st.blk) + (int64_t)q * BW * LDB;
  for (int idx = tid; idx < BW * LDB; idx += blockDim.x) (&L[0][0])[idx] = blk[idx];
  if (tid < 2 * BW) dv[tid] = st.bdinv[q * 2 * BW + tid];
  if (tid < BW) perm[tid] = st.lperm[q * BW + tid];
  __syncthreads();
  // Column::adjust: drop the first half of a 2x2 pivot split by the test
  int np = min(st.npass_raw[q], nd);
  if (np > 0 && isfinite(dv[2 * (np - 1)]) && dv[2 * (np - 1) + 1] != 0.0) np--;
  const T* pan = scratch + F.pan_off;
  T* ldp = scratch + F.ldp_off;
  const int ldp_ = F.m;
  for (int t0 = p + c.local * LDLT_RT; t0 < F.m; t0 += c.count * LDLT_RT) {
    const int r = t0 + tid;
    const bool in_blk = r < p + w;
    const int i = r - p;
    // phase 1: the values failed columns keep (in-block rows all belong to
    // the tile that starts at p, so no other CTA writes what this one reads)
    if (r < F.m) {
      for (int k = np; k < w; ++k) {
        C v = C(0);
        if (in_blk) {
          if (i >= k) {
            int ai = perm[i], ak = perm[k];
            int rr = max(ai, ak), cc = min(ai, ak);
            v = (C)A[(int64_t)(p + cc) * ld + p + rr];
          }
        } else {
          v = (C)A[(int64_t)(p + perm[k]) * ld + r];
        }
        orig[k][tid] = v;
      }
    }
    __syncthreads();
    if (r < F.m) {
      C l[BW];
#pragma unroll
      for (int k = 0; k < BW; ++k) {
        C v = C(0);
        if (k < np) {
          if (in_blk) v = (i > k) ? L[k][i] : (i == k ? C(1) : C(0));
          else v = (C)pan[(int64_t)k * ldp_ + r];
        }
        l[k] = v;
      }
      for (int k = 0; k < w; ++k) {
        if (in_blk && i < k) continue;
        C v = (k < np) ? l[k] : orig[k][tid];
        A[(int64_t)(p + k) * ld + r] = (T)v;
      }
      if (r >= p + np) {
        for (int k = 0; k < np;) {
          if (k + 1 < np && isinf(dv[2 * k + 2])) {
            const double a = dv[2 * k], b = dv[2 * k + 1], cc = dv[2 * k + 3];
            const double det = __dsub_rn(mul_(a, cc), mul_(b, b));
            const double d11 = cc / det, d21 = -b / det, d22 = a / det;
            const double l0 = l[k], l1 = l[k + 1];
            ldp[(int64_t)k * ldp_ + r] = (T)fma_(l0, d11, mul_(l1, d21));
            ldp[(int64_t)(k + 1) * ldp_ + r] = (T)fma_(l0, d21, mul_(l1, d22));
            k += 2;
          } else {
            const double d = dv[2 * k];
            ldp[(int64_t)k * ldp_ + r] = (T)((d == 0.0) ? C(0) : l[k] / (C)d);
            k += 1;
          }
        }
      }
    }
    __syncthreads();
  }
  if (c.local == 0) {
    if (tid < 2 * np) st.dall[F.d_off + 2 * p + tid] = dv[tid];
    if (tid == 0) {
      const int nf = st.nf_cur[q];
      st.npass[q] = np;
      st.p_next[q] = p + np;
      st.nf_next[q] = nf + (w - np);
      if (st.k == F.nblk - 1) st.p_final[q] = p + np;
    }
  }
}

// ---------------------------------------------------------------------------
// Move the f = w - npass failed columns of step k (now at [a, a + f),
// a = p + npass) behind the others: positions [a, n) take the variables in
// the order [a + f, n) then [a, a + f).  Copy rows [a, m) of columns [0, n)
// (lower part) and the variable list out, then write them back permuted.
__device__ __forceinline__ int moved_from(int i, int a, int n, int f) {
  return i < n - f ? i + f : a + (i - (n - f));
}

template <typename T>
__global__ void __launch_bounds__(256) k_app_move_copy(const T* __restrict__ arena,
                                                       T* __restrict__ scratch,
                                                       const LdltFront* __restrict__ fr,
                                                       const CtaMap* __restrict__ cm,
                                                       LdltStep st) {
  const CtaMap c = cm[blockIdx.x];
  const LdltFront F = fr[c.f];
  const int q = F.fidx, w = block_width(F, st.k), np = st.npass[q], f = w - np;
  if (f == 0) return;
  const int a = st.p_cur[q] + np, n = F.n, m = F.m, mm = m - a;
  const T* A = arena + F.off;
  T* mv = scratch + F.mv_off;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int col = c.local * 8 + warp; col < n; col += c.count * 8)
    for (int r = max(a, col) + lane; r < m; r += 32)
      mv[(int64_t)col * mm + (r - a)] = A[(int64_t)col * F.ld + r];
  if (c.local == 0)
    for (int i = a + threadIdx.x; i < n; i += blockDim.x)
      st.mvvar[F.mvvar_off + i] = st.var[F.var_off + i];
}

template <typename T>
__global__ void __launch_bounds__(256) k_app_move_write(T* __restrict__ arena,
                                                        const T* __restrict__ scratch,
                                                        const LdltFront* __restrict__ fr,
                                                        const CtaMap* __restrict__ cm,
                                                        LdltStep st) {
  const CtaMap c = cm[blockIdx.x];
  const LdltFront F = fr[c.f];
  const int q = F.fidx, w = block_width(F, st.k), np = st.npass[q], f = w - np;
  if (f == 0) return;
  const int a = st.p_cur[q] + np, n = F.n, m = F.m, mm = m - a;
  T* A = arena + F.off;
  const T* mv = scratch + F.mv_off;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int col = c.local * 8 + warp; col < n; col += c.count * 8) {
    if (col < a) {
      // eliminated column: permute its rows [a, n)
      for (int r = a + lane; r < n; r += 32)
        A[(int64_t)col * F.ld + r] = mv[(int64_t)col * mm + (moved_from(r, a, n, f) - a)];
    } else {
      const int oc = moved_from(col, a, n, f);
      for (int r = col + lane; r < m; r += 32) {
        T v;
        if (r < n) {
          const int orr = moved_from(r, a, n, f);
          const int hi = max(orr, oc), lo = min(orr, oc);
          v = mv[(int64_t)lo * mm + (hi - a)];
        } else {
          v = mv[(int64_t)oc * mm + (r - a)];
        }
        A[(int64_t)col * F.ld + r] = v;
      }
    }
  }
  if (c.local == 0)
    for (int i = a + threadIdx.x; i < n; i += blockDim.x)
      st.var[F.var_off + i] = st.mvvar[F.mvvar_off + moved_from(i, a, n, f)];
}

// ---------------------------------------------------------------------------
// Trailing update of step k: rows [o, m) x columns [o, n), o = p + npass,
// lower part, C -= (L D) L^T over the npass passed columns.  Lower-triangular
// tile space enumerated column by column; CTAs stride over it.
template <typename T, int TM, int KT>
__global__ void __launch_bounds__(256) k_app_update(T* __restrict__ arena,
                                                    const T* __restrict__ scratch,
                                                    const LdltFront* __restrict__ fr,
                                                    const CtaMap* __restrict__ cm,
                                                    LdltStep st) {
  __shared__ __align__(16) T As[2][KT][TM];
  __shared__ __align__(16) T Bs[2][KT][TM];
  const CtaMap c = cm[blockIdx.x];
  const LdltFront F = fr[c.f];
  const int q = F.fidx, p = st.p_cur[q], np = st.npass[q];
  if (np == 0) return;
  const int o = p + np;
  if (o >= F.n) return;
  const int R = (F.m - o + TM - 1) / TM, C = (F.n - o + TM - 1) / TM;
  const int total = C * R - C * (C - 1) / 2;
  T* front = arena + F.off;
  for (int t = c.local; t < total; t += c.count) {
    int cj = 0, rem = t;
    while (rem >= R - cj) { rem -= R - cj; ++cj; }
    const int ri = cj + rem;
    tile_update_body<T, TM, TM, KT>(front, F.ld, scratch + F.ldp_off, F.m,
                                    front + (int64_t)p * F.ld, F.ld, o + ri * TM, o + cj * TM,
                                    F.m, F.n, 0, np, As, Bs);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Threshold partial pivoting over columns [pstart, n), one CTA per front,
// right-looking updates restricted to the candidate columns (all rows).
template <typename T>
__global__ void __launch_bounds__(256) k_ldlt_tpp(T* __restrict__ arena,
                                                  const LdltFront* __restrict__ fr,
                                                  LdltStep st, double u,
                                                  const int* __restrict__ pstart,
                                                  int* __restrict__ out_nelim) {
  const LdltFront F = fr[blockIdx.x];
  T* A = arena + F.off;
  const int ld = F.ld, m = F.m, n = F.n;
  int* var = st.var + F.var_off;
  double* D = st.dall + F.d_off;
  const int tid = threadIdx.x, nt = blockDim.x;
  __shared__ double rv[8];
  __shared__ int ri[8];
  auto at = [&](int r, int c) -> T& { return A[(int64_t)c * ld + r]; };
  auto sym = [&](int r, int c) -> double { return r >= c ? (double)at(r, c) : (double)at(c, r); };
  auto swap_xy = [&](int x, int y) {
    if (x == y) return;
    if (x > y) { int t = x; x = y; y = t; }
    for (int k = tid; k < m; k += nt) {
      if (k < x) { T t = at(x, k); at(x, k) = at(y, k); at(y, k) = t; }
      else if (k == x) { T t = at(x, x); at(x, x) = at(y, y); at(y, y) = t; }
      else if (k < y) { T t = at(k, x); at(k, x) = at(y, k); at(y, k) = t; }
      else if (k > y) { T t = at(k, x); at(k, x) = at(k, y); at(k, y) = t; }
    }
    if (tid == 0) { int t = var[x]; var[x] = var[y]; var[y] = t; }
    __syncthreads();
  };
  // block max of |col c| over rows [lo, m) excluding ex1, ex2 (first maximum)
  auto colmax = [&](int c, int lo, int ex1, int ex2, int& arg) -> double {
    double b = -1.0;
    int bi = -1;
    for (int r = lo + tid; r < m; r += nt) {
      if (r == ex1 || r == ex2) continue;
      double v = fabs(sym(r, c));
      if (v > b) { b = v; bi = r; }
    }
    warp_argmax(b, bi);
    if ((tid & 31) == 0) { rv[tid >> 5] = b; ri[tid >> 5] = bi; }
    __syncthreads();
    if (tid == 0) {
      for (int qq = 1; qq < nt / 32; ++qq)
        if (rv[qq] > rv[0] || (rv[qq] == rv[0] && ri[qq] >= 0 && (ri[0] < 0 || ri[qq] < ri[0]))) {
          rv[0] = rv[qq]; ri[0] = ri[qq];
        }
    }
    __syncthreads();
    double res = rv[0];
    arg = ri[0];
    __syncthreads();
    return fmax(res, 0.0);
  };
  const double lim = 1.0 / u;
  int ne = pstart[F.fidx];
  while (ne < n) {
    int decided = 0, piv = -1, tpiv = -1;
    for (int c = ne; c < n && !decided; ++c) {
      int t;
      double amax = colmax(c, ne, c, -1, t);
      double acc = fabs(sym(c, c));
      if (amax < st.small && acc < st.small) { decided = 3; piv = c; break; }
      if (acc >= mul_(u, amax)) { decided = 1; piv = c; break; }
      if (t >= 0 && t < n) {
        int dummy;
        double ap2 = colmax(c, ne, c, t, dummy);
        double at2 = colmax(t, ne, c, t, dummy);
        double a11 = sym(c, c), a22 = sym(t, t), a21 = sym(t, c);
        double det = __dsub_rn(mul_(a11, a22), mul_(a21, a21));
        if (fabs(det) > st.small && isfinite(det)) {
          double i11 = a22 / det, i12 = -a21 / det, i22 = a11 / det;
          if (fma_(fabs(i11), ap2, mul_(fabs(i12), at2)) <= lim &&
              fma_(fabs(i12), ap2, mul_(fabs(i22), at2)) <= lim) {
            decided = 2; piv = c; tpiv = t;
          }
        }
      }
    }
    if (!decided) break;
    if (decided == 3) {
      if (!st.action) {
        if (tid == 0) atomicOr(st.status, ST_SINGULAR);
        break;
      }
      swap_xy(ne, piv);
      for (int r = ne + tid; r < m; r += nt) at(r, ne) = T(r == ne ? 1 : 0);
      if (tid == 0) {
        D[2 * ne] = 0.0;
        D[2 * ne + 1] = 0.0;
        atomicOr(st.status, ST_ZERO_PIVOT);
      }
      __syncthreads();
      ne += 1;
    } else if (decided == 1) {
      swap_xy(ne, piv);
      const int k = ne;
      const double di = 1.0 / (double)at(k, k);
      const int wdt = n - k - 1;
      for (int e = tid; e < wdt * (m - k - 1); e += nt) {
        int j = k + 1 + e % wdt, rr = k + 1 + e / wdt;
        if (rr >= j)
          at(rr, j) = (T)fma_(-(double)at(rr, k), mul_((double)at(j, k), di), (double)at(rr, j));
      }
      __syncthreads();
      for (int rr = k + 1 + tid; rr < m; rr += nt) at(rr, k) = (T)mul_((double)at(rr, k), di);
      if (tid == 0) {
        at(k, k) = T(1);
        D[2 * k] = di;
        D[2 * k + 1] = 0.0;
      }
      __syncthreads();
      ne += 1;
    } else {
      const int k = ne;
      swap_xy(k, piv);
      swap_xy(k + 1, (tpiv == k) ? piv : tpiv);
      const double a11 = at(k, k), a21 = at(k + 1, k), a22 = at(k + 1, k + 1);
      const double det = __dsub_rn(mul_(a11, a22), mul_(a21, a21));
      const double i11 = a22 / det, i12 = -a21 / det, i22 = a11 / det;
      const int wdt = n - k - 2;
      for (int e = tid; wdt > 0 && e < wdt * (m - k - 2); e += nt) {
        int j = k + 2 + e % wdt, rr = k + 2 + e / wdt;
        if (rr >= j) {
          const double w1 = at(j, k), w2 = at(j, k + 1);
          const double l1 = fma_(i11, w1, mul_(i12, w2)), l2 = fma_(i12, w1, mul_(i22, w2));
          at(rr, j) = (T)fma_(-(double)at(rr, k + 1), l2,
                              fma_(-(double)at(rr, k), l1, (double)at(rr, j)));
        }
      }
      __syncthreads();
      for (int rr = k + 2 + tid; rr < m; rr += nt) {
        const double w1 = at(rr, k), w2 = at(rr, k + 1);
        at(rr, k) = (T)fma_(i11, w1, mul_(i12, w2));
        at(rr, k + 1) = (T)fma_(i12, w1, mul_(i22, w2));
      }
      if (tid == 0) {
        at(k, k) = T(1);
        at(k + 1, k) = T(0);
        at(k + 1, k + 1) = T(1);
        D[2 * k] = i11;
        D[2 * k + 1] = i12;
        D[2 * k + 2] = dinf();
        D[2 * k + 3] = i22;
      }
      __syncthreads();
      ne += 2;
    }
  }
  if (tid == 0) out_nelim[F.fidx] = ne;
}

// ---------------------------------------------------------------------------
// L*D of contribution rows [n, m) over columns [0, nelim) (F.p = nelim).
template <typename T>
__global__ void __launch_bounds__(LDLT_RT) k_ldlt_calc_ld(const T* __restrict__ arena,
                                                         T* __restrict__ scratch,
                                                         const LdltFront* __restrict__ fr,
                                                         const CtaMap* __restrict__ cm,
                                                         LdltStep st) {
  const CtaMap c = cm[blockIdx.x];
  const LdltFront F = fr[c.f];
  const T* A = arena + F.off;
  const double* D = st.dall + F.d_off;
  T* out = scratch + F.ldp_off;
  const int ne = F.p, ldo = F.m;
  for (int r = F.n + c.local * LDLT_RT + threadIdx.x; r < F.m; r += c.count * LDLT_RT) {
    for (int k = 0; k < ne;) {
      if (k + 1 < ne && isinf(D[2 * k + 2])) {
        const double a = D[2 * k], b = D[2 * k + 1], cc = D[2 * k + 3];
        const double det = __dsub_rn(mul_(a, cc), mul_(b, b));
        const double d11 = cc / det, d21 = -b / det, d22 = a / det;
        const double l1 = A[(int64_t)k * F.ld + r], l2 = A[(int64_t)(k + 1) * F.ld + r];
        out[(int64_t)k * ldo + r] = (T)fma_(l1, d11, mul_(l2, d21));
        out[(int64_t)(k + 1) * ldo + r] = (T)fma_(l1, d21, mul_(l2, d22));
        k += 2;
      } else {
        const double d = D[2 * k];
        const T l = A[(int64_t)k * F.ld + r];
        out[(int64_t)k * ldo + r] = (d == 0.0) ? T(0) : l / (T)d;
        k += 1;
      }
    }
  }
}

template <typename ACC>
__global__ void k_solve_diag(const FrontDesc* __restrict__ fr, const int* __restrict__ var,
                             const double* __restrict__ dall, const int64_t* __restrict__ d_off,
                             ACC* __restrict__ x, int n, int nrhs) {
  const FrontDesc f = fr[blockIdx.x];
  const double* D = dall + d_off[blockIdx.x];
  const int* v = var + f.rl;
  const int ne = f.n;
  for (int e = threadIdx.x; e < ne * nrhs; e += blockDim.x) {
    int k = e % ne, r = e / ne;
    ACC* xr = x + (int64_t)r * n;
    bool second = k > 0 && isinf(D[2 * k]);  // (k-1, k) is a 2x2 pair
    if (second) continue;
    if (k + 1 < ne && isinf(D[2 * k + 2])) {
      double a = xr[v[k]], b = xr[v[k + 1]];
      xr[v[k]] = (ACC)fma_(D[2 * k], a, mul_(D[2 * k + 1], b));
      xr[v[k + 1]] = (ACC)fma_(D[2 * k + 1], a, mul_(D[2 * k + 3], b));
    } else {
      xr[v[k]] = (ACC)mul_(D[2 * k], (double)xr[v[k]]);
    }
  }
}

}  // namespace

template <typename T>
void launch_app_diag(T* arena, T* scratch, const LdltFront* fr, const CtaMap* cm, int ncta,
                     LdltStep st, cudaStream_t s) {
  if (ncta > 0) k_app_diag<T><<<ncta, 128, 0, s>>>(arena, scratch, fr, cm, st);
}
template <typename T>
void launch_app_apply(const T* arena, T* scratch, const LdltFront* fr, const CtaMap* cm, int ncta,
                      LdltStep st, cudaStream_t s) {
  if (ncta > 0) k_app_apply<T><<<ncta, LDLT_RT, 0, s>>>(arena, scratch, fr, cm, st);
}
template <typename T>
void launch_app_commit(T* arena, T* scratch, const LdltFront* fr, const CtaMap* cm, int ncta,
                       LdltStep st, cudaStream_t s) {
  if (ncta > 0) k_app_commit<T><<<ncta, LDLT_RT, 0, s>>>(arena, scratch, fr, cm, st);
}
template <typename T>
void launch_app_move(T* arena, T* scratch, const LdltFront* fr, const CtaMap* cm, int ncta,
                     LdltStep st, cudaStream_t s) {
  if (ncta <= 0) return;
  k_app_move_copy<T><<<ncta, 256, 0, s>>>(arena, scratch, fr, cm, st);
  k_app_move_write<T><<<ncta, 256, 0, s>>>(arena, scratch, fr, cm, st);
}
template <typename T>
void launch_app_update(T* arena, const T* scratch, const LdltFront* fr, const CtaMap* cm,
                       int ncta, LdltStep st, cudaStream_t s) {
  if (ncta > 0)
    k_app_update<T, Tiles<T>::TM, 16><<<ncta, 256, 0, s>>>(arena, scratch, fr, cm, st);
}
template <typename T>
void launch_ldlt_tpp(T* arena, const LdltFront* fr, int nf, LdltStep st, double u_eff,
                     const int* pstart, int* out_nelim, cudaStream_t s) {
  if (nf > 0) k_ldlt_tpp<T><<<nf, 256, 0, s>>>(arena, fr, st, u_eff, pstart, out_nelim);
}
template <typename T>
void launch_ldlt_calc_ld(const T* arena, T* scratch, const LdltFront* fr, const CtaMap* cm,
                         int ncta, LdltStep st, cudaStream_t s) {
  if (ncta > 0) k_ldlt_calc_ld<T><<<ncta, LDLT_RT, 0, s>>>(arena, scratch, fr, cm, st);
}
template <typename ACC>
void launch_solve_diag(const FrontDesc* fr, int nf, const int* var, const double* dall,
                       const int64_t* d_off, ACC* x, int n, int nrhs, cudaStream_t s) {
  if (nf > 0) k_solve_diag<ACC><<<nf, 256, 0, s>>>(fr, var, dall, d_off, x, n, nrhs);
}

#define SG_INST(T)                                                                            \
  template void launch_app_diag<T>(T*, T*, const LdltFront*, const CtaMap*, int, LdltStep,     \
                                   cudaStream_t);                                             \
  template void launch_app_apply<T>(const T*, T*, const LdltFront*, const CtaMap*, int,        \
                                    LdltStep, cudaStream_t);                                  \
  template void launch_app_commit<T>(T*, T*, const LdltFront*, const CtaMap*, int, LdltStep,   \
                                     cudaStream_t);                                           \
  template void launch_app_move<T>(T*, T*, const LdltFront*, const CtaMap*, int, LdltStep,     \
                                   cudaStream_t);                                             \
  template void launch_app_update<T>(T*, const T*, const LdltFront*, const CtaMap*, int,       \
                                     LdltStep, cudaStream_t);                                 \
  template void launch_ldlt_tpp<T>(T*, const LdltFront*, int, LdltStep, double, const int*,    \
                                   int*, cudaStream_t);                                       \
  template void launch_ldlt_calc_ld<T>(const T*, T*, const LdltFront*, const CtaMap*, int,     \
                                       LdltStep, cudaStream_t);                               \
  template void launch_solve_diag<T>(const FrontDesc*, int, const int*, const double*,         \
                                     const int64_t*, T*, int, int, cudaStream_t);
SG_INST(float)
SG_INST(double)
#undef SG_INST

}  // namespace sylver_gb300
