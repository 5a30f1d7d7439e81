// Threshold-pivoted LDL^T kernels (a posteriori pivoting by block column,
// threshold partial pivoting for what is left).  Pivot decisions, 2x2
// inversions and the acceptance test run in FP64 whatever the storage type.
//
// Reference behaviour replaced (math, not code):
//   Block::factor / block_ldlt<T,32>         src/kernels/ldlt_app.hxx:458-560
//   apply_pivot<OP_N> + check_threshold      src/kernels/ldlt_app.hxx:145-255
//   Column::adjust (split 2x2)               include/sylver/kernels/Column.hxx:87-101
//   restore_failed / CopyBackup              src/kernels/ldlt_app.hxx:405-431
//   calcLD + update / form_contrib           src/kernels/ldlt_app.hxx:619-751
//   factor_front_indef_failed (TPP pass)     src/factor_failed.hxx:29-157
// D^-1 uses the reference storage (src/kernels/ldlt_app.hxx:166-171):
// 1x1 [d^-1, 0], 2x2 [a, b, Inf, c] with (a b; b c) = D^-1, zero pivot [0, 0].
//
// Design: the diagonal block is factorised with complete pivoting by one
// warp in shared memory; its rows below are solved and tested in parallel
// (apply); the host reads the first failing column, drops a split 2x2, and the
// commit kernel writes L for the passed columns and restores the failed ones
// from the untouched front (the front itself is the backup: apply only writes
// scratch).  Failed columns start the next block column.
#include <cfloat>

#include "ldlt_dev.hpp"

namespace sylver_gb300 {

namespace {

constexpr int BW = LDLT_BW;
constexpr int LDB = BW + 1;

__device__ __forceinline__ bool is_two_first(const double* d, int k, int np) {
  return k + 1 < np && isinf(d[2 * k + 2]);
}

// ---------------------------------------------------------------------------
// Diagonal block: complete pivoting, 1x1 / 2x2, FP64, one warp.
template <typename T>
__global__ void __launch_bounds__(128) k_ldlt_diag(T* __restrict__ arena,
                                                   const LdltFront* __restrict__ fr,
                                                   LdltStep st) {
  __shared__ double a[BW][LDB];  // a[j][i] = A(i, j), lower part (i >= j) valid
  __shared__ double dv[2 * BW];
  __shared__ int perm[BW];
  const LdltFront F = fr[blockIdx.x];
  T* A = arena + F.off;
  const int ld = F.ld, p = F.p, w = F.w;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int idx = tid; idx < w * w; idx += blockDim.x) {
    int i = idx % w, j = idx / w;
    if (i >= j) a[j][i] = (double)A[(int64_t)(p + j) * ld + p + i];
  }
  if (tid < BW) perm[tid] = tid;
  if (tid < 2 * BW) dv[tid] = 0.0;
  __syncthreads();
  if (warp == 0) {
    // symmetric swap of x < y inside the block (lower storage)
    auto swap_xy = [&](int x, int y) {
      if (x == y) return;
      if (x > y) { int t = x; x = y; y = t; }
      int k = lane;
      if (k < w) {
        double t;
        if (k < x) { t = a[k][x]; a[k][x] = a[k][y]; a[k][y] = t; }
        else if (k == x) { t = a[x][x]; a[x][x] = a[y][y]; a[y][y] = t; }
        else if (k < y) { t = a[x][k]; a[x][k] = a[k][y]; a[k][y] = t; }
        else if (k > y) { t = a[x][k]; a[x][k] = a[y][k]; a[y][k] = t; }
      }
      if (lane == 0) { int t = perm[x]; perm[x] = perm[y]; perm[y] = t; }
      __syncwarp();
    };
    int s = 0;
    while (s < w) {
      // largest remaining entry (lower part, diagonal included)
      double best = -1.0;
      int bi = -1, bj = -1;
      if (lane >= s && lane < w)
        for (int i = lane; i < w; ++i) {
          double v = fabs(a[lane][i]);
          if (v > best) { best = v; bi = i; bj = lane; }
        }
      for (int o = 16; o > 0; o >>= 1) {
        double ob = __shfl_xor_sync(0xffffffffu, best, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        int oj = __shfl_xor_sync(0xffffffffu, bj, o);
        if (ob > best || (ob == best && (oj < bj || (oj == bj && oi < bi)))) {
          best = ob; bi = oi; bj = oj;
        }
      }
      const double amax = best;
      if (!(amax >= st.small)) {
        // the rest of the block is (numerically) zero: zero pivots
        for (int k = s + lane; k < w; k += 32) {
          for (int i = k; i < w; ++i) a[k][i] = (i == k) ? 1.0 : 0.0;
          dv[2 * k] = 0.0;
          dv[2 * k + 1] = 0.0;
        }
        if (lane == 0) atomicOr(st.status, st.action ? ST_ZERO_PIVOT : ST_SINGULAR);
        __syncwarp();
        break;
      }
      const int t = bi, q = bj;  // t >= q
      bool two = false;
      int piv = t;
      if (t != q) {
        double dt = fabs(a[t][t]), dq = fabs(a[q][q]);
        if (fmax(dt, dq) >= st.u * amax) piv = (dt >= dq) ? t : q;
        else two = true;
      }
      if (!two) {
        swap_xy(s, piv);
        const double di = 1.0 / a[s][s];
        // update trailing columns j > s (lane j), rows i >= j
        const int j = lane;
        if (j > s && j < w) {
          double lj = a[s][j] * di;
          for (int i = j; i < w; ++i) a[j][i] -= a[s][i] * lj;
        }
        __syncwarp();
        if (lane > s && lane < w) a[s][lane] *= di;
        if (lane == 0) {
          a[s][s] = 1.0;
          dv[2 * s] = di;
          dv[2 * s + 1] = 0.0;
        }
        __syncwarp();
        s += 1;
      } else {
        swap_xy(s, q);
        int t2 = (t == s) ? q : t;
        swap_xy(s + 1, t2);
        const double a11 = a[s][s], a21 = a[s][s + 1], a22 = a[s + 1][s + 1];
        const double det = a11 * a22 - a21 * a21;
        const double i11 = a22 / det, i12 = -a21 / det, i22 = a11 / det;
        const int j = lane;
        if (j > s + 1 && j < w) {
          double w1 = a[s][j], w2 = a[s + 1][j];
          double l1 = i11 * w1 + i12 * w2, l2 = i12 * w1 + i22 * w2;
          for (int i = j; i < w; ++i) a[j][i] -= a[s][i] * l1 + a[s + 1][i] * l2;
        }
        __syncwarp();
        if (lane > s + 1 && lane < w) {
          double w1 = a[s][lane], w2 = a[s + 1][lane];
          a[s][lane] = i11 * w1 + i12 * w2;
          a[s + 1][lane] = i12 * w1 + i22 * w2;
        }
        if (lane == 0) {
          a[s][s] = 1.0;
          a[s][s + 1] = 0.0;
          a[s + 1][s + 1] = 1.0;
          dv[2 * s] = i11;
          dv[2 * s + 1] = i12;
          dv[2 * s + 2] = __longlong_as_double(0x7ff0000000000000LL);  // +Inf marks 2x2
          dv[2 * s + 3] = i22;
        }
        __syncwarp();
        s += 2;
      }
    }
  }
  __syncthreads();
  double* blk = st.blk + (int64_t)F.fidx * BW * LDB;
  for (int idx = tid; idx < BW * LDB; idx += blockDim.x) blk[idx] = (&a[0][0])[idx];
  if (tid < 2 * BW) st.bdinv[F.fidx * 2 * BW + tid] = dv[tid];
  if (tid < BW) st.lperm[F.fidx * BW + tid] = perm[tid];
  // apply the block permutation to the rows of the already-eliminated
  // columns [0, p) and to the variable list
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

// apply D^-1 to a row of the solved block (reference apply_pivot OP_N)
__device__ __forceinline__ void apply_dinv(double* x, const double* dv, int w, double small) {
  for (int k = 0; k < w;) {
    if (k + 1 < w && isinf(dv[2 * k + 2])) {
      double x1 = x[k], x2 = x[k + 1];
      x[k] = dv[2 * k] * x1 + dv[2 * k + 1] * x2;
      x[k + 1] = dv[2 * k + 1] * x1 + dv[2 * k + 3] * x2;
      k += 2;
    } else {
      double d = dv[2 * k];
      if (d == 0.0) {
        double v = x[k];
        x[k] = (fabs(v) < small) ? 0.0 : __longlong_as_double(0x7ff0000000000000LL) * v;
      } else {
        x[k] *= d;
      }
      k += 1;
    }
  }
}

// ---------------------------------------------------------------------------
// Rows below the diagonal block: L = A P L_kk^-T D^-1, threshold test.
template <typename T>
__global__ void __launch_bounds__(LDLT_RT) k_ldlt_apply(const T* __restrict__ arena,
                                                       T* __restrict__ scratch,
                                                       const LdltFront* __restrict__ fr,
                                                       const RowTask* __restrict__ tasks,
                                                       LdltStep st) {
  __shared__ double L[BW][LDB];
  __shared__ double dv[2 * BW];
  __shared__ int perm[BW];
  __shared__ double xs[BW][LDLT_RT + 1];
  __shared__ int fail;
  const RowTask tk = tasks[blockIdx.x];
  const LdltFront F = fr[tk.f];
  const T* A = arena + F.off;
  const int ld = F.ld, p = F.p, w = F.w, tid = threadIdx.x;
  const double* blk = st.blk + (int64_t)F.fidx * BW * LDB;
  for (int idx = tid; idx < BW * LDB; idx += blockDim.x) (&L[0][0])[idx] = blk[idx];
  if (tid < 2 * BW) dv[tid] = st.bdinv[F.fidx * 2 * BW + tid];
  if (tid < BW) perm[tid] = st.lperm[F.fidx * BW + tid];
  if (tid == 0) fail = w;
  __syncthreads();
  const int r = tk.r0 + tid;
  if (r < F.m) {
    for (int k = 0; k < w; ++k) xs[k][tid] = (double)A[(int64_t)(p + perm[k]) * ld + r];
    // x L^T = a  (unit lower L)
    for (int j = 0; j < w; ++j) {
      double xj = xs[j][tid];
      for (int k = j + 1; k < w; ++k) xs[k][tid] -= xj * L[j][k];
    }
    double x[BW];
#pragma unroll
    for (int k = 0; k < BW; ++k) x[k] = (k < w) ? xs[k][tid] : 0.0;
    apply_dinv(x, dv, w, st.small);
    int first = w;
    const double lim = 1.0 / st.u;
#pragma unroll
    for (int k = BW - 1; k >= 0; --k)
      if (k < w && !(fabs(x[k]) <= lim)) first = k;
    if (first < w) atomicMin(&fail, first);
    T* pan = scratch + F.pan_off;
    const int ldp = F.m;
#pragma unroll
    for (int k = 0; k < BW; ++k)
      if (k < w) pan[(int64_t)k * ldp + r] = (T)x[k];
  }
  __syncthreads();
  if (tid == 0 && fail < w) atomicMin(&st.npass_raw[F.fidx], fail);
}

// ---------------------------------------------------------------------------
// Commit: passed columns get L (and L*D into the update panel), failed
// columns get the original values in the new symmetric order.
template <typename T>
__global__ void __launch_bounds__(LDLT_RT) k_ldlt_commit(T* __restrict__ arena,
                                                        T* __restrict__ scratch,
                                                        const LdltFront* __restrict__ fr,
                                                        const RowTask* __restrict__ tasks,
                                                        LdltStep st) {
  __shared__ double L[BW][LDB];
  __shared__ double dv[2 * BW];
  __shared__ int perm[BW];
  __shared__ double orig[BW][LDLT_RT + 1];
  const RowTask tk = tasks[blockIdx.x];
  const LdltFront F = fr[tk.f];
  T* A = arena + F.off;
  const int ld = F.ld, p = F.p, w = F.w, tid = threadIdx.x;
  const int np = st.npass[F.fidx];
  const double* blk = st.blk + (int64_t)F.fidx * BW * LDB;
  for (int idx = tid; idx < BW * LDB; idx += blockDim.x) (&L[0][0])[idx] = blk[idx];
  if (tid < 2 * BW) dv[tid] = st.bdinv[F.fidx * 2 * BW + tid];
  if (tid < BW) perm[tid] = st.lperm[F.fidx * BW + tid];
  __syncthreads();
  const int r = tk.r0 + tid;
  const bool in_blk = r < p + w;
  const int i = r - p;
  const T* pan = scratch + F.pan_off;
  const int ldp = F.m;
  // phase 1: read the original (pre-step) values that failed columns keep
  if (r < F.m) {
    for (int k = np; k < w; ++k) {
      double v = 0.0;
      if (in_blk) {
        if (i >= k) {
          int ai = perm[i], ak = perm[k];
          int rr = max(ai, ak), cc = min(ai, ak);
          v = (double)A[(int64_t)(p + cc) * ld + p + rr];
        }
      } else {
        v = (double)A[(int64_t)(p + perm[k]) * ld + r];
      }
      orig[k][tid] = v;
    }
  }
  __syncthreads();
  if (r < F.m) {
    double l[BW];
#pragma unroll
    for (int k = 0; k < BW; ++k) {
      double v = 0.0;
      if (k < np) {
        if (in_blk) v = (i > k) ? L[k][i] : (i == k ? 1.0 : 0.0);
        else v = (double)pan[(int64_t)k * ldp + r];
      }
      l[k] = v;
    }
    for (int k = 0; k < w; ++k) {
      if (in_blk && i < k) continue;
      double v = (k < np) ? l[k] : orig[k][tid];
      A[(int64_t)(p + k) * ld + r] = (T)v;
    }
    // L*D of the passed columns for the trailing update
    T* ldp_ = scratch + F.ldp_off;
    for (int k = 0; k < np;) {
      if (is_two_first(dv, k, np)) {
        double a = dv[2 * k], b = dv[2 * k + 1], c = dv[2 * k + 3];
        double det = a * c - b * b;
        double d11 = c / det, d21 = -b / det, d22 = a / det;
        ldp_[(int64_t)k * ldp + r] = (T)(l[k] * d11 + l[k + 1] * d21);
        ldp_[(int64_t)(k + 1) * ldp + r] = (T)(l[k] * d21 + l[k + 1] * d22);
        k += 2;
      } else {
        double d = dv[2 * k];
        ldp_[(int64_t)k * ldp + r] = (T)((d == 0.0) ? 0.0 : l[k] / d);
        k += 1;
      }
    }
  }
  if (tk.r0 == p && tid < 2 * np) st.dall[F.d_off + 2 * p + tid] = dv[tid];
}

// ---------------------------------------------------------------------------
// Threshold partial pivoting over columns [p, n), one CTA per front,
// right-looking updates restricted to the candidate columns (all rows).
template <typename T>
__global__ void __launch_bounds__(256) k_ldlt_tpp(T* __restrict__ arena,
                                                  const LdltFront* __restrict__ fr,
                                                  LdltStep st, double u,
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
  // block max of |col c| over rows [lo, m) excluding ex1, ex2
  auto colmax = [&](int c, int lo, int ex1, int ex2, int& arg) -> double {
    double b = -1.0;
    int bi = -1;
    for (int r = lo + tid; r < m; r += nt) {
      if (r == ex1 || r == ex2) continue;
      double v = fabs(sym(r, c));
      if (v > b) { b = v; bi = r; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      double ob = __shfl_xor_sync(0xffffffffu, b, o);
      int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > b || (ob == b && oi >= 0 && (bi < 0 || oi < bi))) { b = ob; bi = oi; }
    }
    if ((tid & 31) == 0) { rv[tid >> 5] = b; ri[tid >> 5] = bi; }
    __syncthreads();
    if (tid == 0) {
      for (int q = 1; q < nt / 32; ++q)
        if (rv[q] > rv[0] || (rv[q] == rv[0] && ri[q] >= 0 && (ri[0] < 0 || ri[q] < ri[0]))) {
          rv[0] = rv[q]; ri[0] = ri[q];
        }
    }
    __syncthreads();
    double res = rv[0];
    arg = ri[0];
    __syncthreads();
    return fmax(res, 0.0);
  };
  int ne = F.p;
  while (ne < n) {
    int decided = 0, piv = -1, tpiv = -1;
    for (int c = ne; c < n && !decided; ++c) {
      int t;
      double amax = colmax(c, ne, c, -1, t);
      double acc = fabs(sym(c, c));
      if (amax < st.small && acc < st.small) { decided = 3; piv = c; break; }
      if (acc >= u * amax) { decided = 1; piv = c; break; }
      if (t >= 0 && t < n) {
        int dummy;
        double ap2 = colmax(c, ne, c, t, dummy);
        double at2 = colmax(t, ne, c, t, dummy);
        double a11 = sym(c, c), a22 = sym(t, t), a21 = sym(t, c);
        double det = a11 * a22 - a21 * a21;
        if (fabs(det) > st.small && isfinite(det)) {
          double i11 = a22 / det, i12 = -a21 / det, i22 = a11 / det;
          if (fabs(i11) * ap2 + fabs(i12) * at2 <= 1.0 / u &&
              fabs(i12) * ap2 + fabs(i22) * at2 <= 1.0 / u) {
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
        if (rr >= j) at(rr, j) = (T)((double)at(rr, j) - (double)at(rr, k) * ((double)at(j, k) * di));
      }
      __syncthreads();
      for (int rr = k + 1 + tid; rr < m; rr += nt) at(rr, k) = (T)((double)at(rr, k) * di);
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
      int t2 = (tpiv == k) ? piv : tpiv;
      swap_xy(k + 1, t2);
      const double a11 = at(k, k), a21 = at(k + 1, k), a22 = at(k + 1, k + 1);
      const double det = a11 * a22 - a21 * a21;
      const double i11 = a22 / det, i12 = -a21 / det, i22 = a11 / det;
      const int wdt = n - k - 2;
      for (int e = tid; wdt > 0 && e < wdt * (m - k - 2); e += nt) {
        int j = k + 2 + e % wdt, rr = k + 2 + e / wdt;
        if (rr >= j) {
          double w1 = at(j, k), w2 = at(j, k + 1);
          double l1 = i11 * w1 + i12 * w2, l2 = i12 * w1 + i22 * w2;
          at(rr, j) = (T)((double)at(rr, j) - (double)at(rr, k) * l1 - (double)at(rr, k + 1) * l2);
        }
      }
      __syncthreads();
      for (int rr = k + 2 + tid; rr < m; rr += nt) {
        double w1 = at(rr, k), w2 = at(rr, k + 1);
        at(rr, k) = (T)(i11 * w1 + i12 * w2);
        at(rr, k + 1) = (T)(i12 * w1 + i22 * w2);
      }
      if (tid == 0) {
        at(k, k) = T(1);
        at(k + 1, k) = T(0);
        at(k + 1, k + 1) = T(1);
        D[2 * k] = i11;
        D[2 * k + 1] = i12;
        D[2 * k + 2] = __longlong_as_double(0x7ff0000000000000LL);
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
                                                         const RowTask* __restrict__ tasks,
                                                         LdltStep st) {
  const RowTask tk = tasks[blockIdx.x];
  const LdltFront F = fr[tk.f];
  const int r = tk.r0 + threadIdx.x;
  if (r >= F.m) return;
  const T* A = arena + F.off;
  const double* D = st.dall + F.d_off;
  T* out = scratch + F.ldp_off;
  const int ne = F.p, ldo = F.m, i = r;
  for (int k = 0; k < ne;) {
    if (k + 1 < ne && isinf(D[2 * k + 2])) {
      double a = D[2 * k], b = D[2 * k + 1], c = D[2 * k + 3];
      double det = a * c - b * b;
      double d11 = c / det, d21 = -b / det, d22 = a / det;
      double l1 = A[(int64_t)k * F.ld + r], l2 = A[(int64_t)(k + 1) * F.ld + r];
      out[(int64_t)k * ldo + i] = (T)(l1 * d11 + l2 * d21);
      out[(int64_t)(k + 1) * ldo + i] = (T)(l1 * d21 + l2 * d22);
      k += 2;
    } else {
      double d = D[2 * k];
      double l = A[(int64_t)k * F.ld + r];
      out[(int64_t)k * ldo + i] = (T)((d == 0.0) ? 0.0 : l / d);
      k += 1;
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
    bool second = k > 0 && isinf(D[2 * k]) ;  // (k-1, k) is a 2x2 pair
    if (second) continue;
    if (k + 1 < ne && isinf(D[2 * k + 2])) {
      double a = xr[v[k]], b = xr[v[k + 1]];
      xr[v[k]] = (ACC)(D[2 * k] * a + D[2 * k + 1] * b);
      xr[v[k + 1]] = (ACC)(D[2 * k + 1] * a + D[2 * k + 3] * b);
    } else {
      xr[v[k]] = (ACC)(D[2 * k] * (double)xr[v[k]]);
    }
  }
}

}  // namespace

template <typename T>
void launch_ldlt_diag(T* arena, const LdltFront* fr, int nf, LdltStep st, cudaStream_t s) {
  if (nf > 0) k_ldlt_diag<T><<<nf, 128, 0, s>>>(arena, fr, st);
}
template <typename T>
void launch_ldlt_apply(const T* arena, T* scratch, const LdltFront* fr, const RowTask* rt,
                       int nt, LdltStep st, cudaStream_t s) {
  if (nt > 0) k_ldlt_apply<T><<<nt, LDLT_RT, 0, s>>>(arena, scratch, fr, rt, st);
}
template <typename T>
void launch_ldlt_commit(T* arena, T* scratch, const LdltFront* fr, const RowTask* rt, int nt,
                        LdltStep st, cudaStream_t s) {
  if (nt > 0) k_ldlt_commit<T><<<nt, LDLT_RT, 0, s>>>(arena, scratch, fr, rt, st);
}
template <typename T>
void launch_ldlt_tpp(T* arena, const LdltFront* fr, int nf, LdltStep st, double u_eff,
                     int* out_nelim, cudaStream_t s) {
  if (nf > 0) k_ldlt_tpp<T><<<nf, 256, 0, s>>>(arena, fr, st, u_eff, out_nelim);
}
template <typename T>
void launch_ldlt_calc_ld(const T* arena, T* scratch, const LdltFront* fr, const RowTask* rt,
                         int nt, LdltStep st, cudaStream_t s) {
  if (nt > 0) k_ldlt_calc_ld<T><<<nt, LDLT_RT, 0, s>>>(arena, scratch, fr, rt, st);
}
template <typename ACC>
void launch_solve_diag(const FrontDesc* fr, int nf, const int* var, const double* dall,
                       const int64_t* d_off, ACC* x, int n, int nrhs, cudaStream_t s) {
  if (nf > 0) k_solve_diag<ACC><<<nf, 256, 0, s>>>(fr, var, dall, d_off, x, n, nrhs);
}

#define SG_INST(T)                                                                          \
  template void launch_ldlt_diag<T>(T*, const LdltFront*, int, LdltStep, cudaStream_t);      \
  template void launch_ldlt_apply<T>(const T*, T*, const LdltFront*, const RowTask*, int,    \
                                     LdltStep, cudaStream_t);                               \
  template void launch_ldlt_commit<T>(T*, T*, const LdltFront*, const RowTask*, int, LdltStep, \
                                      cudaStream_t);                                        \
  template void launch_ldlt_tpp<T>(T*, const LdltFront*, int, LdltStep, double, int*,        \
                                   cudaStream_t);                                           \
  template void launch_ldlt_calc_ld<T>(const T*, T*, const LdltFront*, const RowTask*, int,  \
                                       LdltStep, cudaStream_t);                             \
  template void launch_solve_diag<T>(const FrontDesc*, int, const int*, const double*,       \
                                     const int64_t*, T*, int, int, cudaStream_t);
SG_INST(float)
SG_INST(double)
#undef SG_INST

}  // namespace sylver_gb300
