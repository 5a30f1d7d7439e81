// CPU FP64 multifrontal oracle -- TEST INFRASTRUCTURE ONLY.
//
// This file is the checker for the GPU factorize/solve path.  It is imported
// only by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
// leg; the product never links or calls it.
//
// It restates, in plain C++ over BLAS, the reference's numeric phase for one
// front at a time in postorder:
//   * front layout and delays: include/sylver/NumericFrontBase.hxx:107-124,
//     src/NumericFront.hxx:73-145 (m = symb.nrow + ndelay_in,
//     n = symb.ncol + ndelay_in, delayed columns placed after the front's own
//     fully-summed columns, src/kernels/assemble.hxx:926-986);
//   * init from the A->front map: src/kernels/assemble.hxx:162-214;
//   * extend-add of child contribution blocks: src/kernels/assemble.hxx:231-286,
//     :344-425 (done before the factorization here; the sum is the same);
//   * posdef: potrf / trsm / syrk into the contribution block
//     (src/tasks/tasks.hxx:276-289, :338, :392-395, :443-448), not-posdef
//     -> flag -6;
//   * indefinite: the reference's a-posteriori pivoting (APP) with block
//     size 32 and one level of blocking (block_size == INNER_BLOCK_SIZE):
//     block-column loop src/factor_indef.hxx:1338-1474; Block::factor with
//     block_ldlt (complete pivoting) on a full 32x32 diagonal block and
//     ldlt_tpp_factor on a partial one (src/kernels/ldlt_app.hxx:458-560);
//     apply_pivot + check_threshold (:145-255, :579-601); Column::adjust
//     (include/sylver/kernels/Column.hxx:87-101); restore of failed columns
//     (src/kernels/ldlt_app.hxx:405-431); updates with calcLD (:619-718);
//     permute_failed (src/factor_indef.hxx:1190-1288); then threshold
//     partial pivoting on the failed columns and delays
//     (src/factor_failed.hxx:29-157), and form_contrib
//     (src/kernels/factor_indef.hxx:251-342).  D is stored inverted in the
//     reference's format (src/kernels/ldlt_app.hxx:166-171);
//   * inertia and 2x2 statistics: src/NumericTree.hxx:143-178;
//   * solves: src/NumericTreePosdef.hxx:357-450 and src/NumericTree.hxx:408-520
//     with the permute/scale wrapper src/spldlt_factorize_mod.F90:901-1060.
//
// SPRAL's block_ldlt and ldlt_tpp_factor are not vendored (empty spral/
// submodule); the pivot searches below follow the published algorithms
// (Duff, Hogg & Lopez, SISC 2020: complete pivoting with a 1x1 / 2x2 choice
// on a full block; TPP with the 1x1 test |a_pp| >= u * max_i |a_ip| and the
// 2x2 test |D^-1| [max_p; max_t] <= 1/u), not SPRAL's source.
//
// Fixed arithmetic order (LDL^T).  Where the reference leaves the order to
// BLAS, this restatement fixes it, and the GPU kernels use the same order:
// every multiply-add below is std::fma (or a separate multiply and add where
// written so), sums run in increasing k, contributions of children are added
// in increasing child index, and an update subtracts its accumulated sum
// once (acc = 0; acc = fma(LD_ik, L_jk, acc) for k = 0, 1, ...; a_ij -= acc).
// With correctly rounded IEEE arithmetic on both sides, the FP64 GPU factors
// then equal these bit for bit, pivot decisions included.  The one layout
// difference: failed columns move behind the unprocessed ones as soon as
// their block is committed instead of staying in place until
// permute_failed; the blocks, the multipliers, the threshold tests and the
// final order are the reference's.
//
// Compiled with -ffp-contract=off.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

extern "C" {
typedef void (*dgemm_t)(const char*, const char*, const int*, const int*, const int*,
                        const double*, const double*, const int*, const double*, const int*,
                        const double*, double*, const int*);
typedef void (*dtrsm_t)(const char*, const char*, const char*, const char*, const int*,
                        const int*, const double*, const double*, const int*, double*,
                        const int*);
typedef void (*dsyrk_t)(const char*, const char*, const int*, const int*, const double*,
                        const double*, const int*, const double*, double*, const int*);
typedef void (*dpotrf_t)(const char*, const int*, double*, const int*, int*);
}

namespace {
dgemm_t g_dgemm = nullptr;
dtrsm_t g_dtrsm = nullptr;
dsyrk_t g_dsyrk = nullptr;
dpotrf_t g_dpotrf = nullptr;
bool g_inplace = false;  // LDL^T block steps in the reference's in-place layout

struct Front {
  int m = 0, n = 0;         // rows, fully-summed columns (incl. delays in)
  int nelim = 0;            // eliminated here
  int ndelay_in = 0;
  std::vector<double> a;    // m x m column-major (lower used)
  std::vector<double> d;    // 2*n, inverted D (indefinite)
  std::vector<int> var;     // front row -> pivot-order variable (0-based)
};

struct Oracle {
  bool posdef;
  int n, nnodes;
  std::vector<int> perm;    // variable -> pivot position (0-based)
  std::vector<Front> fronts;
  int flag = 0;
  int num_neg = 0, num_zero = 0, num_two = 0, num_delay = 0, maxfront = 0;
  int not_first_pass = 0, not_second_pass = 0;
  int zero_pivots = 0;
  int64_t num_factor = 0;
};

inline double& at(std::vector<double>& a, int ld, int i, int j) { return a[(size_t)j * ld + i]; }

// Symmetric swap of indices p < q in an m x m lower-stored matrix.
void sym_swap(std::vector<double>& a, int m, int p, int q) {
  if (p == q) return;
  if (p > q) std::swap(p, q);
  for (int k = 0; k < p; ++k) std::swap(at(a, m, p, k), at(a, m, q, k));
  std::swap(at(a, m, p, p), at(a, m, q, q));
  for (int i = p + 1; i < q; ++i) std::swap(at(a, m, i, p), at(a, m, q, i));
  for (int i = q + 1; i < m; ++i) std::swap(at(a, m, i, p), at(a, m, i, q));
}

constexpr double kRootU = 1e-300;  // relaxed threshold at roots (small-pivot test only)
constexpr int BW = 32;             // APP block size

// First maximum of |col c| over rows [lo, m) except ex1, ex2 (lower storage,
// symmetric access); arg = -1 and 0 returned when no row qualifies.
double colmax(const std::vector<double>& a, int m, int c, int lo, int ex1, int ex2, int& arg) {
  double b = -1.0;
  arg = -1;
  for (int r = lo; r < m; ++r) {
    if (r == ex1 || r == ex2) continue;
    double v = std::fabs(r >= c ? a[(size_t)c * m + r] : a[(size_t)r * m + c]);
    if (v > b) { b = v; arg = r; }
  }
  return std::max(b, 0.0);
}

// Threshold partial pivoting on candidate columns [start, ncand) of the
// m x m front, rows [start, m) (ldlt_tpp_factor); updates only the candidate
// columns (all rows).  Returns the number of eliminated columns (start +
// eliminated here), -1 on a zero pivot with action = false.  The eliminated
// columns hold L (unit diagonal) and d holds D^-1.
int tpp(Front& f, int start, int ncand, double u, double small, bool action, Oracle& o) {
  const int m = f.m;
  auto& a = f.a;
  auto A = [&](int i, int j) -> double& { return a[(size_t)j * m + i]; };
  auto sym = [&](int i, int j) -> double { return i >= j ? A(i, j) : A(j, i); };
  const double lim = 1.0 / u;
  int ne = start;
  while (ne < ncand) {
    int decided = 0, piv = -1, tpiv = -1;
    for (int c = ne; c < ncand && !decided; ++c) {
      int t;
      double amax = colmax(a, m, c, ne, c, -1, t);
      double acc = std::fabs(A(c, c));
      if (amax < small && acc < small) { decided = 3; piv = c; break; }
      if (acc >= u * amax) { decided = 1; piv = c; break; }
      if (t >= 0 && t < ncand) {
        int dummy;
        double ap2 = colmax(a, m, c, ne, c, t, dummy);
        double at2 = colmax(a, m, t, ne, c, t, dummy);
        double a11 = A(c, c), a22 = A(t, t), a21 = sym(t, c);
        double det = a11 * a22 - a21 * a21;
        if (std::fabs(det) > small && std::isfinite(det)) {
          double i11 = a22 / det, i12 = -a21 / det, i22 = a11 / det;
          if (std::fma(std::fabs(i11), ap2, std::fabs(i12) * at2) <= lim &&
              std::fma(std::fabs(i12), ap2, std::fabs(i22) * at2) <= lim) {
            decided = 2; piv = c; tpiv = t;
          }
        }
      }
    }
    if (!decided) break;
    if (decided == 3) {
      if (!action) { o.flag = -5; return -1; }
      sym_swap(a, m, ne, piv);
      std::swap(f.var[ne], f.var[piv]);
      for (int r = ne; r < m; ++r) A(r, ne) = (r == ne) ? 1.0 : 0.0;
      f.d[2 * ne] = 0.0;
      f.d[2 * ne + 1] = 0.0;
      o.zero_pivots++;
      ne += 1;
    } else if (decided == 1) {
      sym_swap(a, m, ne, piv);
      std::swap(f.var[ne], f.var[piv]);
      const int k = ne;
      const double di = 1.0 / A(k, k);
      for (int j = k + 1; j < ncand; ++j) {
        const double lj = A(j, k) * di;
        for (int r = j; r < m; ++r) A(r, j) = std::fma(-A(r, k), lj, A(r, j));
      }
      for (int r = k + 1; r < m; ++r) A(r, k) = A(r, k) * di;
      A(k, k) = 1.0;
      f.d[2 * k] = di;
      f.d[2 * k + 1] = 0.0;
      ne += 1;
    } else {
      const int k = ne;
      sym_swap(a, m, k, piv);
      std::swap(f.var[k], f.var[piv]);
      const int t2 = (tpiv == k) ? piv : tpiv;
      sym_swap(a, m, k + 1, t2);
      std::swap(f.var[k + 1], f.var[t2]);
      const double a11 = A(k, k), a21 = A(k + 1, k), a22 = A(k + 1, k + 1);
      const double det = a11 * a22 - a21 * a21;
      const double i11 = a22 / det, i12 = -a21 / det, i22 = a11 / det;
      for (int j = k + 2; j < ncand; ++j) {
        const double w1 = A(j, k), w2 = A(j, k + 1);
        const double l1 = std::fma(i11, w1, i12 * w2), l2 = std::fma(i12, w1, i22 * w2);
        for (int r = j; r < m; ++r)
          A(r, j) = std::fma(-A(r, k + 1), l2, std::fma(-A(r, k), l1, A(r, j)));
      }
      for (int r = k + 2; r < m; ++r) {
        const double w1 = A(r, k), w2 = A(r, k + 1);
        A(r, k) = std::fma(i11, w1, i12 * w2);
        A(r, k + 1) = std::fma(i12, w1, i22 * w2);
      }
      A(k, k) = 1.0;
      A(k + 1, k) = 0.0;
      A(k + 1, k + 1) = 1.0;
      f.d[2 * k] = i11;
      f.d[2 * k + 1] = i12;
      f.d[2 * k + 2] = std::numeric_limits<double>::infinity();
      f.d[2 * k + 3] = i22;
      ne += 2;
    }
  }
  return ne;
}

// (L D) of one row from its L entries l[0..np) and D^-1 (calcLD): 1x1 l / d,
// 2x2 l * inverse(D^-1).
void calc_ld_row(const double* d, const double* l, int np, double* out) {
  for (int k = 0; k < np;) {
    if (k + 1 < np && std::isinf(d[2 * k + 2])) {
      const double a = d[2 * k], b = d[2 * k + 1], c = d[2 * k + 3];
      const double det = a * c - b * b;
      const double d11 = c / det, d21 = -b / det, d22 = a / det;
      out[k] = std::fma(l[k], d11, l[k + 1] * d21);
      out[k + 1] = std::fma(l[k], d21, l[k + 1] * d22);
      k += 2;
    } else {
      const double dk = d[2 * k];
      out[k] = (dk == 0.0) ? 0.0 : l[k] / dk;
      k += 1;
    }
  }
}

// The diagonal block of a block step: panel P[j][i] (i: panel row, j <
// w: candidate column; rows i < w are the block rows, rows w.. the extra
// contribution rows of a partial block).  Complete pivoting when w == BW,
// threshold partial pivoting otherwise.  Returns the pivots taken.
struct Panel {
  double a[BW][BW + 1];
  double dv[2 * BW];
  int perm[BW];
};

int diag_block(Panel& P, int w, int R, double u, double small, bool action, Oracle& o) {
  auto& a = P.a;
  for (int i = 0; i < BW; ++i) P.perm[i] = i;
  for (int i = 0; i < 2 * BW; ++i) P.dv[i] = 0.0;
  auto swap_xy = [&](int x, int y) {
    if (x == y) return;
    if (x > y) std::swap(x, y);
    for (int kk = 0; kk < R; ++kk) {
      if (kk < x) std::swap(a[kk][x], a[kk][y]);
      else if (kk == x) std::swap(a[x][x], a[y][y]);
      else if (kk < y) std::swap(a[x][kk], a[kk][y]);
      else if (kk > y) std::swap(a[x][kk], a[y][kk]);
    }
    std::swap(P.perm[x], P.perm[y]);
  };
  auto elim1 = [&](int s, int cend) {
    const double di = 1.0 / a[s][s];
    for (int j = s + 1; j < cend; ++j) {
      const double lj = a[s][j] * di;
      for (int i = j; i < R; ++i) a[j][i] = std::fma(-a[s][i], lj, a[j][i]);
    }
    for (int i = s + 1; i < R; ++i) a[s][i] = a[s][i] * di;
    a[s][s] = 1.0;
    P.dv[2 * s] = di;
    P.dv[2 * s + 1] = 0.0;
  };
  auto elim2 = [&](int s, int cend) {
    const double a11 = a[s][s], a21 = a[s][s + 1], a22 = a[s + 1][s + 1];
    const double det = a11 * a22 - a21 * a21;
    const double i11 = a22 / det, i12 = -a21 / det, i22 = a11 / det;
    for (int j = s + 2; j < cend; ++j) {
      const double w1 = a[s][j], w2 = a[s + 1][j];
      const double l1 = std::fma(i11, w1, i12 * w2), l2 = std::fma(i12, w1, i22 * w2);
      for (int i = j; i < R; ++i) a[j][i] = std::fma(-a[s + 1][i], l2, std::fma(-a[s][i], l1, a[j][i]));
    }
    for (int i = s + 2; i < R; ++i) {
      const double w1 = a[s][i], w2 = a[s + 1][i];
      a[s][i] = std::fma(i11, w1, i12 * w2);
      a[s + 1][i] = std::fma(i12, w1, i22 * w2);
    }
    a[s][s] = 1.0;
    a[s][s + 1] = 0.0;
    a[s + 1][s + 1] = 1.0;
    P.dv[2 * s] = i11;
    P.dv[2 * s + 1] = i12;
    P.dv[2 * s + 2] = std::numeric_limits<double>::infinity();
    P.dv[2 * s + 3] = i22;
  };
  int s = 0;
  if (w == BW) {
    // complete pivoting (block_ldlt): first maximum in (column, row) order
    while (s < w) {
      double best = -1.0;
      int bi = -1, bj = -1;
      for (int j = s; j < w; ++j)
        for (int i = j; i < w; ++i) {
          double v = std::fabs(a[j][i]);
          if (v > best) { best = v; bi = i; bj = j; }
        }
      const double amax = best;
      if (!(amax >= small)) {
        for (int kk = s; kk < w; ++kk) {
          for (int i = kk; i < w; ++i) a[kk][i] = (i == kk) ? 1.0 : 0.0;
          P.dv[2 * kk] = 0.0;
          P.dv[2 * kk + 1] = 0.0;
        }
        if (action) o.zero_pivots += w - s;
        else o.flag = -5;
        s = w;
        break;
      }
      const int t = bi, q = bj;
      bool two = false;
      int piv = t;
      if (t != q) {
        double dt = std::fabs(a[t][t]), dq = std::fabs(a[q][q]);
        if (std::max(dt, dq) >= u * amax) piv = (dt >= dq) ? t : q;
        else two = true;
      }
      if (!two) {
        swap_xy(s, piv);
        elim1(s, w);
        s += 1;
      } else {
        swap_xy(s, q);
        swap_xy(s + 1, (t == s) ? q : t);
        elim2(s, w);
        s += 2;
      }
    }
  } else {
    // threshold partial pivoting over the w candidates, rows [s, R)
    const double lim = 1.0 / u;
    auto colv = [&](int i, int col) { return i > col ? a[col][i] : a[i][col]; };
    auto cmax = [&](int col, int ex1, int ex2, int lo, int& arg) {
      double b = -1.0;
      arg = -1;
      for (int i = lo; i < R; ++i) {
        if (i == ex1 || i == ex2) continue;
        double v = std::fabs(colv(i, col));
        if (v > b) { b = v; arg = i; }
      }
      return std::max(b, 0.0);
    };
    while (s < w) {
      int decided = 0, piv = -1, tpiv = -1;
      for (int c = s; c < w && !decided; ++c) {
        int t;
        const double amax = cmax(c, c, -1, s, t);
        const double acc = std::fabs(a[c][c]);
        if (amax < small && acc < small) { decided = 3; piv = c; break; }
        if (acc >= u * amax) { decided = 1; piv = c; break; }
        if (t >= 0 && t < w) {
          int dummy;
          const double ap2 = cmax(c, c, t, s, dummy), at2 = cmax(t, c, t, s, dummy);
          const double a11 = a[c][c], a22 = a[t][t], a21 = colv(t, c);
          const double det = a11 * a22 - a21 * a21;
          if (std::fabs(det) > small && std::isfinite(det)) {
            const double i11 = a22 / det, i12 = -a21 / det, i22 = a11 / det;
            if (std::fma(std::fabs(i11), ap2, std::fabs(i12) * at2) <= lim &&
                std::fma(std::fabs(i12), ap2, std::fabs(i22) * at2) <= lim) {
              decided = 2; piv = c; tpiv = t;
            }
          }
        }
      }
      if (!decided) break;
      if (decided == 3) {
        if (!action) { o.flag = -5; break; }
        swap_xy(s, piv);
        for (int i = s; i < R; ++i) a[s][i] = (i == s) ? 1.0 : 0.0;
        P.dv[2 * s] = 0.0;
        P.dv[2 * s + 1] = 0.0;
        o.zero_pivots++;
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
  return s;
}

// APP block steps on the fully-summed columns of front f; returns the
// number of columns they eliminated (the failed ones end at the back of
// [0, n), in failure order).
int app_front(Front& f, double u, double small, bool action, Oracle& o) {
  const int m = f.m, n = f.n;
  auto& a = f.a;
  auto A = [&](int i, int j) -> double& { return a[(size_t)j * m + i]; };
  const int nblk = (n + BW - 1) / BW;
  const double lim = 1.0 / u;
  int p = 0;
  std::vector<double> pan((size_t)BW * m), ldp((size_t)BW * m);
  Panel P;
  for (int k = 0; k < nblk; ++k) {
    const int w = std::min(BW, n - BW * k);
    const int e = (w == BW) ? 0 : std::min(BW - w, m - n);
    const int R = w + e;
    auto prow = [&](int i) { return i < w ? p + i : n + (i - w); };
    for (int j = 0; j < w; ++j)
      for (int i = j; i < R; ++i) P.a[j][i] = A(prow(i), p + j);
    const int nd = diag_block(P, w, R, u, small, action, o);
    if (o.flag < 0) return -1;
    // block permutation on the rows of the eliminated columns and the variables
    {
      double tmp[BW];
      for (int c = 0; c < p; ++c) {
        for (int i = 0; i < w; ++i) tmp[i] = A(p + P.perm[i], c);
        for (int i = 0; i < w; ++i) A(p + i, c) = tmp[i];
      }
      int tv[BW];
      for (int i = 0; i < w; ++i) tv[i] = f.var[p + P.perm[i]];
      for (int i = 0; i < w; ++i) f.var[p + i] = tv[i];
    }
    // rows below: [p + w, n) then [n + e, m)
    int npass = nd;
    double x[BW];
    for (int r = p + w; r < m; ++r) {
      if (r >= n && r < n + e) continue;
      for (int kk = 0; kk < nd; ++kk) x[kk] = A(r, p + P.perm[kk]);
      for (int j = 0; j < nd; ++j) {
        const double xj = x[j];
        for (int kk = j + 1; kk < nd; ++kk) x[kk] = std::fma(-xj, P.a[j][kk], x[kk]);
      }
      for (int kk = 0; kk < nd;) {
        if (kk + 1 < nd && std::isinf(P.dv[2 * kk + 2])) {
          const double x1 = x[kk], x2 = x[kk + 1];
          x[kk] = std::fma(P.dv[2 * kk], x1, P.dv[2 * kk + 1] * x2);
          x[kk + 1] = std::fma(P.dv[2 * kk + 1], x1, P.dv[2 * kk + 3] * x2);
          kk += 2;
        } else {
          const double dk = P.dv[2 * kk];
          if (dk == 0.0) {
            const double v = x[kk];
            x[kk] = (std::fabs(v) < small) ? 0.0 : std::numeric_limits<double>::infinity() * v;
          } else {
            x[kk] = x[kk] * dk;
          }
          kk += 1;
        }
      }
      for (int kk = 0; kk < nd; ++kk)
        if (std::fabs(x[kk]) > lim) { npass = std::min(npass, kk); break; }
      for (int kk = 0; kk < nd; ++kk) pan[(size_t)kk * m + r] = x[kk];
    }
    for (int i = w; i < R; ++i)
      for (int kk = 0; kk < nd; ++kk) pan[(size_t)kk * m + prow(i)] = P.a[kk][i];
    // Column::adjust
    int np = std::min(npass, nd);
    if (np > 0 && std::isfinite(P.dv[2 * (np - 1)]) && P.dv[2 * (np - 1) + 1] != 0.0) np--;
    // commit rows [p, m): the block rows first from a copy of the block
    {
      std::vector<double> blk((size_t)w * w);
      for (int j = 0; j < w; ++j)
        for (int i = j; i < w; ++i) blk[(size_t)j * w + i] = A(p + i, p + j);
      auto borig = [&](int i, int kk) {
        int ai = P.perm[i], ak = P.perm[kk];
        return blk[(size_t)std::min(ai, ak) * w + std::max(ai, ak)];
      };
      double l[BW], orig[BW];
      for (int r = p; r < m; ++r) {
        const bool in_blk = r < p + w;
        const int i = r - p;
        for (int kk = np; kk < w; ++kk)
          orig[kk] = in_blk ? (i >= kk ? borig(i, kk) : 0.0) : A(r, p + P.perm[kk]);
        for (int kk = 0; kk < np; ++kk)
          l[kk] = in_blk ? (i > kk ? P.a[kk][i] : (i == kk ? 1.0 : 0.0)) : pan[(size_t)kk * m + r];
        for (int kk = 0; kk < w; ++kk) {
          if (in_blk && i < kk) continue;
          A(r, p + kk) = kk < np ? l[kk] : orig[kk];
        }
        if (r >= p + np) {
          double ld[BW];
          calc_ld_row(P.dv, l, np, ld);
          for (int kk = 0; kk < np; ++kk) ldp[(size_t)kk * m + r] = ld[kk];
        }
      }
    }
    for (int t = 0; t < 2 * np; ++t) f.d[2 * p + t] = P.dv[t];
    // trailing update of the fully-summed columns
    const int o0 = p + np;
    if (np > 0) {
      std::vector<double> acc(m);
      for (int j = o0; j < n; ++j) {
        // per entry: acc = 0; acc = fma(LD_ik, L_jk, acc), k ascending; a -= acc
        std::fill(acc.begin() + j, acc.end(), 0.0);
        for (int kk = 0; kk < np; ++kk) {
          const double b = A(j, p + kk);
          const double* lk = &ldp[(size_t)kk * m];
          for (int i = j; i < m; ++i) acc[i] = std::fma(lk[i], b, acc[i]);
        }
        for (int i = j; i < m; ++i) A(i, j) -= acc[i];
      }
    }
    // move the block's failed columns behind the unprocessed ones
    const int fl = w - np;
    if (fl > 0) {
      const int a0 = o0;
      auto from = [&](int i) { return i < n - fl ? i + fl : a0 + (i - (n - fl)); };
      const int mm = m - a0;
      std::vector<double> mv((size_t)mm * n);
      for (int c = 0; c < n; ++c)
        for (int r = std::max(a0, c); r < m; ++r) mv[(size_t)c * mm + (r - a0)] = A(r, c);
      for (int c = 0; c < n; ++c) {
        if (c < a0) {
          for (int r = a0; r < n; ++r) A(r, c) = mv[(size_t)c * mm + (from(r) - a0)];
        } else {
          const int oc = from(c);
          for (int r = c; r < m; ++r) {
            if (r < n) {
              const int orr = from(r);
              A(r, c) = mv[(size_t)std::min(orr, oc) * mm + (std::max(orr, oc) - a0)];
            } else {
              A(r, c) = mv[(size_t)oc * mm + (r - a0)];
            }
          }
        }
      }
      std::vector<int> vv(f.var.begin() + a0, f.var.begin() + n);
      for (int i = a0; i < n; ++i) f.var[i] = vv[from(i) - a0];
    }
    p += np;
  }
  return p;
}

// The same block steps in the reference's own layout: failed columns stay
// in their block; later pivots reach them through the blocks to their left
// (ApplyT: the rows of the pivot block in the failed columns; UpdateT: their
// uneliminated entries), and permute_failed moves them to the back after the
// last block (src/factor_indef.hxx:885-1183, :1190-1288;
// src/kernels/ldlt_app.hxx:405-431, :579-718).  Same arithmetic as
// app_front, so the two must agree bit for bit; used by the tests as a check
// of app_front's layout.
int app_front_inplace(Front& f, double u, double small, bool action, Oracle& o) {
  const int m = f.m, n = f.n;
  auto& a = f.a;
  auto A = [&](int i, int j) -> double& { return a[(size_t)j * m + i]; };
  auto S = [&](int i, int j) -> double& { return i >= j ? A(i, j) : A(j, i); };
  const int nblk = (n + BW - 1) / BW;
  const double lim = 1.0 / u;
  std::vector<char> done(m, 0);     // position eliminated
  std::vector<int> elim_order;      // positions in elimination order
  std::vector<int> failed;          // failed positions, in failure order
  std::vector<double> pan((size_t)BW * m), ldp((size_t)BW * m);
  Panel P;
  int next = 0;                     // eliminated so far (d offset)
  for (int k = 0; k < nblk; ++k) {
    const int c0 = BW * k, w = std::min(BW, n - c0);
    const int e = (w == BW) ? 0 : std::min(BW - w, m - n);
    const int R = w + e;
    auto prow = [&](int i) { return i < w ? c0 + i : n + (i - w); };
    for (int j = 0; j < w; ++j)
      for (int i = j; i < R; ++i) P.a[j][i] = A(prow(i), c0 + j);
    const int nd = diag_block(P, w, R, u, small, action, o);
    if (o.flag < 0) return -1;
    // row permutation of the block in every column to its left (apply_rperm)
    {
      double tmp[BW];
      for (int c = 0; c < c0; ++c) {
        for (int i = 0; i < w; ++i) tmp[i] = A(c0 + P.perm[i], c);
        for (int i = 0; i < w; ++i) A(c0 + i, c) = tmp[i];
      }
      int tv[BW];
      for (int i = 0; i < w; ++i) tv[i] = f.var[c0 + P.perm[i]];
      for (int i = 0; i < w; ++i) f.var[c0 + i] = tv[i];
    }
    // variables the block's pivots apply to: failed columns to the left
    // (ApplyT), later rows (ApplyN); x for each, entries of the block
    // columns read through the block's column permutation
    std::vector<int> rows;
    for (int fc : failed) rows.push_back(fc);
    for (int r = c0 + w; r < m; ++r)
      if (!(r >= n && r < n + e)) rows.push_back(r);
    int npass = nd;
    double x[BW];
    for (int r : rows) {
      for (int kk = 0; kk < nd; ++kk) x[kk] = S(r, c0 + (r < c0 ? kk : P.perm[kk]));
      // left failed column r: its row entries were already permuted above
      for (int j = 0; j < nd; ++j) {
        const double xj = x[j];
        for (int kk = j + 1; kk < nd; ++kk) x[kk] = std::fma(-xj, P.a[j][kk], x[kk]);
      }
      for (int kk = 0; kk < nd;) {
        if (kk + 1 < nd && std::isinf(P.dv[2 * kk + 2])) {
          const double x1 = x[kk], x2 = x[kk + 1];
          x[kk] = std::fma(P.dv[2 * kk], x1, P.dv[2 * kk + 1] * x2);
          x[kk + 1] = std::fma(P.dv[2 * kk + 1], x1, P.dv[2 * kk + 3] * x2);
          kk += 2;
        } else {
          const double dk = P.dv[2 * kk];
          if (dk == 0.0) {
            const double v = x[kk];
            x[kk] = (std::fabs(v) < small) ? 0.0 : std::numeric_limits<double>::infinity() * v;
          } else {
            x[kk] = x[kk] * dk;
          }
          kk += 1;
        }
      }
      for (int kk = 0; kk < nd; ++kk)
        if (std::fabs(x[kk]) > lim) { npass = std::min(npass, kk); break; }
      for (int kk = 0; kk < nd; ++kk) pan[(size_t)kk * m + r] = x[kk];
    }
    for (int i = w; i < R; ++i)
      for (int kk = 0; kk < nd; ++kk) pan[(size_t)kk * m + prow(i)] = P.a[kk][i];
    for (int i = w; i < R; ++i) rows.push_back(prow(i));
    int np = std::min(npass, nd);
    if (np > 0 && std::isfinite(P.dv[2 * (np - 1)]) && P.dv[2 * (np - 1) + 1] != 0.0) np--;
    // commit: the block's own rows, then every other row the step touched
    std::vector<double> blk((size_t)w * w);
    for (int j = 0; j < w; ++j)
      for (int i = j; i < w; ++i) blk[(size_t)j * w + i] = A(c0 + i, c0 + j);
    double l[BW], orig[BW], ld[BW];
    auto put_row = [&](int r, bool in_blk) {
      const int i = r - c0;
      for (int kk = np; kk < w; ++kk) {
        if (in_blk) {
          int ai = P.perm[i], ak = P.perm[kk];
          orig[kk] = i >= kk ? blk[(size_t)std::min(ai, ak) * w + std::max(ai, ak)] : 0.0;
        } else {
          orig[kk] = S(r, c0 + (r < c0 ? kk : P.perm[kk]));
        }
      }
      for (int kk = 0; kk < np; ++kk)
        l[kk] = in_blk ? (i > kk ? P.a[kk][i] : (i == kk ? 1.0 : 0.0)) : pan[(size_t)kk * m + r];
      for (int kk = 0; kk < w; ++kk) {
        if (in_blk && i < kk) continue;
        S(r, c0 + kk) = kk < np ? l[kk] : orig[kk];
      }
      if (!in_blk || i >= np) {
        calc_ld_row(P.dv, l, np, ld);
        for (int kk = 0; kk < np; ++kk) ldp[(size_t)kk * m + r] = ld[kk];
      }
    };
    for (int r = c0; r < c0 + w; ++r) put_row(r, true);
    for (int r : rows) put_row(r, false);
    for (int t = 0; t < 2 * np; ++t) f.d[2 * next + t] = P.dv[t];
    for (int i = 0; i < np; ++i) {
      done[c0 + i] = 1;
      elim_order.push_back(c0 + i);
    }
    next += np;
    // UpdateT / UpdateN: every uneliminated entry among the fully-summed
    // positions not yet done (rows also the contribution rows).  Of the two
    // variables of an entry, the one later in the order [this block's
    // failed, not yet processed, earlier failed (in failure order),
    // contribution rows] takes the L*D side of the product -- the order
    // app_front holds them in when it updates.
    if (np > 0) {
      std::vector<int> ord;
      for (int c = c0 + np; c < c0 + w; ++c) ord.push_back(c);
      for (int c = c0 + w; c < n; ++c) ord.push_back(c);
      for (int fc : failed) ord.push_back(fc);
      for (int r = n; r < m; ++r) ord.push_back(r);
      auto lval = [&](int v, int kk) { return S(v, c0 + kk); };
      const int nfs = (int)ord.size() - (m - n);  // fully-summed entries of ord
      for (int jj = 0; jj < nfs; ++jj) {
        const int j = ord[jj];
        for (int ii = jj; ii < (int)ord.size(); ++ii) {
          const int i = ord[ii];
          double acc = 0.0;
          for (int kk = 0; kk < np; ++kk) acc = std::fma(ldp[(size_t)kk * m + i], lval(j, kk), acc);
          S(i, j) -= acc;
        }
      }
    }
    for (int i = np; i < w; ++i) failed.push_back(c0 + i);
  }
  // permute_failed: eliminated positions first (elimination order), then the
  // failed ones (failure order), rows n.. unchanged
  std::vector<int> from(elim_order);
  from.insert(from.end(), failed.begin(), failed.end());
  for (int r = n; r < m; ++r) from.push_back(r);
  std::vector<double> b(a);
  std::vector<int> vv(f.var);
  for (int j = 0; j < m; ++j)
    for (int i = j; i < m; ++i) {
      int oi = from[i], oj = from[j];
      a[(size_t)j * m + i] = b[(size_t)std::min(oi, oj) * m + std::max(oi, oj)];
    }
  for (int i = 0; i < m; ++i) f.var[i] = vv[from[i]];
  return next;
}

// CB -= (L D) L^T over the eliminated columns (rows/cols >= n), in the fixed
// order: acc = 0; acc = fma(LD_ik, L_jk, acc) for k = 0 .. nelim-1; a_ij -= acc.
void form_contrib(Front& f) {
  const int m = f.m, n = f.n, ne = f.nelim, mc = m - n;
  if (mc <= 0 || ne <= 0) return;
  std::vector<double> ld((size_t)mc * ne), l(ne), out(ne);
  for (int i = 0; i < mc; ++i) {
    for (int k = 0; k < ne; ++k) l[k] = at(f.a, m, n + i, k);
    calc_ld_row(f.d.data(), l.data(), ne, out.data());
    for (int k = 0; k < ne; ++k) ld[(size_t)k * mc + i] = out[k];
  }
  std::vector<double> acc(mc);
  for (int j = 0; j < mc; ++j) {
    std::fill(acc.begin() + j, acc.end(), 0.0);
    for (int k = 0; k < ne; ++k) {
      const double b = at(f.a, m, n + j, k);
      const double* lk = &ld[(size_t)k * mc];
      for (int i = j; i < mc; ++i) acc[i] = std::fma(lk[i], b, acc[i]);
    }
    for (int i = j; i < mc; ++i) at(f.a, m, n + i, n + j) -= acc[i];
  }
}

}  // namespace

extern "C" {

void oracle_set_blas(void* dgemm, void* dtrsm, void* dsyrk, void* dpotrf) {
  g_dgemm = (dgemm_t)dgemm;
  g_dtrsm = (dtrsm_t)dtrsm;
  g_dsyrk = (dsyrk_t)dsyrk;
  g_dpotrf = (dpotrf_t)dpotrf;
}

// Factorize.  Symbolic arrays are the reference's 1-based layout; perm[i] is
// the 1-based pivot position of variable i.  stats receives
// [flag, num_neg, num_zero, num_two, num_delay, maxfront, not_first_pass,
//  not_second_pass, matrix_rank].
void* oracle_factor(int posdef, int n, int nnodes, const int* sptr, const int* sparent,
                    const long* rptr, const int* rlist, const long* nptr, const long* nlist,
                    const int* perm, const double* val, double u, double small, int action,
                    int tpp_cols, int* stats) {
  if (!g_dgemm || !g_dtrsm || !g_dsyrk || !g_dpotrf) return nullptr;
  Oracle* o = new Oracle();
  o->posdef = posdef != 0;
  o->n = n;
  o->nnodes = nnodes;
  o->perm.resize(n);
  for (int i = 0; i < n; ++i) o->perm[i] = perm[i] - 1;
  o->fronts.resize(nnodes);
  std::vector<std::vector<int>> kids(nnodes);
  for (int s = 0; s < nnodes; ++s)
    if (sparent[s] - 1 < nnodes) kids[sparent[s] - 1].push_back(s);
  std::vector<int> map(n, -1);
  for (int s = 0; s < nnodes && o->flag >= 0; ++s) {
    Front& f = o->fronts[s];
    int sncol = sptr[s + 1] - sptr[s];
    int snrow = (int)(rptr[s + 1] - rptr[s]);
    const int* rl = &rlist[rptr[s] - 1];
    int ndin = 0;
    for (int c : kids[s]) ndin += o->fronts[c].n - o->fronts[c].nelim;
    f.ndelay_in = ndin;
    f.n = sncol + ndin;
    f.m = snrow + ndin;
    int m = f.m;
    o->maxfront = std::max(o->maxfront, m);
    f.a.assign((size_t)m * m, 0.0);
    f.d.assign(2 * (size_t)std::max(f.n, 1), 0.0);
    f.var.assign(m, -1);
    for (int i = 0; i < sncol; ++i) f.var[i] = rl[i] - 1;
    int dpos = sncol;
    for (int c : kids[s]) {
      Front& cf = o->fronts[c];
      for (int j = cf.nelim; j < cf.n; ++j) f.var[dpos++] = cf.var[j];
    }
    for (int i = sncol; i < snrow; ++i) f.var[i + ndin] = rl[i] - 1;
    for (int i = 0; i < m; ++i) map[f.var[i]] = i;
    // A entries: dest is (col, row) in the symbolic nrow x ncol front
    for (long k = nptr[s] - 1; k < nptr[s + 1] - 1; ++k) {
      long src = nlist[2 * k] - 1, dest = nlist[2 * k + 1] - 1;
      int c = (int)(dest / snrow), r = (int)(dest % snrow);
      if (r >= sncol) r += ndin;
      at(f.a, m, r, c) += val[src];
    }
    // children: delayed columns and contribution blocks
    for (int c : kids[s]) {
      Front& cf = o->fronts[c];
      int cm = cf.m;
      for (int j = cf.nelim; j < cm; ++j) {
        int pj = map[cf.var[j]];
        for (int i = j; i < cm; ++i) {
          int pi = map[cf.var[i]];
          int r = std::max(pi, pj), cc = std::min(pi, pj);
          at(f.a, m, r, cc) += at(cf.a, cm, i, j);
        }
      }
    }
    // factorize
    if (o->posdef) {
      int nn = f.n;
      if (nn > 0) {
        int info = 0;
        const char L = 'L', R = 'R', T = 'T', N = 'N';
        g_dpotrf(&L, &nn, f.a.data(), &m, &info);
        if (info != 0) {
          o->flag = -6;
          break;
        }
        int mr = m - nn;
        double one = 1.0, mone = -1.0;
        if (mr > 0) {
          g_dtrsm(&R, &L, &T, &N, &mr, &nn, &one, f.a.data(), &m, &f.a[nn], &m);
          g_dsyrk(&L, &N, &mr, &nn, &mone, &f.a[nn], &m, &one, &f.a[(size_t)nn * m + nn], &m);
        }
      }
      f.nelim = nn;
    } else {
      // a-posteriori block steps, then threshold partial pivoting on the
      // failed columns (src/factor_failed.hxx:29-157); fronts with at most
      // tpp_cols fully-summed columns use TPP only (pivot_method = tpp)
      const bool app = f.n > 0 && f.n > tpp_cols;
      int pf = 0;
      if (app) {
        pf = g_inplace ? app_front_inplace(f, u, small, action != 0, *o)
                       : app_front(f, u, small, action != 0, *o);
        if (pf < 0) break;
      }
      int t1 = tpp(f, pf, f.n, u, small, action != 0, *o);
      if (t1 < 0) break;
      int ne = t1;
      bool root = sparent[s] - 1 >= nnodes;
      if (root && ne < f.n) {
        // nothing above a root can take delays: finish with the threshold
        // relaxed to plain partial pivoting (only the small-pivot test stays)
        ne = tpp(f, ne, f.n, kRootU, small, action != 0, *o);
        if (ne < 0) break;
      }
      if (app) {
        o->not_first_pass += f.n - pf;
        if (pf < f.n) o->not_second_pass += f.n - t1;
      } else {
        o->not_first_pass += f.n - t1;
      }
      f.nelim = ne;
      o->num_delay += f.n - ne;
      // the contribution block receives the eliminated columns' update; the
      // delayed columns already hold theirs
      form_contrib(f);
    }
  }
  if (o->flag >= 0) {
    int rank = 0;
    for (int s = 0; s < nnodes; ++s) {
      Front& f = o->fronts[s];
      o->num_factor += (int64_t)f.nelim * f.m - (int64_t)f.nelim * (f.nelim - 1) / 2;
      if (o->posdef) {
        rank += f.nelim;
        continue;
      }
      for (int i = 0; i < f.nelim;) {
        double a11 = f.d[2 * i], a21 = f.d[2 * i + 1];
        if (i + 1 == f.nelim || std::isfinite(f.d[2 * i + 2])) {
          if (a11 == 0.0) { o->num_zero++; }
          else rank++;
          if (a11 < 0.0) o->num_neg++;
          i++;
        } else {
          double a22 = f.d[2 * i + 3];
          o->num_two++;
          double det = a11 * a22 - a21 * a21, tr = a11 + a22;
          if (det < 0) o->num_neg++;
          else if (tr < 0) o->num_neg += 2;
          rank += 2;
          i += 2;
        }
      }
    }
    // uneliminated columns at a root are singular directions
    int uneliminated = 0;
    for (int s = 0; s < nnodes; ++s)
      if (sparent[s] - 1 >= nnodes) uneliminated += o->fronts[s].n - o->fronts[s].nelim;
    if (uneliminated) o->num_zero += uneliminated;
    if (o->num_zero > 0) o->flag = action ? 7 : -5;
    stats[8] = rank;
  }
  stats[0] = o->flag;
  stats[1] = o->num_neg;
  stats[2] = o->num_zero;
  stats[3] = o->num_two;
  stats[4] = o->num_delay;
  stats[5] = o->maxfront;
  stats[6] = o->not_first_pass;
  stats[7] = o->not_second_pass;
  return o;
}

// Solve A x = b in place (x: ldx x nrhs, user variable order).  job follows
// the reference (0 all, 1 fwd, 2 diag, 3 bwd, 4 diag_bwd).
int oracle_solve(void* h, int job, int nrhs, double* x, int ldx) {
  Oracle* o = (Oracle*)h;
  if (!o || o->flag < 0) return -1;
  int n = o->n;
  std::vector<double> x2((size_t)n * nrhs);
  for (int r = 0; r < nrhs; ++r)
    for (int i = 0; i < n; ++i) x2[(size_t)r * n + o->perm[i]] = x[(size_t)r * ldx + i];
  bool fwd = job == 0 || job == 1;
  bool diag = !o->posdef && (job == 0 || job == 2 || job == 4);
  bool bwd = job == 0 || job == 3 || job == 4;
  std::vector<double> xl;
  if (fwd) {
    for (int s = 0; s < o->nnodes; ++s) {
      Front& f = o->fronts[s];
      int m = f.m, ne = f.nelim;
      xl.assign(m, 0.0);
      for (int r = 0; r < nrhs; ++r) {
        double* xr = &x2[(size_t)r * n];
        for (int i = 0; i < m; ++i) xl[i] = xr[f.var[i]];
        for (int k = 0; k < ne; ++k) {
          // unit L for LDL^T (a 2x2 pivot's L block is the identity)
          double yk = o->posdef ? xl[k] / at(f.a, m, k, k) : xl[k];
          xl[k] = yk;
          for (int i = k + 1; i < m; ++i) xl[i] -= at(f.a, m, i, k) * yk;
        }
        for (int i = 0; i < m; ++i) xr[f.var[i]] = xl[i];
      }
    }
  }
  if (diag) {
    for (int s = 0; s < o->nnodes; ++s) {
      Front& f = o->fronts[s];
      for (int r = 0; r < nrhs; ++r) {
        double* xr = &x2[(size_t)r * n];
        for (int k = 0; k < f.nelim;) {
          if (k + 1 < f.nelim && std::isinf(f.d[2 * k + 2])) {
            double a = xr[f.var[k]], b = xr[f.var[k + 1]];
            xr[f.var[k]] = f.d[2 * k] * a + f.d[2 * k + 1] * b;
            xr[f.var[k + 1]] = f.d[2 * k + 1] * a + f.d[2 * k + 3] * b;
            k += 2;
          } else {
            xr[f.var[k]] *= f.d[2 * k];
            k++;
          }
        }
      }
    }
  }
  if (bwd) {
    for (int s = o->nnodes - 1; s >= 0; --s) {
      Front& f = o->fronts[s];
      int m = f.m, ne = f.nelim;
      xl.assign(m, 0.0);
      for (int r = 0; r < nrhs; ++r) {
        double* xr = &x2[(size_t)r * n];
        for (int i = 0; i < m; ++i) xl[i] = xr[f.var[i]];
        for (int k = ne - 1; k >= 0; --k) {
          double acc = xl[k];
          for (int i = k + 1; i < m; ++i) acc -= at(f.a, m, i, k) * xl[i];
          xl[k] = o->posdef ? acc / at(f.a, m, k, k) : acc;
        }
        for (int i = 0; i < ne; ++i) xr[f.var[i]] = xl[i];
      }
    }
  }
  for (int r = 0; r < nrhs; ++r)
    for (int i = 0; i < n; ++i) x[(size_t)r * ldx + i] = x2[(size_t)r * n + o->perm[i]];
  return 0;
}

void oracle_free(void* h) { delete (Oracle*)h; }

// Select the layout of the LDL^T block steps for later factorizations: 0
// failed columns move behind the unprocessed ones at once (app_front, the
// GPU's layout), 1 the reference's in-place layout (app_front_inplace).
void oracle_set_inplace(int on) { g_inplace = on != 0; }

// Front data for detailed comparisons: m, n, nelim of front s; copies the
// front's m x m array and 2n D^-1 entries and pivot-order variables if the
// pointers are non-null.
int oracle_front(void* h, int s, int* mn, double* a, double* d, int* var) {
  Oracle* o = (Oracle*)h;
  if (!o || s < 0 || s >= o->nnodes) return -1;
  Front& f = o->fronts[s];
  mn[0] = f.m;
  mn[1] = f.n;
  mn[2] = f.nelim;
  if (a) std::memcpy(a, f.a.data(), sizeof(double) * f.a.size());
  if (d) std::memcpy(d, f.d.data(), sizeof(double) * 2 * f.n);
  if (var) std::memcpy(var, f.var.data(), sizeof(int) * f.m);
  return 0;
}

}  // extern "C"
