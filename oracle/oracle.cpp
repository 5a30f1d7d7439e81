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
//   * indefinite: threshold partial pivoting with 1x1 and 2x2 pivots and
//     delays for columns that fail the threshold u, the reference's
//     pivot_method=tpp / failed-pivot path (src/factor_failed.hxx:29-157,
//     ldlt_tpp_factor call at :79), then form_contrib
//     (src/kernels/factor_indef.hxx:251-342).  D is stored inverted in the
//     reference's format (src/kernels/ldlt_app.hxx:166-171);
//   * inertia and 2x2 statistics: src/NumericTree.hxx:143-178;
//   * solves: src/NumericTreePosdef.hxx:357-450 and src/NumericTree.hxx:408-520
//     with the permute/scale wrapper src/spldlt_factorize_mod.F90:901-1060.
//
// SPRAL's ldlt_tpp_factor is not vendored (empty spral/ submodule); the TPP
// search below follows the published algorithm (Duff, Hogg & Lopez, SISC
// 2020; 1x1 test |a_pp| >= u * max_i |a_ip|, 2x2 test |D^-1| [max_p; max_t]
// <= 1/u), not SPRAL's source.
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

// Threshold partial pivoting on the first ncand columns of the m x m front.
// Updates only the candidate columns (all rows); returns nelim.  The
// eliminated columns hold L (unit diagonal implied) and d holds D^-1.
int tpp(Front& f, int start, int ncand, double u, double small, bool action, Oracle& o) {
  const int m = f.m;
  auto& a = f.a;
  int nelim = start;
  while (nelim < ncand) {
    bool found = false;
    for (int p = nelim; p < ncand && !found; ++p) {
      // column p entries in rows >= nelim (excluding p), lower storage
      auto colp = [&](int i) -> double { return i > p ? at(a, m, i, p) : at(a, m, p, i); };
      double amax = 0.0;
      int t = -1;
      for (int i = nelim; i < m; ++i) {
        if (i == p) continue;
        double v = std::fabs(colp(i));
        if (v > amax) { amax = v; t = i; }
      }
      double app = at(a, m, p, p);
      if (amax < small && std::fabs(app) < small) {
        if (!action) { o.flag = -5; return -1; }
        // zero pivot: eliminate with d = 0, column of L is zero
        sym_swap(a, m, nelim, p);
        std::swap(f.var[nelim], f.var[p]);
        for (int i = nelim; i < m; ++i) at(a, m, i, nelim) = 0.0;
        f.d[2 * nelim] = 0.0;
        f.d[2 * nelim + 1] = 0.0;
        nelim++;
        found = true;
        break;
      }
      if (std::fabs(app) >= u * amax) {
        sym_swap(a, m, nelim, p);
        std::swap(f.var[nelim], f.var[p]);
        int k = nelim;
        double dinv = 1.0 / at(a, m, k, k);
        // l = a(:,k) * dinv ; update candidate columns j in (k, ncand)
        for (int j = k + 1; j < ncand; ++j) {
          double ljd = at(a, m, j, k);  // (L D)_jk before scaling
          double lj = ljd * dinv;
          for (int i = j; i < m; ++i) at(a, m, i, j) -= at(a, m, i, k) * lj;
        }
        for (int i = k + 1; i < m; ++i) at(a, m, i, k) *= dinv;
        at(a, m, k, k) = 1.0;
        f.d[2 * k] = dinv;
        f.d[2 * k + 1] = 0.0;
        nelim++;
        found = true;
        break;
      }
      if (t >= 0 && t < ncand) {
        auto colt = [&](int i) -> double { return i > t ? at(a, m, i, t) : at(a, m, t, i); };
        double ap2 = 0.0, at2 = 0.0;
        for (int i = nelim; i < m; ++i) {
          if (i == p || i == t) continue;
          ap2 = std::max(ap2, std::fabs(colp(i)));
          at2 = std::max(at2, std::fabs(colt(i)));
        }
        double a11 = app, a22 = at(a, m, t, t), a21 = colp(t);
        double det = a11 * a22 - a21 * a21;
        if (std::fabs(det) > small && std::isfinite(det)) {
          double i11 = a22 / det, i12 = -a21 / det, i22 = a11 / det;
          if (std::fabs(i11) * ap2 + std::fabs(i12) * at2 <= 1.0 / u &&
              std::fabs(i12) * ap2 + std::fabs(i22) * at2 <= 1.0 / u) {
            int k = nelim;
            sym_swap(a, m, k, p);
            std::swap(f.var[k], f.var[p]);
            int tt = (t == k) ? p : t;  // t may have moved to p
            sym_swap(a, m, k + 1, tt);
            std::swap(f.var[k + 1], f.var[tt]);
            // 2x2 block now at (k, k+1); recompute its entries after swaps
            a11 = at(a, m, k, k);
            a21 = at(a, m, k + 1, k);
            a22 = at(a, m, k + 1, k + 1);
            det = a11 * a22 - a21 * a21;
            i11 = a22 / det; i12 = -a21 / det; i22 = a11 / det;
            for (int j = k + 2; j < ncand; ++j) {
              double w1 = at(a, m, j, k), w2 = at(a, m, j, k + 1);
              double l1 = i11 * w1 + i12 * w2, l2 = i12 * w1 + i22 * w2;
              for (int i = j; i < m; ++i)
                at(a, m, i, j) -= at(a, m, i, k) * l1 + at(a, m, i, k + 1) * l2;
            }
            for (int i = k + 2; i < m; ++i) {
              double w1 = at(a, m, i, k), w2 = at(a, m, i, k + 1);
              at(a, m, i, k) = i11 * w1 + i12 * w2;
              at(a, m, i, k + 1) = i12 * w1 + i22 * w2;
            }
            at(a, m, k, k) = 1.0;
            at(a, m, k + 1, k) = 0.0;
            at(a, m, k + 1, k + 1) = 1.0;
            f.d[2 * k] = i11;
            f.d[2 * k + 1] = i12;
            f.d[2 * k + 2] = std::numeric_limits<double>::infinity();
            f.d[2 * k + 3] = i22;
            nelim += 2;
            found = true;
            break;
          }
        }
      }
    }
    if (!found) break;
  }
  return nelim;
}

// CB -= L21 D L21^T over eliminated columns (rows/cols >= n).
void form_contrib(Front& f) {
  int m = f.m, n = f.n, ne = f.nelim, mc = m - n;
  if (mc <= 0 || ne <= 0) return;
  std::vector<double> ld((size_t)mc * ne);
  for (int k = 0; k < ne;) {
    bool two = (k + 1 < ne) && std::isinf(f.d[2 * k + 2]);
    if (!two) {
      double d11 = f.d[2 * k];
      double dd = (d11 == 0.0) ? 0.0 : 1.0 / d11;
      for (int i = 0; i < mc; ++i) ld[(size_t)k * mc + i] = at(f.a, m, n + i, k) * dd;
      k++;
    } else {
      double i11 = f.d[2 * k], i12 = f.d[2 * k + 1], i22 = f.d[2 * k + 3];
      double det = i11 * i22 - i12 * i12;  // D = inv(Dinv)
      double d11 = i22 / det, d12 = -i12 / det, d22 = i11 / det;
      for (int i = 0; i < mc; ++i) {
        double l1 = at(f.a, m, n + i, k), l2 = at(f.a, m, n + i, k + 1);
        ld[(size_t)k * mc + i] = l1 * d11 + l2 * d12;
        ld[(size_t)(k + 1) * mc + i] = l1 * d12 + l2 * d22;
      }
      k += 2;
    }
  }
  const char N = 'N', T = 'T';
  double mone = -1.0, one = 1.0;
  g_dgemm(&N, &T, &mc, &mc, &ne, &mone, ld.data(), &mc, &f.a[(size_t)n], &m, &one,
          &f.a[(size_t)n * m + n], &m);
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
                    int* stats) {
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
      int ne = tpp(f, 0, f.n, u, small, action != 0, *o);
      if (ne < 0) break;
      bool root = sparent[s] - 1 >= nnodes;
      if (root && ne < f.n) {
        // nothing above a root can take delays: finish with the threshold
        // relaxed to plain partial pivoting (only the small-pivot test stays)
        o->not_second_pass += f.n - ne;
        ne = tpp(f, ne, f.n, std::numeric_limits<double>::min(), small, action != 0, *o);
        if (ne < 0) break;
      }
      f.nelim = ne;
      // delayed columns keep their (updated) values for the parent; the
      // contribution block receives the eliminated columns' update
      form_contrib(f);
      // the delayed part of the front must also see the CB-style update for
      // rows/cols in [nelim, n): tpp already updated the candidate columns.
      int nd = f.n - f.nelim;
      o->num_delay += nd;
      o->not_first_pass += nd;  // TPP is this path's only pass
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
