// The reference's C-ABI (include/sylver/sylver.h:73-123, implemented in
// Fortran at src/interfaces/C/sylver_ciface.F90:304-826) and its internal
// C++ seam (src/SymbolicTree.cxx:110-137, src/NumericTree.cxx:27-136,
// src/NumericTreePosdef.cxx:19-83), exported from C++ over the GPU runtime.
//
// Argument checks and flag values follow src/spldlt_factorize_mod.F90
// (factorize :640-670, :855-864; solve :1225-1280).  Differences from the
// reference, all deliberate:
//   * job != 0 solves do what the job value says (the reference always runs
//     the full fwd + diag_bwd sweep once job is present);
//   * CUDA failures return SYLVER_ERROR_CUDA_UNKNOWN instead of exit(1).
#include <cstring>
#include <exception>
#include <new>

#include "../../include/sylver_gb300.h"
#include "analyse.hpp"
#include "ldlt.hpp"
#include "numeric.hpp"
#include "scaling.hpp"

using namespace sylver_gb300;

namespace {

// Values of the cleaned lower-triangle matrix (duplicates summed) from the
// caller's val array.
std::vector<double> clean_values(const AnalyseResult& c, const double* val) {
  std::vector<double> v(c.crow.size(), 0.0);
  for (size_t k = 0; k < c.crow.size(); ++k)
    for (int64_t q = c.srcptr[k]; q < c.srcptr[k + 1]; ++q) v[k] += val[c.src[q]];
  return v;
}

void clear_inform(sylver_inform_t* inf) {
  if (inf) std::memset(inf, 0, sizeof(*inf));
}

void fill_inform_from_akeep(const AKeep& a, sylver_inform_t* inf) {
  inf->flag = a.flag;
  inf->matrix_dup = a.matrix_dup;
  inf->matrix_outrange = a.matrix_outrange;
  inf->matrix_missing_diag = a.matrix_missing_diag;
  inf->matrix_rank = a.n;
  inf->maxdepth = a.st.maxdepth;
  inf->maxfront = a.st.maxfront;
  inf->num_factor = (long)a.st.num_factor;
  inf->num_flops = (long)a.st.num_flops;
  inf->num_sup = a.st.nnodes;
}

void fill_inform_from_fkeep(const FKeep& f, sylver_inform_t* inf) {
  fill_inform_from_akeep(*f.ak, inf);
  inf->flag = f.flag;
  inf->matrix_rank = f.rank;
  inf->maxfront = f.maxfront;
  inf->num_delay = f.num_delay;
  inf->num_neg = f.num_neg;
  inf->num_two = f.num_two;
  inf->num_factor = (long)f.num_factor;
}

// Common factorize body.  val_host or val_dev supplies the values.
void factorize_common(bool posdef, const double* val_host, const double* val_dev,
                      double* scale, void* akeep, void** fkeep, const sylver_options_t* opt,
                      sylver_inform_t* inform, int precision, double ir_tol, int ir_max_iter) {
  clear_inform(inform);
  AKeep* ak = static_cast<AKeep*>(akeep);
  if (!ak || ak->flag < 0) {
    inform->flag = SYLVER_ERROR_CALL_SEQUENCE;
    return;
  }
  fill_inform_from_akeep(*ak, inform);
  if (ak->n == 0 || ak->st.nnodes == 0) {
    inform->flag = SYLVER_SUCCESS;
    inform->matrix_rank = 0;
    return;
  }
  Runtime& rt = Runtime::get();
  if (!rt.init()) {
    inform->flag = SYLVER_ERROR_CUDA_UNKNOWN;
    inform->cuda_error = 1;
    return;
  }
  try {
    FKeep* fk = fkeep ? static_cast<FKeep*>(*fkeep) : nullptr;
    if (fk && (fk->ak != ak || fk->posdef != posdef || fk->precision != precision)) {
      delete fk;
      fk = nullptr;
    }
    if (!fk) {
      fk = new FKeep();
      fk->ak = ak;
      fk->posdef = posdef;
      fk->precision = precision;
      if (posdef) fk->plan_cholesky();
      else plan_ldlt(*fk);
      fk->upload_static(rt.stream);
      if (fkeep) *fkeep = fk;
    }
    fk->ir_tol = ir_tol;
    fk->ir_max_iter = ir_max_iter;
    if (opt) {
      fk->u = opt->u;
      fk->small_piv = opt->small;
      fk->action = opt->action;
    }
    const int64_t nz = ak->nnz_val();
    const double* vdev = val_dev;
    // scaling S A S (src/spldlt_factorize_mod.F90:727-830), applied on the
    // device after the unscaled values are kept for the residual:
    //   scaling <= 0: the caller's `scale` (none when null);
    //   1, 2: maximum-product matching scaling of these values (the
    //         reference's Hungarian and auction variants compute the same
    //         kind of scaling; both use the matching here);
    //   3: the scaling saved by the matching-based ordering;
    //   >= 4: infinity-norm equilibration.
    // Computed scalings are copied to `scale` when it is given.
    const int sopt = opt ? opt->scaling : 0;
    std::vector<double> comp;
    const double* use_scale = nullptr;
    if (sopt <= 0) {
      use_scale = scale;
    } else if (sopt == 3) {
      if (ak->mscale.empty()) {
        inform->flag = SYLVER_ERROR_NO_SAVED_SCALING;
        if (!fkeep) delete fk;
        return;
      }
      comp = ak->mscale;
    } else {
      std::vector<double> hv;
      const double* hval = val_host;
      if (!hval) {
        hv.resize(std::max<int64_t>(nz, 1));
        if (nz) SG_CUDA(cudaMemcpy(hv.data(), val_dev, nz * sizeof(double),
                                   cudaMemcpyDeviceToHost));
        hval = hv.data();
      }
      SymCsc full = expand_lower(ak->n, ak->clean.cptr, ak->clean.crow,
                                 clean_values(ak->clean, hval));
      if (sopt <= 2) {
        std::vector<int> match;
        matching_scaling(full, match, comp);
      } else {
        equilibration_scaling(full, comp);
      }
    }
    if (!comp.empty()) {
      use_scale = comp.data();
      if (scale) std::copy(comp.begin(), comp.end(), scale);
    }
    fk->set_scale(use_scale, rt.stream);
    if (val_host) {
      fk->val.ensure(std::max<int64_t>(nz, 1) * sizeof(double));
      if (nz) SG_CUDA(cudaMemcpyAsync(fk->val.p, val_host, nz * sizeof(double),
                                      cudaMemcpyHostToDevice, rt.stream));
      vdev = fk->val.as<double>();
    }
    int flag = posdef ? fk->factorize(vdev, rt.stream) : factorize_ldlt(*fk, vdev, rt.stream);
    fill_inform_from_fkeep(*fk, inform);
    inform->flag = flag;
    // the matching-based ordering's scaling was not used
    // (src/spldlt_factorize_mod.F90:721-725)
    if (flag == 0 && !ak->mscale.empty() && sopt != 3)
      inform->flag = SYLVER_WARNING_MATCH_ORD_NO_SCALE;
    if (!fkeep) delete fk;
  } catch (const std::bad_alloc&) {
    inform->flag = SYLVER_ERROR_ALLOCATION;
  } catch (const CudaError& e) {
    inform->flag = SYLVER_ERROR_CUDA_UNKNOWN;
    inform->cuda_error = 1;
    if (opt && opt->print_level > 0) fprintf(stderr, "sylver_gb300: %s\n", e.what());
  } catch (const std::exception& e) {
    inform->flag = SYLVER_ERROR_UNKNOWN;
    if (opt && opt->print_level > 0) fprintf(stderr, "sylver_gb300: %s\n", e.what());
  }
}

int solve_checks(int job, int nrhs, int ldx, AKeep* ak, FKeep* fk) {
  if (!ak || !fk || ak->flag < 0 || fk->flag < 0 || fk->ak != ak)
    return SYLVER_ERROR_CALL_SEQUENCE;
  if (ldx < ak->n || nrhs < 1) return SYLVER_ERROR_X_SIZE;
  if (job < 0 || job > 4) return SYLVER_ERROR_JOB_OOR;
  if (fk->posdef && (job == SYLVER_SOLVE_JOB_DIAG || job == SYLVER_SOLVE_JOB_DIAG_BWD))
    return SYLVER_ERROR_JOB_OOR;
  return 0;
}

void solve_common(int job, int nrhs, double* x, bool x_on_device, int ldx, void* akeep,
                  void* fkeep, const sylver_options_t* opt, sylver_inform_t* inform) {
  clear_inform(inform);
  AKeep* ak = static_cast<AKeep*>(akeep);
  FKeep* fk = static_cast<FKeep*>(fkeep);
  if (ak && ak->st.nnodes == 0 && ak->flag >= 0) return;
  int chk = solve_checks(job, nrhs, ldx, ak, fk);
  if (chk) {
    inform->flag = chk;
    return;
  }
  fill_inform_from_fkeep(*fk, inform);
  inform->flag = std::max(0, fk->flag);  // keep factorize warnings
  Runtime& rt = Runtime::get();
  try {
    const int n = ak->n;
    double* xd = x;
    DevMem tmp;
    if (!x_on_device) {
      tmp.ensure((size_t)n * nrhs * sizeof(double));
      xd = tmp.as<double>();
      SG_CUDA(cudaMemcpy2DAsync(xd, n * sizeof(double), x, (size_t)ldx * sizeof(double),
                                n * sizeof(double), nrhs, cudaMemcpyHostToDevice, rt.stream));
    }
    int ldd = x_on_device ? ldx : n;
    int rc = fk->solve(job, nrhs, xd, ldd, rt.stream);
    if (!x_on_device) {
      SG_CUDA(cudaMemcpy2DAsync(x, (size_t)ldx * sizeof(double), xd, n * sizeof(double),
                                n * sizeof(double), nrhs, cudaMemcpyDeviceToHost, rt.stream));
    }
    SG_CUDA(cudaStreamSynchronize(rt.stream));
    if (rc < 0) inform->flag = rc;
    else if (rc > 0) inform->flag = std::max(inform->flag, rc);
  } catch (const std::bad_alloc&) {
    inform->flag = SYLVER_ERROR_ALLOCATION;
  } catch (const CudaError& e) {
    inform->flag = SYLVER_ERROR_CUDA_UNKNOWN;
    inform->cuda_error = 1;
    if (opt && opt->print_level > 0) fprintf(stderr, "sylver_gb300: %s\n", e.what());
  } catch (const std::exception& e) {
    inform->flag = SYLVER_ERROR_UNKNOWN;
  }
}

}  // namespace

extern "C" {

void sylver_init(int ncpu, int ngpu) {
  (void)ncpu;
  (void)ngpu;
  Runtime::get().init();
}

void sylver_finalize(void) {
  Runtime& rt = Runtime::get();
  if (rt.ok) cudaStreamSynchronize(rt.stream);
}

void sylver_default_options(sylver_options_t* o) {
  // defaults: src/sylver_datatypes_mod.F90:97-198; array_base 0 as the C
  // wrapper sets it (sylver_ciface.F90:314)
  std::memset(o, 0, sizeof(*o));
  o->array_base = 0;
  o->print_level = 0;
  o->unit_diagnostics = 6;
  o->unit_error = 6;
  o->unit_warning = 6;
  o->ordering = 1;
  o->nemin = 32;
  o->prune_tree = true;
  o->min_gpu_work = 5000000000L;
  o->scaling = 0;
  o->pivot_method = 2;
  o->small = 1e-20;
  o->u = 0.01;
  o->small_subtree_threshold = 4000000L;
  o->nb = 256;
  o->cpu_topology = 1;
  o->action = true;
  o->use_gpu = true;
  o->gpu_perf_coeff = 1.0;
  o->failed_pivot_method = 1;
  o->scheduler = 1;
}

void spldlt_analyse(int n, int* order, long const* ptr, int const* row, double const* val,
                    void** akeep, bool check, sylver_options_t const* options,
                    sylver_inform_t* inform) {
  clear_inform(inform);
  if (!akeep) {
    inform->flag = SYLVER_ERROR_UNKNOWN;
    return;
  }
  if (*akeep) {
    delete static_cast<AKeep*>(*akeep);
    *akeep = nullptr;
  }
  try {
    AKeep* ak = new AKeep();
    *akeep = ak;
    ak->n = n;
    ak->check = check;
    const int ordering = options ? options->ordering : 1;
    if (ordering < 0 || ordering > 2) {
      ak->flag = inform->flag = SYLVER_ERROR_ORDER;  // src/spldlt_analyse_mod.F90:692-696
      return;
    }
    if (ordering == 2 && !val) {
      ak->flag = inform->flag = SYLVER_ERROR_VAL;  // :698-703
      return;
    }
    AnalyseInput in{n, reinterpret_cast<const int64_t*>(ptr), row, order, check, ordering,
                    options ? options->nemin : 32};
    ak->clean = clean_matrix(in);
    ak->matrix_outrange = ak->clean.matrix_outrange;
    ak->matrix_dup = ak->clean.matrix_dup;
    ak->matrix_missing_diag = ak->clean.matrix_missing_diag;
    if (ak->clean.flag < 0) {
      ak->flag = ak->clean.flag;
      inform->flag = ak->flag;
      return;
    }
    // matching-based ordering (match_order_metis, :787-816): the order comes
    // from the compressed matching graph and its scaling is saved for
    // factorize (options.scaling = 3)
    std::vector<int> morder;
    int msing = 0;
    if (ordering == 2) {
      SymCsc full = expand_lower(n, ak->clean.cptr, ak->clean.crow, clean_values(ak->clean, val));
      std::vector<int> match;
      msing = matching_scaling(full, match, ak->mscale);
      std::vector<int> pos = matching_order(full, match);
      morder.resize(n);
      for (int i = 0; i < n; ++i) morder[i] = pos[i] + 1;
      in.order = morder.data();
      in.ordering = 0;
    }
    std::string err;
    int fl = analyse(in, ak->clean, ak->st, err);
    if (fl < 0) {
      ak->flag = fl;
      inform->flag = fl;
      return;
    }
    ak->flag = ak->clean.flag;
    if (msing && ak->flag == 0) ak->flag = SYLVER_WARNING_ANAL_SINGULAR;
    ak->build_full_csr();
    fill_inform_from_akeep(*ak, inform);
  } catch (const std::bad_alloc&) {
    inform->flag = SYLVER_ERROR_ALLOCATION;
    if (*akeep) static_cast<AKeep*>(*akeep)->flag = SYLVER_ERROR_ALLOCATION;
  }
}

void spldlt_factorize(bool posdef, long const* ptr, int const* row, double const* val,
                      double* scale, void* akeep, void** fkeep,
                      sylver_options_t const* options, sylver_inform_t* inform) {
  (void)ptr;
  (void)row;
  factorize_common(posdef, val, nullptr, scale, akeep, fkeep, options, inform, SYLVER_GB300_FP64,
                   1e-14, 0);
}

void spldlt_factorize_mixed(bool posdef, long const* ptr, int const* row, double const* val,
                            double* scale, void* akeep, void** fkeep,
                            sylver_options_t const* options, sylver_inform_t* inform,
                            int precision, double ir_tol, int ir_max_iter) {
  (void)ptr;
  (void)row;
  factorize_common(posdef, val, nullptr, scale, akeep, fkeep, options, inform, precision, ir_tol,
                   ir_max_iter);
}

void spldlt_factorize_device(bool posdef, double const* val_dev, void* akeep, void** fkeep,
                             sylver_options_t const* options, sylver_inform_t* inform,
                             int precision, double ir_tol, int ir_max_iter) {
  factorize_common(posdef, nullptr, val_dev, nullptr, akeep, fkeep, options, inform, precision,
                   ir_tol, ir_max_iter);
}

void spldlt_solve(int job, int nrhs, double* x, int ldx, void* akeep, void* fkeep,
                  sylver_options_t const* options, sylver_inform_t* inform) {
  // a scaling given at factorize time is applied by the device solve
  solve_common(job, nrhs, x, false, ldx, akeep, fkeep, options, inform);
}

void spldlt_solve_device(int job, int nrhs, double* x_dev, int ldx, void* akeep, void* fkeep,
                         sylver_options_t const* options, sylver_inform_t* inform) {
  solve_common(job, nrhs, x_dev, true, ldx, akeep, fkeep, options, inform);
}

void spldlt_free_akeep(void** akeep) {
  if (!akeep || !*akeep) return;
  delete static_cast<AKeep*>(*akeep);
  *akeep = nullptr;
}

void spldlt_free_fkeep(void** fkeep) {
  if (!fkeep || !*fkeep) return;
  delete static_cast<FKeep*>(*fkeep);
  *fkeep = nullptr;
}

int sylver_gb300_solve_stats(void const* fkeep, int* ir_iters, double* bwd_err) {
  const FKeep* fk = static_cast<const FKeep*>(fkeep);
  if (!fk) return -1;
  if (ir_iters) *ir_iters = fk->last_ir_iters;
  if (bwd_err) *bwd_err = fk->last_bwd_err;
  return 0;
}

int sylver_gb300_solve_history(void const* fkeep, double* bwd_err, int max_entries) {
  const FKeep* fk = static_cast<const FKeep*>(fkeep);
  if (!fk) return -1;
  int k = 0;
  for (double v : fk->ir_hist) {
    if (k >= max_entries) break;
    if (bwd_err) bwd_err[k] = v;
    k++;
  }
  return k;
}

int sylver_gb300_akeep_sizes(void const* akeep, int* n, int* nnodes, long* rlist_len,
                             long* nlist_len) {
  const AKeep* ak = static_cast<const AKeep*>(akeep);
  if (!ak) return -1;
  if (n) *n = ak->n;
  if (nnodes) *nnodes = ak->st.nnodes;
  if (rlist_len) *rlist_len = (long)ak->st.rlist.size();
  if (nlist_len) *nlist_len = (long)ak->st.nlist.size();
  return ak->flag;
}

int sylver_gb300_akeep_arrays(void const* akeep, int* sptr, int* sparent, long* rptr,
                              int* rlist, long* nptr, long* nlist, int* perm) {
  const AKeep* ak = static_cast<const AKeep*>(akeep);
  if (!ak) return -1;
  const SymbolicTree& st = ak->st;
  if (sptr) std::copy(st.sptr.begin(), st.sptr.end(), sptr);
  if (sparent) std::copy(st.sparent.begin(), st.sparent.end(), sparent);
  if (rptr) for (size_t i = 0; i < st.rptr.size(); ++i) rptr[i] = (long)st.rptr[i];
  if (rlist) std::copy(st.rlist.begin(), st.rlist.end(), rlist);
  if (nptr) for (size_t i = 0; i < st.nptr.size(); ++i) nptr[i] = (long)st.nptr[i];
  if (nlist) for (size_t i = 0; i < st.nlist.size(); ++i) nlist[i] = (long)st.nlist[i];
  if (perm) for (size_t i = 0; i < st.perm.size(); ++i) perm[i] = st.perm[i] + 1;
  return 0;
}

int sylver_gb300_akeep_scaling(void const* akeep, double* scale) {
  const AKeep* ak = static_cast<const AKeep*>(akeep);
  if (!ak || ak->mscale.empty()) return 0;
  if (scale) std::copy(ak->mscale.begin(), ak->mscale.end(), scale);
  return (int)ak->mscale.size();
}

int sylver_gb300_fkeep_diag(void const* fkeep, double* d, int* piv_order) {
  const FKeep* fk = static_cast<const FKeep*>(fkeep);
  if (!fk) return -1;
  return ldlt_export_diag(*fk, d, piv_order);
}

int sylver_gb300_fkeep_fronts(void const* fkeep, int* m, int* n, int* nelim) {
  const FKeep* fk = static_cast<const FKeep*>(fkeep);
  if (!fk) return -1;
  return ldlt_export_fronts(*fk, m, n, nelim);
}

long sylver_gb300_fkeep_factor_bytes(void const* fkeep, void* dst, long cap) {
  const FKeep* fk = static_cast<const FKeep*>(fkeep);
  if (!fk) return -1;
  const long bytes = (long)fk->factor_bytes();
  if (dst && cap >= bytes && bytes > 0) {
    Runtime& rt = Runtime::get();
    if (cudaMemcpyAsync(dst, fk->factor_base(), (size_t)bytes, cudaMemcpyDeviceToHost, rt.stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(rt.stream) != cudaSuccess)
      return -1;
  }
  return bytes;
}

void* sylver_gb300_stream(void) {
  Runtime& rt = Runtime::get();
  rt.init();
  return (void*)rt.stream;
}

int sylver_gb300_profile_factor(void* fkeep, double const* val_dev, double* ms, long* launches,
                                double* flops) {
  FKeep* fk = static_cast<FKeep*>(fkeep);
  if (!fk) return SYLVER_ERROR_CALL_SEQUENCE;
  try {
    return fk->profile(val_dev, ms, launches, flops, Runtime::get().stream);
  } catch (const std::exception&) {
    return SYLVER_ERROR_CUDA_UNKNOWN;
  }
}

int sylver_gb300_profile_levels(void* fkeep, double const* val_dev, double* level_ms,
                                int max_levels) {
  FKeep* fk = static_cast<FKeep*>(fkeep);
  if (!fk || !level_ms) return SYLVER_ERROR_CALL_SEQUENCE;
  const int nl = (int)fk->levels.size();
  if (max_levels < nl) return SYLVER_ERROR_X_SIZE;
  std::vector<double> ms(12), fl(12);
  std::vector<long> cnt(12);
  for (int l = 0; l < nl; ++l) level_ms[l] = 0.0;
  try {
    int rc = fk->profile(val_dev, ms.data(), cnt.data(), fl.data(), Runtime::get().stream,
                         level_ms);
    return rc < 0 ? rc : nl;
  } catch (const std::exception&) {
    return SYLVER_ERROR_CUDA_UNKNOWN;
  }
}

int sylver_gb300_profile_solve(void* fkeep, int nrhs, double* ms, long* launches) {
  FKeep* fk = static_cast<FKeep*>(fkeep);
  if (!fk || !ms || !launches) return SYLVER_ERROR_CALL_SEQUENCE;
  try {
    return fk->profile_solve(nrhs, ms, launches, Runtime::get().stream);
  } catch (const std::exception&) {
    return SYLVER_ERROR_CUDA_UNKNOWN;
  }
}

int sylver_gb300_fkeep_counters(void const* fkeep, long* kernel_launches, int* nlevels,
                                double* factor_ms) {
  const FKeep* fk = static_cast<const FKeep*>(fkeep);
  if (!fk) return -1;
  if (kernel_launches) *kernel_launches = fk->launches;
  if (nlevels) *nlevels = (int)fk->levels.size();
  if (factor_ms) *factor_ms = fk->factor_ms;
  return 0;
}

// ---- internal C-ABI #2 -------------------------------------------------------

void* spldlt_create_symbolic_tree(void* akeep, int n, int nnodes, int const* sptr,
                                  int const* sparent, long const* rptr, int const* rlist,
                                  long const* nptr, long const* nlist, int nsubtrees,
                                  int const* subtrees, int const* small,
                                  int const* contrib_dest, int const* exec_loc) {
  (void)akeep;
  (void)nsubtrees;
  (void)subtrees;
  (void)small;
  (void)contrib_dest;
  (void)exec_loc;
  AKeep* ak = new AKeep();
  ak->n = n;
  SymbolicTree& st = ak->st;
  st.n = n;
  st.nnodes = nnodes;
  st.sptr.assign(sptr, sptr + nnodes + 1);
  st.sparent.assign(sparent, sparent + nnodes);
  st.rptr.assign(rptr, rptr + nnodes + 1);
  st.rlist.assign(rlist, rlist + (rptr[nnodes] - 1));
  st.nptr.assign(nptr, nptr + nnodes + 1);
  st.nlist.assign(nlist, nlist + 2 * (nptr[nnodes] - 1));
  // pivot order is the identity at this seam: rlist already holds pivots
  st.perm.resize(n);
  st.invp.resize(n);
  for (int i = 0; i < n; ++i) st.perm[i] = st.invp[i] = i;
  st.derive();
  ak->clean.cptr.assign(n + 1, 0);
  ak->build_full_csr();
  return ak;
}

void spldlt_destroy_symbolic_tree(void* symbolic_tree) { delete static_cast<AKeep*>(symbolic_tree); }

void* spldlt_create_numeric_tree_dbl(bool posdef, void* fkeep, void* symbolic_tree,
                                     double* aval, const double* scaling, void** child_contrib,
                                     sylver_options_c* options, sylver_inform_c* inform) {
  (void)fkeep;
  (void)child_contrib;
  sylver_options_t o;
  sylver_default_options(&o);
  if (options) {
    o.u = options->u;
    o.small = options->small;
    o.action = options->action;
    o.print_level = options->print_level;
  }
  sylver_inform_t inf;
  void* fk = nullptr;
  AKeep* ak = static_cast<AKeep*>(symbolic_tree);
  // the seam's aval is indexed by nlist sources directly
  int64_t nz = 0;
  for (size_t k = 0; k < ak->st.nlist.size(); k += 2) nz = std::max<int64_t>(nz, ak->st.nlist[k]);
  ak->clean.src.resize(nz);
  for (int64_t k = 0; k < nz; ++k) ak->clean.src[k] = k;
  ak->clean.srcptr.assign(1, 0);
  // scaling is indexed by the tree's variables, which are this handle's user
  // order (identity permutation at this seam)
  factorize_common(posdef, aval, nullptr, const_cast<double*>(scaling), ak, &fk, &o, &inf,
                   SYLVER_GB300_FP64, 1e-14, 0);
  if (inform) {
    std::memset(inform, 0, sizeof(*inform));
    inform->flag = inf.flag;
    inform->num_delay = inf.num_delay;
    inform->num_neg = inf.num_neg;
    inform->num_two = inf.num_two;
    inform->maxfront = inf.maxfront;
    if (fk) {
      inform->num_zero = static_cast<FKeep*>(fk)->num_zero;
      inform->not_first_pass = static_cast<FKeep*>(fk)->not_first_pass;
      inform->not_second_pass = static_cast<FKeep*>(fk)->not_second_pass;
    }
  }
  return fk;
}

void* spldlt_create_numeric_tree_posdef_dbl(void* fkeep, void* symbolic_tree, double* aval,
                                            const double* scaling, void** child_contrib,
                                            sylver_options_c* options, sylver_inform_c* inform) {
  return spldlt_create_numeric_tree_dbl(true, fkeep, symbolic_tree, aval, scaling,
                                        child_contrib, options, inform);
}

void spldlt_destroy_numeric_tree_dbl(bool posdef, void* tree) {
  (void)posdef;
  delete static_cast<FKeep*>(tree);
}

void spldlt_destroy_numeric_tree_posdef_dbl(void* tree) { delete static_cast<FKeep*>(tree); }

static int tree_solve(bool posdef, void const* tree, int nrhs, double* x, int ldx, int job) {
  const FKeep* cfk = static_cast<const FKeep*>(tree);
  if (!cfk || nrhs < 1) return SYLVER_ERROR_UNKNOWN;
  if (posdef && (job == 2 || job == 4)) return SYLVER_ERROR_JOB_OOR;
  FKeep* fk = const_cast<FKeep*>(cfk);
  try {
    Runtime& rt = Runtime::get();
    int n = fk->ak->n;
    DevMem tmp;
    tmp.ensure((size_t)n * nrhs * sizeof(double));
    SG_CUDA(cudaMemcpy2DAsync(tmp.p, n * sizeof(double), x, (size_t)ldx * sizeof(double),
                              n * sizeof(double), nrhs, cudaMemcpyHostToDevice, rt.stream));
    // the symbolic seam has identity permutation, so user order = pivot order
    int rc = fk->solve_raw(job, nrhs, tmp.as<double>(), n, rt.stream);
    SG_CUDA(cudaMemcpy2DAsync(x, (size_t)ldx * sizeof(double), tmp.p, n * sizeof(double),
                              n * sizeof(double), nrhs, cudaMemcpyDeviceToHost, rt.stream));
    SG_CUDA(cudaStreamSynchronize(rt.stream));
    return rc;
  } catch (const std::bad_alloc&) {
    return SYLVER_ERROR_ALLOCATION;
  } catch (const std::exception&) {
    return SYLVER_ERROR_CUDA_UNKNOWN;
  }
}

int spldlt_tree_solve_fwd_dbl(bool posdef, void const* tree, int nrhs, double* x, int ldx) {
  return tree_solve(posdef, tree, nrhs, x, ldx, SYLVER_SOLVE_JOB_FWD);
}
int spldlt_tree_solve_bwd_dbl(bool posdef, void const* tree, int nrhs, double* x, int ldx) {
  return tree_solve(posdef, tree, nrhs, x, ldx, SYLVER_SOLVE_JOB_BWD);
}
int spldlt_tree_solve_diag_dbl(bool posdef, void const* tree, int nrhs, double* x, int ldx) {
  return tree_solve(posdef, tree, nrhs, x, ldx, SYLVER_SOLVE_JOB_DIAG);
}
int spldlt_tree_solve_diag_bwd_dbl(bool posdef, void const* tree, int nrhs, double* x, int ldx) {
  return tree_solve(posdef, tree, nrhs, x, ldx, SYLVER_SOLVE_JOB_DIAG_BWD);
}
int spldlt_tree_solve_fwd_posdef_dbl(void const* tree, int nrhs, double* x, int ldx) {
  return tree_solve(true, tree, nrhs, x, ldx, SYLVER_SOLVE_JOB_FWD);
}
int spldlt_tree_solve_bwd_posdef_dbl(void const* tree, int nrhs, double* x, int ldx) {
  return tree_solve(true, tree, nrhs, x, ldx, SYLVER_SOLVE_JOB_BWD);
}

}  // extern "C"

extern "C" {

void sylver_gb300_set_schedule(sylver_gb300_schedule_t const* s) {
  Schedule& c = Schedule::current();
  c = Schedule();
  if (!s) return;
  c.small_front_rows = s->small_front_rows;
  c.tc_min_cb_rows = s->tc_min_cb_rows;
  c.solve_large_cols = s->solve_large_cols;
  c.ldlt_tpp_cols = s->ldlt_tpp_cols;
  c.fs_panel_cols = s->fs_panel_cols;
  c.fs_panel_group = s->fs_panel_group;
  c.front_memory = s->front_memory;
  c.solve_dataflow = s->solve_dataflow;
}

void sylver_gb300_get_schedule(sylver_gb300_schedule_t* s) {
  if (!s) return;
  const Schedule& c = Schedule::current();
  s->small_front_rows = c.small_front_rows;
  s->tc_min_cb_rows = c.tc_min_cb_rows;
  s->solve_large_cols = c.solve_large_cols;
  s->ldlt_tpp_cols = c.ldlt_tpp_cols;
  s->fs_panel_cols = c.fs_panel_cols;
  s->fs_panel_group = c.fs_panel_group;
  s->front_memory = c.front_memory;
  s->solve_dataflow = c.solve_dataflow;
}

}  // extern "C"
