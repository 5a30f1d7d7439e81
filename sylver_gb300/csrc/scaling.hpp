// Scalings and the matching-based ordering of the analysis / factorize
// phases (host).
//
// The reference takes these from SPRAL (spral_scaling: hungarian_scale_sym,
// auction_scale_sym, equilib_scale_sym; spral_match_order:
// match_order_metis), called at src/spldlt_factorize_mod.F90:727-830 and
// src/spldlt_analyse_mod.F90:787-816.  SPRAL is not vendored; these are
// restatements of the published methods:
//   * maximum-product matching with dual variables, symmetric scaling
//     (Duff & Koster, SIMAX 2001 -- the MC64 approach; Duff & Pralet, SIMAX
//     2005 for the symmetric scaling s_i = exp((u_i + v_i - log a_max,i)/2));
//   * the matching's cycles split into 1x1 and 2x2 blocks, the graph
//     compressed over the 2x2 pairs and ordered by nested dissection, pairs
//     kept adjacent (Duff & Pralet 2005; Hogg & Scott, RAL-TR-2008-021);
//   * infinity-norm equilibration by repeated symmetric row/column scaling
//     (Ruiz, RAL-TR-2001-034; the MC77 method).
#pragma once

#include <cstdint>
#include <vector>

namespace sylver_gb300 {

// Full symmetric matrix in 0-based CSC (both triangles).
struct SymCsc {
  int n = 0;
  std::vector<int64_t> ptr;
  std::vector<int> row;
  std::vector<double> val;
};

// Build the full symmetric CSC from a lower-triangle CSC (0-based) whose
// entry k has value lval[k].
SymCsc expand_lower(int n, const std::vector<int64_t>& cptr, const std::vector<int>& crow,
                    const std::vector<double>& lval);

// Maximum-product matching.  match[j] = row matched to column j (-1 if the
// matrix is structurally singular and j stays unmatched); scale = symmetric
// scaling with |s_i a_ij s_j| <= 1 and 1 on the matched entries (unmatched
// variables get 1).  Returns 0, or 1 when structurally singular.
int matching_scaling(const SymCsc& a, std::vector<int>& match, std::vector<double>& scale);

// Infinity-norm equilibration: |s_i a_ij s_j| <= 1 with every row's maximum
// near 1 after `iters` sweeps.
void equilibration_scaling(const SymCsc& a, std::vector<double>& scale, int iters = 20);

// Matching-based ordering: pairs from the matching's cycles, compressed
// graph ordered by nested dissection, each pair given consecutive positions.
// Returns order[i] = pivot position (0-based) of variable i.
std::vector<int> matching_order(const SymCsc& a, const std::vector<int>& match);

}  // namespace sylver_gb300
