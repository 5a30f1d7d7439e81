// Symbolic analysis producing the reference's SymbolicTree input arrays.
//
// The reference obtains these arrays from SPRAL's basic_analyse + METIS and
// its own build_map (src/spldlt_analyse_mod.F90:130-232, :307-580) and hands
// them to spldlt_create_symbolic_tree (src/SymbolicTree.cxx:110-137).  All
// index arrays keep the reference's 1-based (Fortran) convention so that a
// caller holding SPRAL output can pass it straight through.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace sylver_gb300 {

struct SymbolicTree {
  int n = 0;
  int nnodes = 0;
  std::vector<int> sptr;      // nnodes+1, 1-based first pivot of each front
  std::vector<int> sparent;   // nnodes, 1-based; roots point at nnodes+1
  std::vector<int64_t> rptr;  // nnodes+1, 1-based into rlist
  std::vector<int> rlist;     // 1-based pivot-order row indices per front
  std::vector<int64_t> nptr;  // nnodes+1, 1-based into nlist pairs
  std::vector<int64_t> nlist; // 2 per entry: (src in val, dest in nrow x ncol), 1-based
  std::vector<int> perm;      // perm[i]  = pivot position (0-based) of variable i
  std::vector<int> invp;      // invp[k]  = variable (0-based) at pivot position k

  // derived (0-based helpers)
  std::vector<int> nrow, ncol;            // per front
  std::vector<std::vector<int>> children; // per front (0-based)
  std::vector<int> level;                 // height from leaves (leaf = 0)
  int nlevels = 0;

  // statistics (reference inform fields)
  int64_t num_factor = 0;  // entries in L
  int64_t num_flops = 0;   // compute_flops convention
  int maxfront = 0;
  int maxdepth = 0;

  void derive();           // fill nrow/ncol/children/level and stats
};

// Matrix as handed to spldlt_analyse: lower-triangle CSC, 1-based ptr/row.
struct AnalyseInput {
  int n;
  const int64_t* ptr;
  const int* row;
  const int* order;  // optional user order (1-based positions), may be null
  bool check;
  int ordering;      // 0: user order, otherwise internal nested dissection
  int nemin;
};

struct AnalyseResult {
  int flag = 0;  // reference SYLVER_* flag
  int matrix_outrange = 0, matrix_dup = 0, matrix_missing_diag = 0;
  // cleaned matrix in 0-based lower CSC with a map to original val slots:
  // entry k of the clean matrix sums val[src[srcptr[k]..srcptr[k+1])]
  std::vector<int64_t> cptr;
  std::vector<int> crow;
  std::vector<int64_t> srcptr;
  std::vector<int64_t> src;
};

// Validate/clean the matrix (checks mirror SPRAL's check of ptr/row input).
AnalyseResult clean_matrix(const AnalyseInput& in);

// Full symbolic analysis. Returns reference flag (0 ok, <0 error, >0 warning).
int analyse(const AnalyseInput& in, const AnalyseResult& clean, SymbolicTree& st,
            std::string& err);

// Internal nested dissection on the adjacency graph of the clean matrix.
std::vector<int> nested_dissection_order(int n, const std::vector<int64_t>& xadj,
                                         const std::vector<int>& adj);

}  // namespace sylver_gb300
