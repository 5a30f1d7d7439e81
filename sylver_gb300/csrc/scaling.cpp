// Scalings and the matching-based ordering (see scaling.hpp for the methods
// and the reference call sites).
#include "scaling.hpp"

#include <algorithm>
#include <cmath>
#include <functional>
#include <limits>
#include <numeric>
#include <queue>

#include "analyse.hpp"

namespace sylver_gb300 {

SymCsc expand_lower(int n, const std::vector<int64_t>& cptr, const std::vector<int>& crow,
                    const std::vector<double>& lval) {
  SymCsc a;
  a.n = n;
  std::vector<int64_t> cnt(n + 1, 0);
  for (int c = 0; c < n; ++c)
    for (int64_t k = cptr[c]; k < cptr[c + 1]; ++k) {
      int r = crow[k];
      cnt[c + 1]++;
      if (r != c) cnt[r + 1]++;
    }
  a.ptr.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) a.ptr[i + 1] = a.ptr[i] + cnt[i + 1];
  a.row.assign(a.ptr[n], 0);
  a.val.assign(a.ptr[n], 0.0);
  std::vector<int64_t> pos(a.ptr.begin(), a.ptr.end() - 1);
  for (int c = 0; c < n; ++c)
    for (int64_t k = cptr[c]; k < cptr[c + 1]; ++k) {
      int r = crow[k];
      a.row[pos[c]] = r;
      a.val[pos[c]++] = lval[k];
      if (r != c) {
        a.row[pos[r]] = c;
        a.val[pos[r]++] = lval[k];
      }
    }
  return a;
}

int matching_scaling(const SymCsc& a, std::vector<int>& match, std::vector<double>& scale) {
  const int n = a.n;
  const double inf = std::numeric_limits<double>::infinity();
  // cost c_ij = log(max_i |a_ij|) - log |a_ij| >= 0 (zeros are not edges)
  std::vector<double> lmax(n, -inf), cost(a.row.size(), inf);
  for (int j = 0; j < n; ++j)
    for (int64_t k = a.ptr[j]; k < a.ptr[j + 1]; ++k)
      if (a.val[k] != 0.0) lmax[j] = std::max(lmax[j], std::log(std::fabs(a.val[k])));
  for (int j = 0; j < n; ++j)
    for (int64_t k = a.ptr[j]; k < a.ptr[j + 1]; ++k)
      if (a.val[k] != 0.0) cost[k] = lmax[j] - std::log(std::fabs(a.val[k]));
  // duals: rows u, columns v; reduced cost c_ij - u_i - v_j >= 0, tight on
  // matched edges.  v = 0, u_i = min over row i (= column i, symmetric).
  std::vector<double> u(n, inf), v(n, 0.0);
  for (int j = 0; j < n; ++j)
    for (int64_t k = a.ptr[j]; k < a.ptr[j + 1]; ++k)
      if (cost[k] < inf) u[a.row[k]] = std::min(u[a.row[k]], cost[k]);
  for (int i = 0; i < n; ++i)
    if (u[i] == inf) u[i] = 0.0;
  std::vector<int> row_of_col(n, -1), col_of_row(n, -1);
  // cheap start: tight edges to free rows
  for (int j = 0; j < n; ++j)
    for (int64_t k = a.ptr[j]; k < a.ptr[j + 1]; ++k) {
      const int i = a.row[k];
      if (cost[k] < inf && col_of_row[i] < 0 && cost[k] - u[i] - v[j] <= 0.0) {
        row_of_col[j] = i;
        col_of_row[i] = j;
        break;
      }
    }
  // shortest augmenting paths (Dijkstra on reduced costs) from each free column
  std::vector<double> dist(n, inf);
  std::vector<int> pred(n, -1), visited;
  std::vector<char> done(n, 0);
  using QE = std::pair<double, int>;
  bool singular = false;
  for (int j0 = 0; j0 < n; ++j0) {
    if (row_of_col[j0] >= 0) continue;
    std::priority_queue<QE, std::vector<QE>, std::greater<QE>> pq;
    std::vector<int> touched;
    auto relax = [&](int j, double base) {
      for (int64_t k = a.ptr[j]; k < a.ptr[j + 1]; ++k) {
        if (cost[k] == inf) continue;
        const int i = a.row[k];
        if (done[i]) continue;
        const double nd = base + std::max(cost[k] - u[i] - v[j], 0.0);
        if (nd < dist[i]) {
          if (dist[i] == inf) touched.push_back(i);
          dist[i] = nd;
          pred[i] = j;
          pq.push({nd, i});
        }
      }
    };
    relax(j0, 0.0);
    int sink = -1;
    double Lsink = 0.0;
    visited.clear();
    while (!pq.empty()) {
      auto [d, i] = pq.top();
      pq.pop();
      if (done[i] || d > dist[i]) continue;
      done[i] = 1;
      visited.push_back(i);
      if (col_of_row[i] < 0) {
        sink = i;
        Lsink = d;
        break;
      }
      relax(col_of_row[i], d);
    }
    if (sink < 0) {
      singular = true;
    } else {
      // dual update: finalized rows i (all visited but the sink) and the
      // columns of their matched edges, then j0
      v[j0] += Lsink;
      for (int i : visited) {
        if (i == sink) continue;
        const double delta = Lsink - dist[i];
        u[i] -= delta;
        v[col_of_row[i]] += delta;
      }
      // augment along the predecessor chain
      int i = sink;
      while (true) {
        const int j = pred[i];
        const int inext = row_of_col[j];
        row_of_col[j] = i;
        col_of_row[i] = j;
        if (j == j0) break;
        i = inext;
      }
    }
    for (int i : touched) {
      dist[i] = inf;
      pred[i] = -1;
      done[i] = 0;
    }
  }
  match = row_of_col;
  scale.assign(n, 1.0);
  for (int i = 0; i < n; ++i)
    if (row_of_col[i] >= 0 && lmax[i] > -inf) scale[i] = std::exp(0.5 * (u[i] + v[i] - lmax[i]));
  return singular ? 1 : 0;
}

void equilibration_scaling(const SymCsc& a, std::vector<double>& scale, int iters) {
  const int n = a.n;
  scale.assign(n, 1.0);
  std::vector<double> r(n);
  for (int it = 0; it < iters; ++it) {
    std::fill(r.begin(), r.end(), 0.0);
    for (int j = 0; j < n; ++j)
      for (int64_t k = a.ptr[j]; k < a.ptr[j + 1]; ++k) {
        const int i = a.row[k];
        r[j] = std::max(r[j], std::fabs(scale[i] * a.val[k] * scale[j]));
      }
    double worst = 0.0;
    for (int i = 0; i < n; ++i) {
      if (r[i] > 0.0) scale[i] /= std::sqrt(r[i]);
      worst = std::max(worst, std::fabs(1.0 - r[i]));
    }
    if (worst < 1e-2) break;
  }
}

std::vector<int> matching_order(const SymCsc& a, const std::vector<int>& match) {
  const int n = a.n;
  // sigma: column j matched with row match[j] -- a permutation of the
  // variables for a symmetric matrix; split its cycles into pairs
  std::vector<int> comp(n, -1);
  int nc = 0;
  std::vector<char> seen(n, 0);
  for (int s = 0; s < n; ++s) {
    if (seen[s]) continue;
    std::vector<int> cyc;
    int j = s;
    while (j >= 0 && !seen[j]) {
      seen[j] = 1;
      cyc.push_back(j);
      j = match[j];
    }
    size_t k = 0;
    for (; k + 1 < cyc.size(); k += 2) {
      comp[cyc[k]] = nc;
      comp[cyc[k + 1]] = nc;
      nc++;
    }
    if (k < cyc.size()) comp[cyc[k]] = nc++;
  }
  // compressed graph: union of the members' neighbours
  std::vector<std::vector<int>> members(nc);
  for (int i = 0; i < n; ++i) members[comp[i]].push_back(i);
  std::vector<int64_t> xadj(nc + 1, 0);
  std::vector<int> adj, mark(nc, -1);
  for (int c = 0; c < nc; ++c) {
    for (int i : members[c])
      for (int64_t k = a.ptr[i]; k < a.ptr[i + 1]; ++k) {
        const int d = comp[a.row[k]];
        if (d == c || mark[d] == c) continue;
        mark[d] = c;
        adj.push_back(d);
      }
    xadj[c + 1] = (int64_t)adj.size();
  }
  std::vector<int> pc = nested_dissection_order(nc, xadj, adj);
  std::vector<int> byp(nc);
  for (int c = 0; c < nc; ++c) byp[pc[c]] = c;
  std::vector<int> order(n);
  int pos = 0;
  for (int q = 0; q < nc; ++q)
    for (int i : members[byp[q]]) order[i] = pos++;
  return order;
}

}  // namespace sylver_gb300
