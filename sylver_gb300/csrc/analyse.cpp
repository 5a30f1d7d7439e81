// Symbolic analysis: matrix check/clean, ordering, elimination tree, column
// counts, supernode amalgamation, row lists and the A->front map.
//
// Produces the arrays the reference feeds to spldlt_create_symbolic_tree
// (src/SymbolicTree.cxx:110-137): sptr, sparent, rptr, rlist, nptr, nlist.
// The reference computes them with SPRAL's basic_analyse and its own
// build_map (src/spldlt_analyse_mod.F90:130-232); SPRAL is not vendored, so
// this file restates the published algorithms:
//   * elimination tree with path compression (J. Liu, 1986);
//   * column counts by row-subtree leaves / least common ancestors
//     (Gilbert, Ng & Peyton, SIMAX 1994);
//   * fundamental supernodes plus nemin amalgamation (merge a child into its
//     parent when both eliminate fewer than nemin columns, SSIDS's rule);
//   * the A->front map with the layout of build_map: dest = col*nrow + row
//     inside the nrow x ncol front, both 1-based.
#include "analyse.hpp"

#include <algorithm>
#include <cstring>
#include <numeric>
#include <stdexcept>

namespace sylver_gb300 {

namespace {

enum {
  FLAG_SUCCESS = 0,
  ERROR_A_N_OOR = -2,
  ERROR_A_PTR = -3,
  ERROR_A_ALL_OOR = -4,
  ERROR_ORDER = -8,
  WARNING_IDX_OOR = 1,
  WARNING_DUP_IDX = 2,
  WARNING_DUP_AND_OOR = 3,
  WARNING_MISSING_DIAGONAL = 4,
  WARNING_MISS_DIAG_OORDUP = 5,
};

// Symmetric adjacency (no diagonal) of a 0-based lower CSC pattern.
void build_adjacency(int n, const std::vector<int64_t>& cptr, const std::vector<int>& crow,
                     std::vector<int64_t>& xadj, std::vector<int>& adj) {
  std::vector<int64_t> cnt(n + 1, 0);
  for (int j = 0; j < n; ++j)
    for (int64_t k = cptr[j]; k < cptr[j + 1]; ++k) {
      int i = crow[k];
      if (i == j) continue;
      cnt[i + 1]++;
      cnt[j + 1]++;
    }
  xadj.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) xadj[i + 1] = xadj[i] + cnt[i + 1];
  adj.assign(xadj[n], 0);
  std::vector<int64_t> pos(xadj.begin(), xadj.end() - 1);
  for (int j = 0; j < n; ++j)
    for (int64_t k = cptr[j]; k < cptr[j + 1]; ++k) {
      int i = crow[k];
      if (i == j) continue;
      adj[pos[i]++] = j;
      adj[pos[j]++] = i;
    }
}

// Relabel a graph: vertex v becomes p[v].
void permute_graph(int n, const std::vector<int64_t>& xadj, const std::vector<int>& adj,
                   const std::vector<int>& p, std::vector<int64_t>& nx, std::vector<int>& na) {
  std::vector<int> ip(n);
  for (int v = 0; v < n; ++v) ip[p[v]] = v;
  nx.assign(n + 1, 0);
  for (int w = 0; w < n; ++w) {
    int v = ip[w];
    nx[w + 1] = nx[w] + (xadj[v + 1] - xadj[v]);
  }
  na.assign(nx[n], 0);
  for (int w = 0; w < n; ++w) {
    int v = ip[w];
    int64_t o = nx[w];
    for (int64_t k = xadj[v]; k < xadj[v + 1]; ++k) na[o++] = p[adj[k]];
    std::sort(na.begin() + nx[w], na.begin() + nx[w + 1]);
  }
}

// Elimination tree (Liu) of a symmetric pattern given as full adjacency.
std::vector<int> etree(int n, const std::vector<int64_t>& xadj, const std::vector<int>& adj) {
  std::vector<int> parent(n, -1), anc(n, -1);
  for (int j = 0; j < n; ++j) {
    for (int64_t k = xadj[j]; k < xadj[j + 1]; ++k) {
      int r = adj[k];
      if (r >= j) continue;
      while (anc[r] != -1 && anc[r] != j) {
        int t = anc[r];
        anc[r] = j;
        r = t;
      }
      if (anc[r] == -1) {
        anc[r] = j;
        parent[r] = j;
      }
    }
  }
  return parent;
}

// Postorder of a forest; children visited in increasing index.
std::vector<int> postorder(int n, const std::vector<int>& parent) {
  std::vector<int> head(n, -1), next(n, -1);
  for (int j = n - 1; j >= 0; --j) {
    if (parent[j] == -1) continue;
    next[j] = head[parent[j]];
    head[parent[j]] = j;
  }
  std::vector<int> post;
  post.reserve(n);
  std::vector<int> stack;
  for (int r = 0; r < n; ++r) {
    if (parent[r] != -1) continue;
    stack.push_back(r);
    while (!stack.empty()) {
      int v = stack.back();
      if (head[v] != -1) {
        int c = head[v];
        head[v] = next[c];
        stack.push_back(c);
      } else {
        stack.pop_back();
        post.push_back(v);
      }
    }
  }
  return post;
}

// Column counts of L (diagonal included) for a postordered etree, after
// Gilbert, Ng & Peyton: each column's count is the number of row subtrees it
// belongs to, accumulated from leaf/LCA corrections.
std::vector<int64_t> column_counts(int n, const std::vector<int>& parent,
                                   const std::vector<int64_t>& xadj,
                                   const std::vector<int>& adj) {
  std::vector<int> first(n, -1), maxfirst(n, -1), prevleaf(n, -1), anc(n);
  std::vector<int64_t> delta(n, 0);
  for (int k = 0; k < n; ++k) {
    int j = k;
    delta[j] = (first[j] == -1) ? 1 : 0;
    while (j != -1 && first[j] == -1) {
      first[j] = k;
      j = parent[j];
    }
  }
  for (int i = 0; i < n; ++i) anc[i] = i;
  for (int j = 0; j < n; ++j) {
    if (parent[j] != -1) delta[parent[j]]--;
    for (int64_t p = xadj[j]; p < xadj[j + 1]; ++p) {
      int i = adj[p];
      if (i <= j || first[j] <= maxfirst[i]) continue;  // j not a leaf of row subtree i
      maxfirst[i] = first[j];
      int jprev = prevleaf[i];
      prevleaf[i] = j;
      delta[j]++;
      if (jprev == -1) continue;  // first leaf of row subtree i
      int q = jprev;
      while (q != anc[q]) q = anc[q];
      for (int s = jprev; s != q;) {
        int sp = anc[s];
        anc[s] = q;
        s = sp;
      }
      delta[q]--;  // q = lca(jprev, j)
    }
    if (parent[j] != -1) anc[j] = parent[j];
  }
  for (int j = 0; j < n; ++j)
    if (parent[j] != -1) delta[parent[j]] += delta[j];
  return delta;
}

}  // namespace

// ---------------------------------------------------------------------------

AnalyseResult clean_matrix(const AnalyseInput& in) {
  AnalyseResult res;
  int n = in.n;
  if (n < 0) {
    res.flag = ERROR_A_N_OOR;
    return res;
  }
  if (n == 0) {
    res.cptr.assign(1, 0);
    return res;
  }
  if (in.ptr[0] != 1) {
    res.flag = ERROR_A_PTR;
    return res;
  }
  for (int j = 0; j < n; ++j)
    if (in.ptr[j + 1] < in.ptr[j]) {
      res.flag = ERROR_A_PTR;
      return res;
    }
  int64_t nz = in.ptr[n] - 1;
  // gather (row, col, src) triples in the lower triangle
  struct Ent { int r, c; int64_t s; };
  std::vector<Ent> ents;
  ents.reserve(nz);
  int64_t oor = 0;
  for (int j = 0; j < n; ++j)
    for (int64_t k = in.ptr[j] - 1; k < in.ptr[j + 1] - 1; ++k) {
      int r = in.row[k] - 1;
      if (r < 0 || r >= n) {
        oor++;
        continue;
      }
      int c = j;
      if (r < c) {
        if (!in.check) {  // unchecked input must be lower triangular
          oor++;
          continue;
        }
        std::swap(r, c);
      }
      ents.push_back({r, c, k});
    }
  if (nz > 0 && ents.empty()) {
    res.flag = ERROR_A_ALL_OOR;
    return res;
  }
  std::stable_sort(ents.begin(), ents.end(), [](const Ent& a, const Ent& b) {
    return a.c != b.c ? a.c < b.c : a.r < b.r;
  });
  res.cptr.assign(n + 1, 0);
  res.srcptr.push_back(0);
  int64_t dup = 0;
  for (size_t k = 0; k < ents.size(); ++k) {
    bool same = k > 0 && ents[k].r == ents[k - 1].r && ents[k].c == ents[k - 1].c;
    if (same) {
      dup++;
    } else {
      if (k > 0) res.srcptr.push_back((int64_t)res.src.size());
      res.crow.push_back(ents[k].r);
      res.cptr[ents[k].c + 1]++;
    }
    res.src.push_back(ents[k].s);
  }
  res.srcptr.push_back((int64_t)res.src.size());
  for (int j = 0; j < n; ++j) res.cptr[j + 1] += res.cptr[j];
  int64_t missing = 0;
  for (int j = 0; j < n; ++j) {
    bool has = false;
    for (int64_t k = res.cptr[j]; k < res.cptr[j + 1]; ++k)
      if (res.crow[k] == j) has = true;
    if (!has) missing++;
  }
  res.matrix_outrange = (int)oor;
  res.matrix_dup = (int)dup;
  res.matrix_missing_diag = (int)missing;
  int flag = FLAG_SUCCESS;
  if (oor && dup) flag = WARNING_DUP_AND_OOR;
  else if (oor) flag = WARNING_IDX_OOR;
  else if (dup) flag = WARNING_DUP_IDX;
  if (missing) flag = (flag == FLAG_SUCCESS) ? WARNING_MISSING_DIAGONAL : WARNING_MISS_DIAG_OORDUP;
  res.flag = flag;
  return res;
}

// ---------------------------------------------------------------------------
// Nested dissection by breadth-first level structures: a pseudo-peripheral
// root, the level that best balances the two sides as separator, trimmed to
// the vertices that actually touch the far side.  Used when the caller does
// not supply an order (stand-in for METIS, which is not available).

std::vector<int> nested_dissection_order(int n, const std::vector<int64_t>& xadj,
                                         const std::vector<int>& adj) {
  std::vector<int> pos(n, -1);
  std::vector<int> lab(n, 0), lvl(n, -1);
  int next_label = 1;
  struct Task { std::vector<int> verts; int lo; int label; };
  std::vector<Task> stack;
  {
    std::vector<int> all(n);
    std::iota(all.begin(), all.end(), 0);
    stack.push_back({std::move(all), 0, 0});
  }
  const int leaf = 64;
  std::vector<int> queue;
  auto bfs = [&](int root, int label, std::vector<int>& order) {
    order.clear();
    order.push_back(root);
    lvl[root] = 0;
    for (size_t h = 0; h < order.size(); ++h) {
      int v = order[h];
      for (int64_t k = xadj[v]; k < xadj[v + 1]; ++k) {
        int w = adj[k];
        if (lab[w] != label || lvl[w] != -1) continue;
        lvl[w] = lvl[v] + 1;
        order.push_back(w);
      }
    }
  };
  while (!stack.empty()) {
    Task t = std::move(stack.back());
    stack.pop_back();
    auto& vs = t.verts;
    if ((int)vs.size() <= leaf) {
      for (size_t i = 0; i < vs.size(); ++i) pos[vs[i]] = t.lo + (int)i;
      continue;
    }
    for (int v : vs) lvl[v] = -1;
    bfs(vs[0], t.label, queue);
    if (queue.size() < vs.size()) {
      // disconnected: split into components, each its own sub-problem
      std::vector<std::vector<int>> comps;
      comps.push_back(queue);
      for (int v : vs)
        if (lvl[v] == -1) {
          bfs(v, t.label, queue);
          comps.push_back(queue);
        }
      int lo = t.lo;
      for (auto& c : comps) {
        int label = next_label++;
        for (int v : c) lab[v] = label;
        int sz = (int)c.size();
        stack.push_back({std::move(c), lo, label});
        lo += sz;
      }
      continue;
    }
    // pseudo-peripheral root: repeat BFS from a min-degree vertex of the last level
    int root = vs[0];
    int ecc = lvl[queue.back()];
    for (int it = 0; it < 4; ++it) {
      int last = lvl[queue.back()];
      int best = queue.back();
      int64_t bdeg = INT64_MAX;
      for (auto it2 = queue.rbegin(); it2 != queue.rend() && lvl[*it2] == last; ++it2) {
        int64_t d = xadj[*it2 + 1] - xadj[*it2];
        if (d < bdeg) { bdeg = d; best = *it2; }
      }
      for (int v : vs) lvl[v] = -1;
      bfs(best, t.label, queue);
      int e = lvl[queue.back()];
      if (e <= ecc && it > 0) break;
      ecc = e;
      root = best;
    }
    (void)root;
    int nl = lvl[queue.back()] + 1;
    std::vector<int64_t> cnt(nl, 0);
    for (int v : vs) cnt[lvl[v]]++;
    int64_t total = (int64_t)vs.size(), below = 0;
    int L = 1;
    int64_t bestbal = INT64_MAX;
    for (int l = 1; l < nl - 1; ++l) {
      below += cnt[l - 1];
      int64_t above = total - below - cnt[l];
      int64_t bal = std::llabs(below - above);
      if (bal < bestbal) { bestbal = bal; L = l; }
    }
    std::vector<int> p1, p2, sep;
    if (nl < 3) {
      for (size_t i = 0; i < vs.size(); ++i) pos[vs[i]] = t.lo + (int)i;
      continue;
    }
    for (int v : vs) {
      if (lvl[v] < L) p1.push_back(v);
      else if (lvl[v] > L) p2.push_back(v);
      else {
        bool touches = false;
        for (int64_t k = xadj[v]; k < xadj[v + 1]; ++k) {
          int w = adj[k];
          if (lab[w] == t.label && lvl[w] == L + 1) { touches = true; break; }
        }
        (touches ? sep : p1).push_back(v);
      }
    }
    if (p1.empty() || p2.empty()) {
      for (size_t i = 0; i < vs.size(); ++i) pos[vs[i]] = t.lo + (int)i;
      continue;
    }
    int lo = t.lo;
    int l1 = next_label++, l2 = next_label++;
    for (int v : p1) lab[v] = l1;
    for (int v : p2) lab[v] = l2;
    int s1 = (int)p1.size(), s2 = (int)p2.size();
    int slo = lo + s1 + s2;
    for (size_t i = 0; i < sep.size(); ++i) {
      pos[sep[i]] = slo + (int)i;
      lab[sep[i]] = -1;
    }
    stack.push_back({std::move(p1), lo, l1});
    stack.push_back({std::move(p2), lo + s1, l2});
  }
  return pos;
}

// ---------------------------------------------------------------------------

void SymbolicTree::derive() {
  nrow.assign(nnodes, 0);
  ncol.assign(nnodes, 0);
  children.assign(nnodes, {});
  level.assign(nnodes, 0);
  num_factor = 0;
  num_flops = 0;
  maxfront = 0;
  for (int s = 0; s < nnodes; ++s) {
    nrow[s] = (int)(rptr[s + 1] - rptr[s]);
    ncol[s] = sptr[s + 1] - sptr[s];
    int64_t m = nrow[s], c = ncol[s];
    num_factor += c * m - c * (c - 1) / 2;
    for (int64_t j = m - c + 1; j <= m; ++j) num_flops += j * j;
    maxfront = std::max(maxfront, nrow[s]);
  }
  for (int s = 0; s < nnodes; ++s) {
    int p = sparent[s] - 1;
    if (p >= 0 && p < nnodes) children[p].push_back(s);
  }
  // fronts are numbered in postorder, so children precede parents
  nlevels = 0;
  std::vector<int> depth(nnodes, 0);
  for (int s = 0; s < nnodes; ++s) {
    int h = 0;
    for (int c : children[s]) h = std::max(h, level[c] + 1);
    level[s] = h;
    nlevels = std::max(nlevels, h + 1);
  }
  maxdepth = 0;
  for (int s = nnodes - 1; s >= 0; --s) {
    int p = sparent[s] - 1;
    depth[s] = (p >= 0 && p < nnodes) ? depth[p] + 1 : 1;
    maxdepth = std::max(maxdepth, depth[s]);
  }
}

int analyse(const AnalyseInput& in, const AnalyseResult& clean, SymbolicTree& st,
            std::string& err) {
  const int n = in.n;
  st = SymbolicTree();
  st.n = n;
  if (n == 0) {
    st.nnodes = 0;
    st.sptr = {1};
    st.rptr = {1};
    st.nptr = {1};
    st.derive();
    return 0;
  }
  std::vector<int64_t> xadj;
  std::vector<int> adj;
  build_adjacency(n, clean.cptr, clean.crow, xadj, adj);

  // 1. initial ordering
  std::vector<int> p0(n);
  if (in.ordering == 0) {
    if (!in.order) {
      err = "ordering=0 needs a user order";
      return ERROR_ORDER;
    }
    std::vector<char> seen(n, 0);
    for (int i = 0; i < n; ++i) {
      int o = in.order[i] - 1;
      if (o < 0 || o >= n || seen[o]) {
        err = "order is not a permutation";
        return ERROR_ORDER;
      }
      seen[o] = 1;
      p0[i] = o;
    }
  } else {
    p0 = nested_dissection_order(n, xadj, adj);
  }

  // 2. elimination tree in the initial order, then postorder it
  std::vector<int64_t> x1;
  std::vector<int> a1;
  permute_graph(n, xadj, adj, p0, x1, a1);
  std::vector<int> par1 = etree(n, x1, a1);
  std::vector<int> post = postorder(n, par1);
  std::vector<int> ipost(n);
  for (int k = 0; k < n; ++k) ipost[post[k]] = k;
  std::vector<int> p2(n);  // variable -> postordered position
  for (int v = 0; v < n; ++v) p2[v] = ipost[p0[v]];
  std::vector<int> parent(n, -1);
  for (int j = 0; j < n; ++j)
    if (par1[j] != -1) parent[ipost[j]] = ipost[par1[j]];
  std::vector<int64_t> x2;
  std::vector<int> a2;
  permute_graph(n, xadj, adj, p2, x2, a2);

  // 3. column counts
  std::vector<int64_t> cc = column_counts(n, parent, x2, a2);

  // 4. supernodes: fundamental chains + nemin amalgamation, bottom-up
  const int nemin = std::max(1, in.nemin);
  std::vector<int> nch(n, 0);
  for (int j = 0; j < n; ++j)
    if (parent[j] != -1) nch[parent[j]]++;
  std::vector<std::vector<int>> kids(n);
  for (int j = 0; j < n; ++j)
    if (parent[j] != -1) kids[parent[j]].push_back(j);
  std::vector<int64_t> sn_nelim(n, 1), sn_nrow(n);
  std::vector<int> absorbed(n, -1);  // column rep -> absorbing rep
  for (int j = 0; j < n; ++j) sn_nrow[j] = cc[j];
  for (int p = 0; p < n; ++p) {
    for (int c : kids[p]) {
      bool fundamental = (nch[p] == 1) && (sn_nrow[c] - sn_nelim[c] == cc[p]);
      bool small = sn_nelim[c] < nemin && sn_nelim[p] < nemin;
      if (fundamental || small) {
        absorbed[c] = p;
        sn_nrow[p] = std::max(sn_nrow[p] + sn_nelim[c], sn_nrow[c]);
        sn_nelim[p] += sn_nelim[c];
      }
    }
  }
  // representative (top column) of every column's supernode
  std::vector<int> rep(n);
  for (int j = n - 1; j >= 0; --j) rep[j] = (absorbed[j] == -1) ? j : rep[absorbed[j]];
  // supernode tree over representatives; postorder it
  std::vector<int> sidx(n, -1);
  std::vector<int> reps;
  for (int j = 0; j < n; ++j)
    if (rep[j] == j) {
      sidx[j] = (int)reps.size();
      reps.push_back(j);
    }
  int ns = (int)reps.size();
  std::vector<int> spar(ns, -1);
  for (int s = 0; s < ns; ++s) {
    int r = reps[s];
    if (parent[r] != -1) spar[s] = sidx[rep[parent[r]]];
  }
  std::vector<int> spost = postorder(ns, spar);
  std::vector<int> ispost(ns);
  for (int k = 0; k < ns; ++k) ispost[spost[k]] = k;
  // columns of each supernode (ascending postordered index)
  std::vector<std::vector<int>> scols(ns);
  for (int j = 0; j < n; ++j) scols[ispost[sidx[rep[j]]]].push_back(j);
  std::vector<int> p3(n);  // postordered position -> final position
  st.nnodes = ns;
  st.sptr.assign(ns + 1, 1);
  {
    int k = 0;
    for (int s = 0; s < ns; ++s) {
      st.sptr[s] = k + 1;
      for (int j : scols[s]) p3[j] = k++;
    }
    st.sptr[ns] = k + 1;
  }
  st.sparent.assign(ns, ns + 1);
  for (int s = 0; s < ns; ++s) {
    int old = spost[s];
    st.sparent[s] = (spar[old] == -1) ? ns + 1 : ispost[spar[old]] + 1;
  }
  st.perm.assign(n, 0);
  st.invp.assign(n, 0);
  for (int v = 0; v < n; ++v) {
    st.perm[v] = p3[p2[v]];
    st.invp[st.perm[v]] = v;
  }

  // 5. row lists by merging children's contribution rows with A's pattern
  std::vector<int64_t> xf;
  std::vector<int> af;
  permute_graph(n, xadj, adj, st.perm, xf, af);
  std::vector<std::vector<int>> skids(ns);
  for (int s = 0; s < ns; ++s)
    if (st.sparent[s] <= ns) skids[st.sparent[s] - 1].push_back(s);
  std::vector<int> mark(n, -1);
  st.rptr.assign(ns + 1, 1);
  st.rlist.clear();
  std::vector<int> extra;
  for (int s = 0; s < ns; ++s) {
    int sa = st.sptr[s] - 1, en = st.sptr[s + 1] - 1;
    st.rptr[s] = (int64_t)st.rlist.size() + 1;
    extra.clear();
    for (int j = sa; j < en; ++j)
      for (int64_t k = xf[j]; k < xf[j + 1]; ++k) {
        int i = af[k];
        if (i >= en && mark[i] != s) {
          mark[i] = s;
          extra.push_back(i);
        }
      }
    for (int c : skids[s]) {
      int64_t r0 = st.rptr[c] - 1 + (st.sptr[c + 1] - st.sptr[c]);
      int64_t r1 = st.rptr[c + 1] - 1;
      for (int64_t k = r0; k < r1; ++k) {
        int i = st.rlist[k] - 1;
        if (i >= en && mark[i] != s) {
          mark[i] = s;
          extra.push_back(i);
        }
      }
    }
    std::sort(extra.begin(), extra.end());
    for (int j = sa; j < en; ++j) st.rlist.push_back(j + 1);
    for (int i : extra) st.rlist.push_back(i + 1);
  }
  st.rptr[ns] = (int64_t)st.rlist.size() + 1;

  // 6. A -> front map (build_map layout): one pair per original entry
  std::vector<int> snode_of(n);
  for (int s = 0; s < ns; ++s)
    for (int j = st.sptr[s] - 1; j < st.sptr[s + 1] - 1; ++j) snode_of[j] = s;
  struct Pair { int64_t src, dest; };
  std::vector<std::vector<Pair>> per(ns);
  std::vector<int> loc(n, -1);
  // bucket clean entries by front first, then resolve local rows per front
  std::vector<std::vector<int64_t>> bucket(ns);
  for (int c = 0; c < n; ++c)
    for (int64_t k = clean.cptr[c]; k < clean.cptr[c + 1]; ++k) {
      int r = clean.crow[k];
      int pr = st.perm[r], pc = st.perm[c];
      int lo = std::min(pr, pc);
      bucket[snode_of[lo]].push_back(k);
    }
  st.nptr.assign(ns + 1, 1);
  st.nlist.clear();
  for (int s = 0; s < ns; ++s) {
    int sa = st.sptr[s] - 1;
    int m = (int)(st.rptr[s + 1] - st.rptr[s]);
    for (int64_t k = st.rptr[s] - 1; k < st.rptr[s + 1] - 1; ++k)
      loc[st.rlist[k] - 1] = (int)(k - (st.rptr[s] - 1));
    std::vector<Pair> pairs;
    for (int64_t k : bucket[s]) {
      // recover column of clean entry k
      int r = clean.crow[k];
      int c = (int)(std::upper_bound(clean.cptr.begin(), clean.cptr.end(), k) - clean.cptr.begin()) - 1;
      int pr = st.perm[r], pc = st.perm[c];
      int lo = std::min(pr, pc), hi = std::max(pr, pc);
      int64_t dest = (int64_t)(lo - sa) * m + loc[hi];
      for (int64_t q = clean.srcptr[k]; q < clean.srcptr[k + 1]; ++q)
        pairs.push_back({clean.src[q], dest});
    }
    std::sort(pairs.begin(), pairs.end(), [](const Pair& a, const Pair& b) {
      return a.dest != b.dest ? a.dest < b.dest : a.src < b.src;
    });
    st.nptr[s] = (int64_t)st.nlist.size() / 2 + 1;
    for (auto& pq : pairs) {
      st.nlist.push_back(pq.src + 1);
      st.nlist.push_back(pq.dest + 1);
    }
  }
  st.nptr[ns] = (int64_t)st.nlist.size() / 2 + 1;
  st.derive();
  return 0;
}

}  // namespace sylver_gb300
