// Symbolic analysis of the multifrontal LU: nested-dissection ordering by
// recursive coordinate bisection and the front structure of every node.
#include <algorithm>
#include <cmath>
#include <functional>

#include "mf.h"

namespace sucem {

namespace {

struct ND {
  const int32_t* indptr;
  const int32_t* indices;
  const double* xyz;
  int leaf;
  std::vector<int> mark;     // side of a variable in the current split
  std::vector<int> gen;      // generation stamp of mark
  int cur = 0;
  std::vector<int64_t> order;  // new -> old
  std::vector<MFNode> nodes;

  int make_node(const std::vector<int64_t>& vars, const std::vector<int>& children) {
    MFNode nd;
    nd.start = (int64_t)order.size();
    for (int64_t v : vars) order.push_back(v);
    nd.end = (int64_t)order.size();
    nd.k = nd.end - nd.start;
    nd.children = children;
    int lvl = 0;
    for (int c : children) lvl = std::max(lvl, nodes[c].level + 1);
    nd.level = lvl;
    nodes.push_back(nd);
    int id = (int)nodes.size() - 1;
    for (int c : children) nodes[c].parent = id;
    return id;
  }

  // returns node id, or -1 for an empty set
  int build(std::vector<int64_t>& vars) {
    if (vars.empty()) return -1;
    if ((int64_t)vars.size() <= leaf) return make_node(vars, {});
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t v : vars)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], xyz[3 * v + d]);
        hi[d] = std::max(hi[d], xyz[3 * v + d]);
      }
    int axis = 0;
    for (int d = 1; d < 3; ++d)
      if (hi[d] - lo[d] > hi[axis] - lo[axis]) axis = d;
    const size_t mid = vars.size() / 2;
    std::nth_element(vars.begin(), vars.begin() + mid, vars.end(), [&](int64_t a, int64_t b) {
      const double xa = xyz[3 * a + axis], xb = xyz[3 * b + axis];
      return xa < xb || (xa == xb && a < b);
    });
    ++cur;
    for (size_t i = 0; i < vars.size(); ++i) {
      mark[vars[i]] = i < mid ? 1 : 2;
      gen[vars[i]] = cur;
    }
    auto touches = [&](int64_t v, int other) {
      for (int32_t q = indptr[v]; q < indptr[v + 1]; ++q) {
        const int64_t w = indices[q];
        if (gen[w] == cur && mark[w] == other) return true;
      }
      return false;
    };
    std::vector<int64_t> sepL, sepR;
    for (size_t i = 0; i < vars.size(); ++i) {
      if (i < mid) {
        if (touches(vars[i], 2)) sepL.push_back(vars[i]);
      } else {
        if (touches(vars[i], 1)) sepR.push_back(vars[i]);
      }
    }
    const bool use_left = sepL.size() <= sepR.size();
    std::vector<int64_t>& sep = use_left ? sepL : sepR;
    if (sep.size() * 10 >= vars.size() * 9) return make_node(vars, {});  // no useful split
    ++cur;
    for (int64_t v : sep) {
      mark[v] = 3;
      gen[v] = cur;
    }
    std::vector<int64_t> left, right;
    for (size_t i = 0; i < vars.size(); ++i) {
      const int64_t v = vars[i];
      if (gen[v] == cur && mark[v] == 3) continue;
      (i < mid ? left : right).push_back(v);
    }
    std::vector<int64_t> sepv(sep.begin(), sep.end());
    std::vector<int64_t>().swap(vars);
    std::vector<int> kids;
    int a = build(left);
    if (a >= 0) kids.push_back(a);
    int b = build(right);
    if (b >= 0) kids.push_back(b);
    return make_node(sepv, kids);
  }
};

// Element-based nested dissection: the cells are bisected at the median of
// their centroids along the longest extent; the separator is the set of
// DOFs that belong to cells on both sides (the interface surface of the two
// cell sets), so DOFs left and right never share a cell.
struct CellND {
  const int64_t* dof_cell_ptr;   // DOF -> incident cells (CSR)
  const int32_t* dof_cells;
  const double* cxyz;            // cell centroids
  int leaf;
  std::vector<int> side, gen;    // per cell
  int cur = 0;
  ND* out;                       // node/order storage shared with ND

  int build(std::vector<int32_t>& C, std::vector<int64_t>& D) {
    if (D.empty()) return -1;
    if ((int64_t)D.size() <= leaf || C.size() <= 1) return out->make_node(D, {});
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int32_t c : C)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], cxyz[3 * (int64_t)c + d]);
        hi[d] = std::max(hi[d], cxyz[3 * (int64_t)c + d]);
      }
    int axis = 0;
    for (int d = 1; d < 3; ++d)
      if (hi[d] - lo[d] > hi[axis] - lo[axis]) axis = d;
    const size_t mid = C.size() / 2;
    std::nth_element(C.begin(), C.begin() + mid, C.end(), [&](int32_t a, int32_t b) {
      const double xa = cxyz[3 * (int64_t)a + axis], xb = cxyz[3 * (int64_t)b + axis];
      return xa < xb || (xa == xb && a < b);
    });
    ++cur;
    for (size_t i = 0; i < C.size(); ++i) {
      side[C[i]] = i < mid ? 1 : 2;
      gen[C[i]] = cur;
    }
    std::vector<int64_t> sep, D1, D2;
    for (int64_t d : D) {
      int seen = 0;
      for (int64_t q = dof_cell_ptr[d]; q < dof_cell_ptr[d + 1]; ++q) {
        const int32_t c = dof_cells[q];
        if (gen[c] == cur) seen |= side[c];
      }
      if (seen == 3)
        sep.push_back(d);
      else if (seen == 1)
        D1.push_back(d);
      else
        D2.push_back(d);
    }
    if (sep.size() * 10 >= D.size() * 9) return out->make_node(D, {});
    std::vector<int32_t> C1(C.begin(), C.begin() + mid), C2(C.begin() + mid, C.end());
    std::vector<int32_t>().swap(C);
    std::vector<int64_t>().swap(D);
    std::vector<int> kids;
    int a = build(C1, D1);
    if (a >= 0) kids.push_back(a);
    int b = build(C2, D2);
    if (b >= 0) kids.push_back(b);
    return out->make_node(sep, kids);
  }
};

}  // namespace

std::string mf_finish(MFSymbolic& sym, int64_t n, const int32_t* indptr, const int32_t* indices,
                      std::vector<int64_t>&& order, std::vector<MFNode>&& nodes);

std::string mf_analyse_cells(MFSymbolic& sym, int64_t n, const int32_t* indptr,
                             const int32_t* indices, int64_t nt, int nd, const int32_t* cell_dofs,
                             const double* cell_xyz, int leaf_size) {
  if (n <= 0) return "empty matrix";
  std::vector<int64_t> ptr(n + 1, 0);
  for (int64_t i = 0; i < nt * nd; ++i) {
    const int32_t d = cell_dofs[i];
    if (d >= n) return "cell DOF index out of range";
    if (d >= 0) ptr[d + 1]++;
  }
  for (int64_t d = 0; d < n; ++d) ptr[d + 1] += ptr[d];
  std::vector<int32_t> dc(ptr[n]);
  {
    std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
    for (int64_t c = 0; c < nt; ++c)
      for (int j = 0; j < nd; ++j) {
        const int32_t d = cell_dofs[c * nd + j];
        if (d >= 0) dc[fill[d]++] = (int32_t)c;
      }
  }
  ND store;
  store.order.reserve(n);
  CellND cn;
  cn.dof_cell_ptr = ptr.data();
  cn.dof_cells = dc.data();
  cn.cxyz = cell_xyz;
  cn.leaf = std::max(16, leaf_size);
  cn.side.assign(nt, 0);
  cn.gen.assign(nt, 0);
  cn.out = &store;
  std::vector<int32_t> C(nt);
  for (int64_t c = 0; c < nt; ++c) C[c] = (int32_t)c;
  // DOFs in no cell (possible for sub-matrices) go into their own leaf
  std::vector<int64_t> D, lonely;
  for (int64_t d = 0; d < n; ++d) (ptr[d + 1] > ptr[d] ? D : lonely).push_back(d);
  std::vector<int> roots;
  int r = cn.build(C, D);
  if (r >= 0) roots.push_back(r);
  if (!lonely.empty()) roots.push_back(store.make_node(lonely, {}));
  if (roots.size() > 1) {
    std::vector<int64_t> none;
    store.make_node(none, roots);
  }
  if ((int64_t)store.order.size() != n) return "ordering failed";
  return mf_finish(sym, n, indptr, indices, std::move(store.order), std::move(store.nodes));
}

// Pseudo-coordinates for a matrix without geometry: breadth-first distances
// from three far-apart vertices of each connected component (components
// are laid out one after another along the first axis).
static void graph_coordinates(int64_t n, const int32_t* indptr, const int32_t* indices,
                              std::vector<double>& xyz) {
  xyz.assign(n * 3, 0.0);
  std::vector<int64_t> dist(n, -1), comp_nodes, queue;
  std::vector<char> seen(n, 0);
  double offset = 0;
  auto bfs = [&](int64_t src, std::vector<int64_t>& d) {
    for (int64_t v : comp_nodes) d[v] = -1;
    queue.clear();
    queue.push_back(src);
    d[src] = 0;
    int64_t far = src;
    for (size_t h = 0; h < queue.size(); ++h) {
      const int64_t v = queue[h];
      if (d[v] > d[far]) far = v;
      for (int32_t q = indptr[v]; q < indptr[v + 1]; ++q) {
        const int64_t w = indices[q];
        if (d[w] < 0) {
          d[w] = d[v] + 1;
          queue.push_back(w);
        }
      }
    }
    return far;
  };
  for (int64_t s = 0; s < n; ++s) {
    if (seen[s]) continue;
    // collect the component
    comp_nodes.clear();
    comp_nodes.push_back(s);
    seen[s] = 1;
    for (size_t h = 0; h < comp_nodes.size(); ++h) {
      const int64_t v = comp_nodes[h];
      for (int32_t q = indptr[v]; q < indptr[v + 1]; ++q)
        if (!seen[indices[q]]) {
          seen[indices[q]] = 1;
          comp_nodes.push_back(indices[q]);
        }
    }
    std::vector<int64_t>& d = dist;
    const int64_t a = bfs(s, d);
    const int64_t b = bfs(a, d);
    std::vector<int64_t> d1(comp_nodes.size());
    for (size_t i = 0; i < comp_nodes.size(); ++i) d1[i] = d[comp_nodes[i]];
    const int64_t c = bfs(b, d);
    std::vector<int64_t> d2(comp_nodes.size());
    int64_t best = s;
    int64_t bestv = -1;
    for (size_t i = 0; i < comp_nodes.size(); ++i) {
      d2[i] = d[comp_nodes[i]];
      const int64_t mv = std::min(d1[i], d2[i]);
      if (mv > bestv) {
        bestv = mv;
        best = comp_nodes[i];
      }
    }
    (void)c;
    bfs(best, d);
    double span = 0;
    for (size_t i = 0; i < comp_nodes.size(); ++i) {
      const int64_t v = comp_nodes[i];
      xyz[3 * v] = offset + (double)d1[i];
      xyz[3 * v + 1] = (double)d2[i];
      xyz[3 * v + 2] = (double)d[v];
      span = std::max(span, (double)d1[i]);
    }
    offset += span + 2.0;
  }
}

std::string mf_analyse(MFSymbolic& sym, int64_t n, const int32_t* indptr, const int32_t* indices,
                       const double* xyz_in, int leaf_size) {
  if (n <= 0) return "empty matrix";
  std::vector<double> pseudo;
  const double* xyz = xyz_in;
  if (!xyz) {
    graph_coordinates(n, indptr, indices, pseudo);
    xyz = pseudo.data();
  }
  ND nd;
  nd.indptr = indptr;
  nd.indices = indices;
  nd.xyz = xyz;
  nd.leaf = std::max(16, leaf_size);
  nd.mark.assign(n, 0);
  nd.gen.assign(n, 0);
  nd.order.reserve(n);
  std::vector<int64_t> all(n);
  for (int64_t i = 0; i < n; ++i) all[i] = i;
  // disconnected pieces are handled by the bisection itself (empty separators)
  int root = nd.build(all);
  if (root < 0 || (int64_t)nd.order.size() != n) return "ordering failed";
  return mf_finish(sym, n, indptr, indices, std::move(nd.order), std::move(nd.nodes));
}

// Front structure, scatter lists and extend-add maps of an ordering whose
// nodes are in postorder.  The update set U of a node needs only its
// children's, so U is built level by level with the nodes of a level in
// parallel; the scatter lists and extend-add maps are counted per node,
// laid out by prefix sums in node order and filled in parallel, so the
// result does not depend on the thread count.
std::string mf_finish(MFSymbolic& sym, int64_t n, const int32_t* indptr, const int32_t* indices,
                      std::vector<int64_t>&& order, std::vector<MFNode>&& nodes) {
  sym.n = n;
  sym.nnz = indptr[n];
  sym.perm = std::move(order);
  sym.iperm.assign(n, 0);
  for (int64_t i = 0; i < n; ++i) sym.iperm[sym.perm[i]] = i;
  sym.nodes = std::move(nodes);
  const int64_t nn = (int64_t)sym.nodes.size();

  // ---- update sets, level by level (children first) ----
  int max_level = 0;
  for (const MFNode& nd_s : sym.nodes) max_level = std::max(max_level, nd_s.level);
  std::vector<std::vector<int64_t>> by_level(max_level + 1);
  for (int64_t s = 0; s < nn; ++s) by_level[sym.nodes[s].level].push_back(s);
  for (const auto& lv : by_level) {
#pragma omp parallel
    {
      std::vector<int64_t> buf;
#pragma omp for schedule(dynamic, 1)
      for (int64_t t = 0; t < (int64_t)lv.size(); ++t) {
        MFNode& nd_s = sym.nodes[lv[t]];
        // only ancestors (new index >= end) enter U
        buf.clear();
        for (int c : nd_s.children)
          for (int64_t u : sym.nodes[c].U)
            if (u >= nd_s.end) buf.push_back(u);
        for (int64_t i = nd_s.start; i < nd_s.end; ++i) {
          const int64_t o = sym.perm[i];
          for (int32_t q = indptr[o]; q < indptr[o + 1]; ++q) {
            const int64_t jn = sym.iperm[indices[q]];
            if (jn >= nd_s.end) buf.push_back(jn);
          }
        }
        std::sort(buf.begin(), buf.end());
        buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
        nd_s.U.assign(buf.begin(), buf.end());
        nd_s.f = nd_s.k + (int64_t)nd_s.U.size();
      }
    }
  }
  sym.max_level = 0;
  sym.arena = 0;
  sym.max_front = 0;
  sym.flops = 0;
  for (int64_t s = 0; s < nn; ++s) {
    MFNode& nd_s = sym.nodes[s];
    nd_s.front_off = sym.arena;
    sym.arena += nd_s.f * nd_s.f;
    sym.max_front = std::max(sym.max_front, nd_s.f);
    sym.max_level = std::max(sym.max_level, nd_s.level);
    for (int64_t i = 0; i < nd_s.k; ++i) sym.flops += double(nd_s.f - i - 1) * double(nd_s.f - i - 1);
  }

  // ---- scatter lists and extend-add maps ----
  auto pos_in = [&](const MFNode& nd_s, int64_t jn) -> int64_t {
    if (jn < nd_s.end) return jn - nd_s.start;
    auto it = std::lower_bound(nd_s.U.begin(), nd_s.U.end(), jn);
    return nd_s.k + (it - nd_s.U.begin());
  };
  // pass 1: entries per node (an own-row entry, plus its transpose when the
  // column belongs to an ancestor)
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t s = 0; s < nn; ++s) {
    MFNode& nd_s = sym.nodes[s];
    int64_t cnt = 0;
    for (int64_t i = nd_s.start; i < nd_s.end; ++i) {
      const int64_t o = sym.perm[i];
      for (int32_t q = indptr[o]; q < indptr[o + 1]; ++q) {
        const int64_t jn = sym.iperm[indices[q]];
        if (jn >= nd_s.start) cnt += jn >= nd_s.end ? 2 : 1;
      }
    }
    nd_s.scat_len = cnt;
  }
  int64_t tot = 0, ea_tot = 0;
  for (int64_t s = 0; s < nn; ++s) {
    MFNode& nd_s = sym.nodes[s];
    nd_s.scat_off = tot;
    tot += nd_s.scat_len;
    nd_s.ea_off = ea_tot;
    if (nd_s.parent >= 0) ea_tot += (int64_t)nd_s.U.size();
  }
  sym.scat_src.assign(tot, 0);
  sym.scat_dst.assign(tot, 0);
  sym.ea_map.assign(ea_tot, 0);
  // pass 2: fill every node's segment in row order
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : bad)
  for (int64_t s = 0; s < nn; ++s) {
    const MFNode& nd_s = sym.nodes[s];
    int64_t w = nd_s.scat_off;
    for (int64_t i = nd_s.start; i < nd_s.end; ++i) {
      const int64_t o = sym.perm[i];
      const int64_t pi = i - nd_s.start;
      for (int32_t q = indptr[o]; q < indptr[o + 1]; ++q) {
        const int64_t jo = indices[q];
        const int64_t jn = sym.iperm[jo];
        if (jn < nd_s.start) continue;  // eliminated in a descendant
        const int64_t pj = pos_in(nd_s, jn);
        sym.scat_src[w] = q;
        sym.scat_dst[w++] = nd_s.front_off + pi * nd_s.f + pj;
        if (jn >= nd_s.end) {  // column entry A(j, i) of the ancestor row j
          const int32_t* b = indices + indptr[jo];
          const int32_t* e = indices + indptr[jo + 1];
          const int32_t* t = std::lower_bound(b, e, (int32_t)o);
          if (t == e || *t != o) {
            bad = 1;
            sym.scat_src[w] = 0;
          } else {
            sym.scat_src[w] = (int32_t)(t - indices);
          }
          sym.scat_dst[w++] = nd_s.front_off + pj * nd_s.f + pi;
        }
      }
    }
    if (nd_s.parent >= 0) {
      const MFNode& par = sym.nodes[nd_s.parent];
      int64_t e = nd_s.ea_off;
      for (int64_t u : nd_s.U) sym.ea_map[e++] = (int32_t)pos_in(par, u);
    }
  }
  if (bad) return "matrix pattern is not structurally symmetric";
  return "";
}

}  // namespace sucem
