// Host builder for the N1curl function space (the part of DOLFIN that the
// reference reaches through dolfin.FunctionSpace and dolfin.assemble's
// sparsity pass: sucemfem/ProblemConfigurations/EMProblem.py:100-105,
// sucemfem/SystemMatrices.py:54).
//
// Numbering rules (DOLFIN's, so the DOF numbers of orders 1 and 2 are
// bit-exact with the reference's; orders 3 and 4 keep the same entity-major
// layout, their per-entity order being the element's DOF order):
//  * each cell's vertices are sorted by global index (mesh ordering);
//  * edges and faces are numbered by first encounter while walking the cells
//    in order and each cell's local entities in UFC order;
//  * order 1: dof = edge; order 2: dofs 2e, 2e+1 per edge, then
//    2E + 2f, 2E + 2f + 1 per face; order k in general: k DOFs per edge,
//    then k(k-1) per face, then k(k-1)(k-2)/2 per cell, entity by entity
//    (the numbering above for k <= 2).
// The CSR pattern is the union of all cell-pair couplings with sorted
// columns (explicit zeros kept), i.e. DOLFIN's cell sparsity pattern.
#include "space.h"

#include <algorithm>
#include <cstring>
#include <numeric>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace sucem {

namespace {

// First-encounter numbering of entities keyed by their smallest vertex.
struct EntityTable {
  // per smallest vertex: list of (other-vertex key, id)
  std::vector<std::vector<std::pair<int64_t, int32_t>>> buckets;
  int32_t count = 0;
  explicit EntityTable(int64_t nv) : buckets(nv) {}
  int32_t find_or_add(int32_t vmin, int64_t rest) {
    auto& b = buckets[vmin];
    for (auto& p : b)
      if (p.first == rest) return p.second;
    b.emplace_back(rest, count);
    return count++;
  }
};

}  // namespace

std::string build_space(Space& s, const double* coords, int64_t nv, const int64_t* cells,
                        int64_t nt, int order) {
  if (order < 1 || order > 4) return "order must be 1, 2, 3 or 4";
  if (nv <= 0 || nt <= 0) return "empty mesh";
  if (nv >= (int64_t(1) << 31) || nt >= (int64_t(1) << 31)) return "mesh too large for int32 ids";
  s.order = order;
  s.ndof_cell = order * (order + 2) * (order + 3) / 2;
  s.dofs_per_entity = order <= 2 ? order : 0;
  s.dofs_edge = order;
  s.dofs_face = order * (order - 1);
  s.dofs_cell = order * (order - 1) * (order - 2) / 2;
  s.rec_bytes = order == 1 ? 8 : (order == 2 ? 24 : 0);
  s.nv = nv;
  s.nt = nt;
  s.coords.assign(coords, coords + nv * 3);
  s.cells.resize(nt * 4);
  for (int64_t c = 0; c < nt; ++c) {
    int64_t v[4];
    for (int k = 0; k < 4; ++k) {
      v[k] = cells[c * 4 + k];
      if (v[k] < 0 || v[k] >= nv) return "cell vertex index out of range";
    }
    std::sort(v, v + 4);
    for (int k = 0; k < 3; ++k)
      if (v[k] == v[k + 1]) return "degenerate cell (repeated vertex)";
    for (int k = 0; k < 4; ++k) s.cells[c * 4 + k] = int32_t(v[k]);
  }

  // ---- entities (serial: the numbering is order dependent) ----
  s.cell_edges.resize(nt * 6);
  s.cell_faces.resize(nt * 4);
  {
    EntityTable et(nv);
    for (int64_t c = 0; c < nt; ++c) {
      const int32_t* v = &s.cells[c * 4];
      for (int le = 0; le < 6; ++le) {
        int32_t a = v[kEdgeVerts[le][0]], b = v[kEdgeVerts[le][1]];
        s.cell_edges[c * 6 + le] = et.find_or_add(a, b);
      }
    }
    s.ne = et.count;
    s.edges.resize(s.ne * 2);
    for (int64_t vm = 0; vm < nv; ++vm)
      for (auto& p : et.buckets[vm]) {
        s.edges[p.second * 2] = int32_t(vm);
        s.edges[p.second * 2 + 1] = int32_t(p.first);
      }
  }
  {
    EntityTable ft(nv);
    for (int64_t c = 0; c < nt; ++c) {
      const int32_t* v = &s.cells[c * 4];
      for (int lf = 0; lf < 4; ++lf) {
        int32_t a = v[kFaceVerts[lf][0]], b = v[kFaceVerts[lf][1]], d = v[kFaceVerts[lf][2]];
        s.cell_faces[c * 4 + lf] = ft.find_or_add(a, int64_t(b) * nv + d);
      }
    }
    s.nf = ft.count;
    s.faces.resize(s.nf * 3);
    for (int64_t vm = 0; vm < nv; ++vm)
      for (auto& p : ft.buckets[vm]) {
        s.faces[p.second * 3] = int32_t(vm);
        s.faces[p.second * 3 + 1] = int32_t(p.first / nv);
        s.faces[p.second * 3 + 2] = int32_t(p.first % nv);
      }
  }

  // ---- exterior facets ----
  std::vector<int32_t> face_count(s.nf, 0);
  for (int64_t i = 0; i < nt * 4; ++i) face_count[s.cell_faces[i]]++;
  s.ext_mask.assign(nt, 0);
  s.n_ext_facets = 0;
  for (int64_t c = 0; c < nt; ++c)
    for (int lf = 0; lf < 4; ++lf)
      if (face_count[s.cell_faces[c * 4 + lf]] == 1) {
        s.ext_mask[c] |= uint8_t(1u << lf);
        s.n_ext_facets++;
      }

  // ---- DOF map ----
  const int nd = s.ndof_cell;
  const int de = s.dofs_edge, df = s.dofs_face, dc = s.dofs_cell;
  const int64_t face0 = de * s.ne, cell0 = face0 + df * s.nf;
  s.n = cell0 + dc * nt;
  if (s.n >= (int64_t(1) << 31)) return "too many DOFs for int32 indices";
  s.cell_dofs.resize(nt * nd);
  for (int64_t c = 0; c < nt; ++c) {
    int32_t* d = &s.cell_dofs[c * nd];
    for (int le = 0; le < 6; ++le)
      for (int j = 0; j < de; ++j) d[de * le + j] = int32_t(de * s.cell_edges[c * 6 + le] + j);
    for (int lf = 0; lf < 4; ++lf)
      for (int j = 0; j < df; ++j)
        d[6 * de + df * lf + j] = int32_t(face0 + df * int64_t(s.cell_faces[c * 4 + lf]) + j);
    for (int j = 0; j < dc; ++j) d[6 * de + 4 * df + j] = int32_t(cell0 + dc * c + j);
  }

  // ---- entity -> incident cells (in cell order) ----
  // entities: edges, then faces (order >= 2), then cells (order >= 3)
  s.n_ent = s.ne + (order >= 2 ? s.nf : 0) + (order >= 3 ? nt : 0);
  auto ent_first_dof = [&](int64_t k) -> int64_t {
    if (k < s.ne) return de * k;
    if (k < s.ne + s.nf) return face0 + df * (k - s.ne);
    return cell0 + dc * (k - s.ne - s.nf);
  };
  auto ent_ndof = [&](int64_t k) -> int { return k < s.ne ? de : (k < s.ne + s.nf ? df : dc); };
  s.ent_ptr.assign(s.n_ent + 1, 0);
  for (int64_t c = 0; c < nt; ++c) {
    for (int le = 0; le < 6; ++le) s.ent_ptr[s.cell_edges[c * 6 + le] + 1]++;
    if (order >= 2)
      for (int lf = 0; lf < 4; ++lf) s.ent_ptr[s.ne + s.cell_faces[c * 4 + lf] + 1]++;
    if (order >= 3) s.ent_ptr[s.ne + s.nf + c + 1]++;
  }
  for (int64_t k = 0; k < s.n_ent; ++k) s.ent_ptr[k + 1] += s.ent_ptr[k];
  const int64_t ninc = s.ent_ptr[s.n_ent];
  s.inc_cell.resize(ninc);
  std::vector<uint8_t> inc_local(ninc);
  {
    std::vector<int32_t> fill(s.ent_ptr.begin(), s.ent_ptr.end() - 1);
    for (int64_t c = 0; c < nt; ++c) {
      for (int le = 0; le < 6; ++le) {
        int32_t k = s.cell_edges[c * 6 + le];
        int32_t pos = fill[k]++;
        s.inc_cell[pos] = int32_t(c);
        inc_local[pos] = uint8_t(le);
      }
      if (order >= 2)
        for (int lf = 0; lf < 4; ++lf) {
          int64_t k = s.ne + s.cell_faces[c * 4 + lf];
          int32_t pos = fill[k]++;
          s.inc_cell[pos] = int32_t(c);
          inc_local[pos] = uint8_t(6 + lf);
        }
      if (order >= 3) {
        int32_t pos = fill[s.ne + s.nf + c]++;
        s.inc_cell[pos] = int32_t(c);
        inc_local[pos] = uint8_t(10);
      }
    }
  }

  // ---- pattern: column list per entity (shared by its rows) ----
  std::vector<int64_t> ent_len(s.n_ent, 0);
  std::vector<int64_t> ent_col_ptr(s.n_ent + 1, 0);
  std::vector<int32_t> ent_cols;
  {
    // pass 1: lengths
#pragma omp parallel
    {
      std::vector<int32_t> buf;
#pragma omp for schedule(dynamic, 1024)
      for (int64_t k = 0; k < s.n_ent; ++k) {
        buf.clear();
        for (int32_t i = s.ent_ptr[k]; i < s.ent_ptr[k + 1]; ++i) {
          const int32_t* d = &s.cell_dofs[int64_t(s.inc_cell[i]) * nd];
          buf.insert(buf.end(), d, d + nd);
        }
        std::sort(buf.begin(), buf.end());
        ent_len[k] = std::unique(buf.begin(), buf.end()) - buf.begin();
      }
    }
    for (int64_t k = 0; k < s.n_ent; ++k) ent_col_ptr[k + 1] = ent_col_ptr[k] + ent_len[k];
    ent_cols.resize(ent_col_ptr[s.n_ent]);
    int64_t maxlen = 0;
    for (int64_t k = 0; k < s.n_ent; ++k) maxlen = std::max(maxlen, ent_len[k]);
    if (order <= 2 && maxlen > 255)
      return "a CSR row has more than 255 columns (cell valence too high for the 8-bit slot tables)";
    s.max_row = int(maxlen);
    s.inc_rec.assign(ninc * s.rec_bytes, 0);
    // pass 2: columns and slots
#pragma omp parallel
    {
      std::vector<int32_t> buf;
#pragma omp for schedule(dynamic, 1024)
      for (int64_t k = 0; k < s.n_ent; ++k) {
        buf.clear();
        for (int32_t i = s.ent_ptr[k]; i < s.ent_ptr[k + 1]; ++i) {
          const int32_t* d = &s.cell_dofs[int64_t(s.inc_cell[i]) * nd];
          buf.insert(buf.end(), d, d + nd);
        }
        std::sort(buf.begin(), buf.end());
        buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
        std::copy(buf.begin(), buf.end(), ent_cols.begin() + ent_col_ptr[k]);
        if (order >= 3) continue;
        for (int32_t i = s.ent_ptr[k]; i < s.ent_ptr[k + 1]; ++i) {
          uint8_t* rec = &s.inc_rec[int64_t(i) * s.rec_bytes];
          rec[0] = inc_local[i];
          const int32_t* d = &s.cell_dofs[int64_t(s.inc_cell[i]) * nd];
          for (int b = 0; b < nd; ++b)
            rec[1 + b] = uint8_t(std::lower_bound(buf.begin(), buf.end(), d[b]) - buf.begin());
        }
      }
    }
  }
  // rows: entity k owns the rows of its DOFs (consecutive, in entity order)
  s.indptr.assign(s.n + 1, 0);
  for (int64_t k = 0; k < s.n_ent; ++k)
    for (int j = 0; j < ent_ndof(k); ++j) s.indptr[ent_first_dof(k) + j + 1] = ent_len[k];
  for (int64_t r = 0; r < s.n; ++r) s.indptr[r + 1] += s.indptr[r];
  s.nnz = s.indptr[s.n];
  if (s.nnz >= (int64_t(1) << 31)) return "pattern has 2^31 or more entries";
  s.indices.resize(s.nnz);
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < s.n_ent; ++k)
    for (int j = 0; j < ent_ndof(k); ++j)
      std::copy(ent_cols.begin() + ent_col_ptr[k], ent_cols.begin() + ent_col_ptr[k + 1],
                s.indices.begin() + s.indptr[ent_first_dof(k) + j]);

  // ---- orders 3-4: the cell entries that sum into each CSR entry ----
  // Row r (a DOF of entity k) receives, from every cell incident to k, the
  // entries (a, b) with cell_dofs[c][a] = r.  Per CSR entry the list holds
  // them in ascending cell order (within one cell only one b maps to a
  // column), which fixes the summation order of the assembly.
  if (order >= 3) {
    if (nt * int64_t(nd) * nd >= (int64_t(1) << 31))
      return "mesh too large for the order-3/4 entry lists (2^31 cell entries)";
    s.entry_ptr.assign(s.nnz + 1, 0);
    s.entry_src.assign(nt * int64_t(nd) * nd, 0);
    // first contribution of each row: entity k's rows each take ninc(k) * nd
    std::vector<int64_t> row_first(s.n + 1, 0);
    for (int64_t k = 0; k < s.n_ent; ++k)
      for (int j = 0; j < ent_ndof(k); ++j)
        row_first[ent_first_dof(k) + j + 1] = int64_t(s.ent_ptr[k + 1] - s.ent_ptr[k]) * nd;
    for (int64_t r = 0; r < s.n; ++r) row_first[r + 1] += row_first[r];
    s.entry_ptr[s.nnz] = int32_t(row_first[s.n]);
#pragma omp parallel
    {
      std::vector<int32_t> slot, cur;
#pragma omp for schedule(dynamic, 256)
      for (int64_t k = 0; k < s.n_ent; ++k) {
        const int32_t i0 = s.ent_ptr[k], i1 = s.ent_ptr[k + 1];
        const auto b0 = ent_cols.begin() + ent_col_ptr[k], b1 = ent_cols.begin() + ent_col_ptr[k + 1];
        const int64_t len = ent_col_ptr[k + 1] - ent_col_ptr[k];
        // column slot of every local DOF of every incident cell (shared by the rows)
        slot.resize(size_t(i1 - i0) * nd);
        for (int32_t i = i0; i < i1; ++i) {
          const int32_t* d = &s.cell_dofs[int64_t(s.inc_cell[i]) * nd];
          for (int b = 0; b < nd; ++b)
            slot[size_t(i - i0) * nd + b] = int32_t(std::lower_bound(b0, b1, d[b]) - b0);
        }
        for (int j = 0; j < ent_ndof(k); ++j) {
          const int64_t r = ent_first_dof(k) + j, q0 = s.indptr[r];
          cur.assign(len, 0);
          for (size_t t = 0; t < slot.size(); ++t) cur[slot[t]]++;
          int64_t run = row_first[r];
          for (int64_t p = 0; p < len; ++p) {
            const int32_t n_p = cur[p];
            s.entry_ptr[q0 + p] = int32_t(run);
            cur[p] = int32_t(run);
            run += n_p;
          }
          for (int32_t i = i0; i < i1; ++i) {
            const int64_t c = s.inc_cell[i];
            const int32_t* d = &s.cell_dofs[c * nd];
            int a = 0;
            while (d[a] != r) ++a;
            for (int b = 0; b < nd; ++b)
              s.entry_src[cur[slot[size_t(i - i0) * nd + b]]++] = int32_t((c * nd + a) * nd + b);
          }
        }
      }
    }
    // thread order of the kernel: within each row, entries by list length
    // (stable), so that a warp's lanes walk lists of similar length
    s.entry_perm.resize(s.nnz);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < s.n; ++r) {
      const int64_t q0 = s.indptr[r], q1 = s.indptr[r + 1];
      for (int64_t q = q0; q < q1; ++q) s.entry_perm[q] = int32_t(q);
      std::stable_sort(s.entry_perm.begin() + q0, s.entry_perm.begin() + q1,
                       [&](int32_t x, int32_t y) {
                         return s.entry_ptr[x + 1] - s.entry_ptr[x] < s.entry_ptr[y + 1] - s.entry_ptr[y];
                       });
    }
  }

  // ---- DOF locations (used by the nested-dissection ordering) ----
  s.dof_xyz.assign(s.n * 3, 0.0);
  for (int64_t e = 0; e < s.ne; ++e)
    for (int j = 0; j < de; ++j)
      for (int d = 0; d < 3; ++d)
        s.dof_xyz[(de * e + j) * 3 + d] =
            0.5 * (s.coords[s.edges[2 * e] * 3 + d] + s.coords[s.edges[2 * e + 1] * 3 + d]);
  for (int64_t f = 0; f < s.nf; ++f)
    for (int j = 0; j < df; ++j)
      for (int d = 0; d < 3; ++d)
        s.dof_xyz[(face0 + df * f + j) * 3 + d] =
            (s.coords[s.faces[3 * f] * 3 + d] + s.coords[s.faces[3 * f + 1] * 3 + d] +
             s.coords[s.faces[3 * f + 2] * 3 + d]) / 3.0;
  for (int64_t c = 0; c < nt; ++c)
    for (int j = 0; j < dc; ++j)
      for (int d = 0; d < 3; ++d) {
        double x = 0;
        for (int v = 0; v < 4; ++v) x += s.coords[s.cells[c * 4 + v] * 3 + d];
        s.dof_xyz[(cell0 + dc * c + j) * 3 + d] = 0.25 * x;
      }

  // ---- boundary DOFs (closure of the exterior facets) ----
  {
    std::vector<uint8_t> mark(s.n, 0);
    for (int64_t c = 0; c < nt; ++c) {
      if (!s.ext_mask[c]) continue;
      for (int lf = 0; lf < 4; ++lf) {
        if (!(s.ext_mask[c] >> lf & 1)) continue;
        for (int le = 0; le < 6; ++le) {
          if (kEdgeVerts[le][0] == lf || kEdgeVerts[le][1] == lf) continue;  // edge not on face lf
          for (int j = 0; j < de; ++j) mark[s.cell_dofs[c * nd + de * le + j]] = 1;
        }
        for (int j = 0; j < df; ++j) mark[s.cell_dofs[c * nd + 6 * de + df * lf + j]] = 1;
      }
    }
    s.boundary_dofs.clear();
    for (int64_t r = 0; r < s.n; ++r)
      if (mark[r]) s.boundary_dofs.push_back(int32_t(r));
  }
  build_row_schedule(s);
  return "";
}

}  // namespace sucem
