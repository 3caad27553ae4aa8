// Host-side schedule of the entity-per-lane assembly kernel (orders 1-2):
// which 32 entities (rows) a warp owns and in which order each lane visits
// the cells incident to its entity.  Built once per function space from the
// entity -> incident-cell tables of space.cpp.
//
// The kernel gives each lane one entity and walks the lanes' incidences in
// lock-step, local-entity-major: all lanes first take their incidences in
// which the entity is local edge (face) 0, then 1, ...  The element-matrix
// rows of local entity le are then the same straight-line code for every
// lane (the reference constants of that le inlined), and only the number
// of steps per le is the warp's maximum over its lanes.  To keep those
// steps full and the lanes' shared-memory slots aligned, entities are
// sorted by (boundary class, kind, incidence counts per le, a hash of their
// column-slot pattern, id) before they are cut into warps: in structured
// and jittered meshes the entities of one warp then have identical
// incidence structure.
#include <algorithm>
#include <cstring>
#include <numeric>

#include "space.h"

namespace sucem {

void build_row_schedule(Space& s) {
  s.n_tasks = s.n_tasks_interior = 0;
  s.task_ent.clear();
  s.task_meta.clear();
  s.step_words.clear();
  if (s.order > 2) return;
  const int nd = s.ndof_cell;
  const int planes = (nd + 3) / 4;
  s.slot_planes = planes;
  const int64_t n_ent = s.n_ent;
  const int64_t ne = s.ne;

  // boundary class: the entity lies on an exterior facet
  std::vector<uint8_t> on_bnd(n_ent, 0);
  for (int64_t c = 0; c < s.nt; ++c) {
    const int m = s.ext_mask[c];
    if (!m) continue;
    for (int lf = 0; lf < 4; ++lf) {
      if (!(m >> lf & 1)) continue;
      for (int le = 0; le < 6; ++le)
        if (kEdgeVerts[le][0] != lf && kEdgeVerts[le][1] != lf) on_bnd[s.cell_edges[c * 6 + le]] = 1;
      if (s.order == 2) on_bnd[ne + s.cell_faces[c * 4 + lf]] = 1;
    }
  }

  // per entity: incidences reordered by local index (stable: cell order
  // within an index), counts per local index and the slot-pattern hash
  std::vector<int32_t> inc_order(s.inc_cell.size());
  std::vector<uint8_t> cnt((size_t)n_ent * 8, 0);
  std::vector<uint64_t> hsh(n_ent, 0);
  const int rb = s.rec_bytes;
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t k = 0; k < n_ent; ++k) {
    const int32_t i0 = s.ent_ptr[k], i1 = s.ent_ptr[k + 1];
    const int base = k < ne ? 0 : 6;  // rec[0]: 0..5 edges, 6..9 faces
    int32_t* out = &inc_order[i0];
    int w = 0;
    for (int le = 0; le < (k < ne ? 6 : 4); ++le)
      for (int32_t i = i0; i < i1; ++i)
        if (s.inc_rec[(int64_t)i * rb] == base + le) {
          out[w++] = i;
          cnt[k * 8 + le] = (uint8_t)std::min(255, cnt[k * 8 + le] + 1);
        }
    uint64_t h = 1469598103934665603ull;  // FNV-1a over (le, slots) in visiting order
    for (int q = 0; q < w; ++q) {
      const uint8_t* rec = &s.inc_rec[(int64_t)out[q] * rb];
      for (int b = 0; b <= nd; ++b) {
        h ^= rec[b];
        h *= 1099511628211ull;
      }
    }
    hsh[k] = h;
  }

  // entity order: interior first, then boundary; edges before faces; then
  // counts, slot pattern and id
  std::vector<int64_t> ord(n_ent);
  std::iota(ord.begin(), ord.end(), 0);
  auto key_less = [&](int64_t a, int64_t b) {
    if (on_bnd[a] != on_bnd[b]) return on_bnd[a] < on_bnd[b];
    const bool fa = a >= ne, fb = b >= ne;
    if (fa != fb) return fb;
    const int c = std::memcmp(&cnt[a * 8], &cnt[b * 8], 8);
    if (c != 0) return c < 0;
    if (hsh[a] != hsh[b]) return hsh[a] < hsh[b];
    return a < b;
  };
  std::sort(ord.begin(), ord.end(), key_less);

  // cut into warp tasks that never mix boundary classes or kinds
  std::vector<int64_t> task_first;
  for (int64_t i = 0; i < n_ent;) {
    const int64_t k = ord[i];
    int64_t j = i + 1;
    while (j < n_ent && j - i < 32 && on_bnd[ord[j]] == on_bnd[k] && (ord[j] >= ne) == (k >= ne)) ++j;
    task_first.push_back(i);
    i = j;
  }
  task_first.push_back(n_ent);
  const int64_t nt_ = (int64_t)task_first.size() - 1;
  s.n_tasks = nt_;
  s.task_ent.assign(nt_ * 32, -1);
  s.task_meta.assign(nt_ * 4, 0);
  std::vector<int64_t> step_base(nt_ + 1, 0);
  for (int64_t t = 0; t < nt_; ++t) {
    uint8_t trip[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = task_first[t]; i < task_first[t + 1]; ++i) {
      const int64_t k = ord[i];
      s.task_ent[t * 32 + (i - task_first[t])] = (int32_t)k;
      for (int le = 0; le < 8; ++le) trip[le] = std::max(trip[le], cnt[k * 8 + le]);
    }
    int steps = 0;
    for (int le = 0; le < 8; ++le) steps += trip[le];
    step_base[t + 1] = step_base[t] + steps;
    const int64_t k0 = ord[task_first[t]];
    if (!on_bnd[k0]) s.n_tasks_interior = t + 1;
    // the task's accumulator stride: its longest row, made odd (slot
    // vectors of the 32 lanes then fall in distinct banks)
    int64_t lmax = 1;
    for (int64_t i = task_first[t]; i < task_first[t + 1]; ++i) {
      const int64_t r = (int64_t)s.dofs_per_entity * ord[i];
      lmax = std::max<int64_t>(lmax, s.indptr[r + 1] - s.indptr[r]);
    }
    int32_t* meta = &s.task_meta[t * 4];
    std::memcpy(&meta[1], trip, 8);
    meta[3] = (k0 >= ne ? 1 : 0) | (int32_t)((lmax | 1) << 8);
  }
  const int64_t words_per_step = (int64_t)(1 + planes) * 32;
  s.step_words.assign(step_base[nt_] * words_per_step, 0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t t = 0; t < nt_; ++t) {
    s.task_meta[t * 4] = (int32_t)step_base[t];
    const uint8_t* trip = reinterpret_cast<const uint8_t*>(&s.task_meta[t * 4 + 1]);
    // empty lanes: cell -1
    for (int64_t st = step_base[t]; st < step_base[t + 1]; ++st)
      for (int l = 0; l < 32; ++l) s.step_words[st * words_per_step + l] = 0xffffffffu;
    for (int l = 0; l < 32; ++l) {
      const int32_t k = s.task_ent[t * 32 + l];
      if (k < 0) continue;
      const int32_t i0 = s.ent_ptr[k];
      int q = 0;  // position in the entity's reordered incidences
      int64_t st = step_base[t];
      for (int le = 0; le < 8; ++le) {
        for (int u = 0; u < trip[le]; ++u, ++st) {
          if (u >= cnt[k * 8 + le]) continue;
          const int32_t inc = inc_order[i0 + q++];
          uint32_t* blk = &s.step_words[st * words_per_step];
          blk[l] = (uint32_t)s.inc_cell[inc];
          const uint8_t* rec = &s.inc_rec[(int64_t)inc * rb];
          for (int b = 0; b < nd; ++b)
            blk[32 * (1 + b / 4) + l] |= (uint32_t)rec[1 + b] << (8 * (b % 4));
        }
      }
    }
  }
}

}  // namespace sucem
