// Host-side function space: mesh entities, N1curl DOF map, CSR pattern and
// the entity -> incident-cell tables the row-gather assembly kernels read.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace sucem {

// UFC local numbering of a tetrahedron.
static const int kEdgeVerts[6][2] = {{2, 3}, {1, 3}, {1, 2}, {0, 3}, {0, 2}, {0, 1}};
static const int kFaceVerts[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};

struct DeviceSpace;  // device copies, defined in the CUDA sources

struct Space {
  int order = 1;
  int ndof_cell = 6;        // k(k+2)(k+3)/2: 6, 20, 45, 84 for orders 1-4
  int dofs_per_entity = 1;  // 1 (order 1) or 2 (order 2); orders 3-4: per edge
  int dofs_edge = 1, dofs_face = 0, dofs_cell = 0;  // k, k(k-1), k(k-1)(k-2)/2
  int64_t nv = 0, nt = 0, ne = 0, nf = 0;
  int64_t n = 0;            // global dimension
  int64_t nnz = 0;
  int max_row = 0;          // longest CSR row

  std::vector<double> coords;          // nv*3
  std::vector<int32_t> cells;          // nt*4, vertices sorted per cell
  std::vector<int32_t> cell_edges;     // nt*6 (first-encounter numbering)
  std::vector<int32_t> cell_faces;     // nt*4
  std::vector<int32_t> edges;          // ne*2
  std::vector<int32_t> faces;          // nf*3
  std::vector<int32_t> cell_dofs;      // nt*ndof_cell
  std::vector<uint8_t> ext_mask;       // nt: bit f set if local face f is exterior
  int64_t n_ext_facets = 0;

  // CSR pattern (rows sorted, columns sorted)
  std::vector<int64_t> indptr;         // n+1
  std::vector<int32_t> indices;        // nnz

  // Row-gather tables.  Entities are the edges (order 1) or the edges
  // followed by the faces (order 2; orders 3-4 add the cells); entity k
  // owns the consecutive rows of its DOFs, which share one column list.
  // inc_rec is built for orders 1-2 only.
  int64_t n_ent = 0;
  std::vector<int32_t> ent_ptr;        // n_ent+1
  std::vector<int32_t> inc_cell;       // per incidence: the cell
  std::vector<uint8_t> inc_rec;        // per incidence: rec_bytes bytes:
                                       //   [0] local entity index (0..5 edge, 6..9 face)
                                       //   [1..ndof_cell] column slot of each local dof
  int rec_bytes = 8;

  // orders 3-4 (entry-gather assembly): CSR entry q sums the cell entries
  // entry_src[entry_ptr[q] .. entry_ptr[q+1]), each coded
  // (c * ndof_cell + a) * ndof_cell + b, in ascending cell order
  std::vector<int32_t> entry_ptr;      // nnz+1
  std::vector<int32_t> entry_src;      // nt*ndof_cell^2
  std::vector<int32_t> entry_perm;     // nnz: the CSR entry of each kernel thread (each row's
                                       //   entries by list length)

  // Entity-per-lane assembly schedule (orders 1-2).  Entities are grouped
  // into warp tasks of 32 (one entity per lane) that share the entity kind
  // (edge / face) and the boundary class (on an exterior facet or not), in
  // an order that puts entities with the same incidence structure side by
  // side.  A task walks its lanes' incidences local-entity-major: for each
  // local index le (edges 0..5, faces 0..3) trip[le] steps, step t giving
  // every lane its t-th incident cell with the entity at local index le
  // (cell order within le, so the summation order is fixed).  One step is a
  // block of 32 records laid out as planes of 32 words: the cells (-1: the
  // lane has no incidence in this step), then ceil(ndof_cell / 4) words of
  // column slots (byte b = slot of the cell's local DOF b in the entity's
  // column list).
  int64_t n_tasks = 0;                 // warp tasks
  int64_t n_tasks_interior = 0;        // tasks [0, n_tasks_interior) have no boundary entity
  std::vector<int32_t> task_ent;       // n_tasks*32: entity per lane (-1: none)
  std::vector<int32_t> task_meta;      // n_tasks*4: first step block, trips le 0-3 (bytes),
                                       //   trips le 4-7 (bytes), flags (bit 0: faces;
                                       //   bits 8-23: accumulator stride P, the task's
                                       //   longest row made odd)
  std::vector<uint32_t> step_words;    // step blocks, (1 + slot_planes) * 32 words each
  int slot_planes = 0;                 // ceil(ndof_cell / 4)

  std::vector<int32_t> boundary_dofs;  // closure of the exterior facets, sorted
  std::vector<double> dof_xyz;         // n*3: edge midpoint / face centroid of each DOF

  DeviceSpace* dev = nullptr;
};

// Builds everything above; returns an empty string or an error message.
std::string build_space(Space& s, const double* coords, int64_t nv, const int64_t* cells,
                        int64_t nt, int order);

// The entity-per-lane assembly schedule of an order-1/2 space (called by
// build_space once the incidence tables exist).
void build_row_schedule(Space& s);

}  // namespace sucem
