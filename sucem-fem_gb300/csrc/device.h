// Device-resident copies of a Space and the kernel launchers.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "space.h"

namespace sucem {

struct DeviceSpace {
  int device = 0;
  int64_t nt = 0, nv = 0, n = 0, nnz = 0, n_ent = 0, ninc = 0;
  int order = 1, nd = 6, dpe = 1, rec_bytes = 8, max_row = 0;
  int4* cells = nullptr;          // nt
  float4* xyz_hi = nullptr;       // nv (w unused)
  float4* xyz_lo = nullptr;       // nv
  double* xyz = nullptr;          // nv*3
  uint8_t* ext_mask = nullptr;    // nt
  int32_t* ent_ptr = nullptr;     // n_ent+1
  int32_t* inc_cell = nullptr;    // ninc
  uint8_t* inc_rec = nullptr;     // ninc*rec_bytes
  int32_t* indptr = nullptr;      // n+1
  int32_t* indices = nullptr;     // nnz
  int32_t* cell_dofs = nullptr;   // nt*nd
  int32_t* entry_ptr = nullptr;   // orders 3-4: nnz+1, cell entries summed into each CSR entry
  int32_t* entry_src = nullptr;   // nt*nd*nd, (c * nd + a) * nd + b in ascending cell order
  int32_t* entry_perm = nullptr;  // nnz: CSR entry of each thread of the order-3/4 kernel
  int32_t* boundary_dofs = nullptr;
  int64_t n_boundary = 0;
  int32_t* bidx = nullptr;        // nt: index among cells with exterior facets, -1 otherwise
  // exterior facets (cell, local face) and the far-field scratch of the
  // NTFF (allocated on first use)
  int32_t* ext_facets = nullptr;  // n_ext*2
  int64_t n_ext = 0;
  double* ntff_pts = nullptr;     // n_ext*9 points x 16 doubles
  // dual functional (physical point, tangent) of every boundary DOF, for
  // interpolating expressions onto the boundary (allocated on first use)
  double* bdof_pt = nullptr;      // n_boundary*6
  // point location: uniform grid of cell bounding boxes (built on first use)
  int32_t* bin_ptr = nullptr;     // nbins+1
  int32_t* bin_cells = nullptr;   // cells overlapping each bin
  int grid_n[3] = {0, 0, 0};
  double grid_lo[3] = {0, 0, 0}, grid_inv[3] = {0, 0, 0};
  int64_t nb = 0;                 // number of cells with exterior facets
  // per-cell coefficient scratch of the assembly (allocated on first use)
  float* g_f = nullptr;           // nt*12
  double* g_d = nullptr;
  float* g2_f = nullptr;          // nt*24: float hi + lo coefficients (separate FP32 matrices)
  float* h2_f = nullptr;          // nb*24: float hi + lo tangential coefficients
  float* h_f = nullptr;           // nb*12
  double* h_d = nullptr;
  // entity-per-lane assembly schedule (orders 1-2, see Space)
  int64_t n_tasks = 0, n_tasks_interior = 0;
  int slot_planes = 0;
  int32_t* task_ent = nullptr;    // n_tasks*32
  int4* task_meta = nullptr;      // n_tasks
  uint32_t* step_words = nullptr; // step blocks
  std::vector<uint16_t> task_P;   // host copy of every task's accumulator stride
  // tasks of each block of the assembly kernel, packed per shared-memory
  // need (key: bytes per accumulator slot and boundary layout; built once)
  struct TaskBlocks {
    int32_t* first = nullptr;     // device: first task of each block (+ end)
    int64_t n_int = 0, n_bnd = 0; // interior blocks, then boundary blocks
    int64_t smem = 0;             // largest block's shared memory
  };
  std::map<int, TaskBlocks> task_blocks;
  // reference tensors in the cell kernel's layout [a][b][12] (KC m=0..5, KM m=0..5)
  float* kab_f = nullptr;
  double* kab_d = nullptr;
  // reference tensors [6][nd][nd] (curl, mass), [4][3][nd][nd] (face tangential)
  float* kc_f = nullptr;
  float* km_f = nullptr;
  float* kt_f = nullptr;
  float* kt_lo_f = nullptr;       // kt_d - kt_f rounded to float (compensated FP32 ABC terms)
  double* kc_d = nullptr;
  double* km_d = nullptr;
  double* kt_d = nullptr;
};

// Copies the host space to the current device.  Returns "" or an error.
std::string upload_space(Space& s, int device);
void free_device_space(DeviceSpace* d);

// Assembly: row-gather for orders 1-2, cell-based (atomic adds at the
// precomputed CSR positions) for orders 3-4.  real_bytes = 4 (float) or 8
// (double).
//   mode 0: S, T, B written to separate real arrays (any may be null)
//   mode 1: A = S - k0^2 T + j k0 B written as interleaved complex
struct AssembleArgs {
  int real_bytes = 8;
  int mode = 0;
  const void* eps_r = nullptr;     // per cell, Real; null = 1
  const void* mu_r_inv = nullptr;  // per cell, Real; null = 1
  void* S = nullptr;
  void* T = nullptr;
  void* B = nullptr;
  void* A = nullptr;
  double k0 = 0.0;
};
cudaError_t launch_assemble(DeviceSpace& d, const AssembleArgs& a, cudaStream_t stream);

}  // namespace sucem
