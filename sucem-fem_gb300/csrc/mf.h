// Multifrontal sparse LU: symbolic analysis (host) and numeric factor/solve
// (device).  Replaces the direct solvers the reference calls:
// dolfin.LUSolver(S - sigma*M) (sucemfem/ProblemConfigurations/
// EMVectorWaveEigenproblem.py:76-85), UMFPACKSolver / spsolve and the
// spilu preconditioner (sucemfem/Utilities/LinalgSolvers.py:118-121,262-277).
//
// Ordering: nested dissection by recursive coordinate bisection of the DOF
// locations with one-sided vertex separators on the matrix graph.  Each
// separator (or leaf block) is a node of the assembly tree; a node's front
// holds its own variables followed by the ancestor variables they couple to.
// No pivoting: a pivot smaller than tau*max|A| is replaced by tau*max|A|
// (static pivoting) and the count is reported; iterative refinement in the
// caller recovers the accuracy.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

namespace sucem {

struct MFNode {
  int64_t start = 0, end = 0;       // own variables, new numbering [start, end)
  int64_t k = 0;                    // end - start
  int64_t f = 0;                    // front size = k + |U|
  int parent = -1;
  int level = 0;                    // height: leaves 0, parent = 1 + max(children)
  std::vector<int> children;
  std::vector<int64_t> U;           // ancestor variables (new numbering, sorted)
  int64_t front_off = 0;            // offset of the f*f front in the arena
  int64_t scat_off = 0, scat_len = 0;  // original-entry scatter list
  int64_t ea_off = 0;               // extend-add map into the parent front (|U| ints)
};

struct MFSymbolic {
  int64_t n = 0, nnz = 0;
  std::vector<int64_t> perm;        // perm[new] = old
  std::vector<int64_t> iperm;       // iperm[old] = new
  std::vector<MFNode> nodes;        // postorder
  int max_level = 0;
  int64_t arena = 0;                // sum of f^2
  int64_t max_front = 0;
  double flops = 0;                 // multiply-adds of the factorisation
  // scatter list: value index in the CSR, destination index in the arena
  std::vector<int32_t> scat_src;
  std::vector<int64_t> scat_dst;
  std::vector<int32_t> ea_map;      // per node: positions of U in the parent front
};

// Builds the ordering and the symbolic factorisation of a CSR pattern with
// symmetric structure.  xyz: n*3 coordinates of the DOFs (used for the
// bisection).  Returns "" or an error message.
std::string mf_analyse(MFSymbolic& sym, int64_t n, const int32_t* indptr, const int32_t* indices,
                       const double* xyz, int leaf_size);

// Same with the element-based ordering: cell_dofs (nt*nd, -1 = DOF not in
// this matrix) and cell centroids cell_xyz (nt*3).  Separators are the DOFs
// shared by the two halves of a cell bisection, i.e. interface surfaces.
std::string mf_analyse_cells(MFSymbolic& sym, int64_t n, const int32_t* indptr,
                             const int32_t* indices, int64_t nt, int nd, const int32_t* cell_dofs,
                             const double* cell_xyz, int leaf_size);

}  // namespace sucem

namespace sucem {
struct MFHandle;
cudaError_t mf_factor(MFHandle& h, int dtype, const void* vals, double tau, cudaStream_t st);
cudaError_t mf_solve(MFHandle& h, int io_dtype, const void* b, void* x, cudaStream_t st);
int mf_perturbed(MFHandle& h);
// 0: the last factorisation is usable; -1: a bounded wait of its
// tensor-core update gave up (invalid factor); -2: not factored or a CUDA
// error.  Waits for the factorisation the first time it is asked.
int mf_factor_status(MFHandle& h);
// host-side failure injection for tests: marks the last factorisation as if
// a bounded wait of its tensor-core update had given up
cudaError_t mf_mark_timed_out(MFHandle& h);
// plan parameters of the single-precision factorisation (0 = default):
// super-panel width (a multiple of 64) and the pivot-block threshold of the
// tensor-core panel updates; the device state is rebuilt at the next factor
cudaError_t mf_configure(MFHandle& h, int superpanel, int panel_k);
// tensor-core update launches of the last factorisation: out[0] launches,
// out[1] their summed event-timed duration (ms), out[2] algorithmic flops
void mf_tc_stats(MFHandle& h, double* out);
void mf_free(MFHandle& h);
// self-test of the bounded mbarrier wait of the tensor-core kernel:
// *gave_up = 1 when a wait nothing arrives at ran out after `polls` polls
cudaError_t mf_wait_selftest(int polls, int* gave_up);
}  // namespace sucem
