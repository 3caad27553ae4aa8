// C-ABI of the multifrontal sparse LU (declarations: include/sucem_gb300.h).
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <string>

#include "../../include/sucem_gb300.h"
#include "mf.h"

namespace sucem {
int fail(const std::string& msg, int code);
int cuda_fail(cudaError_t e, const char* where);
void count_launch(int k);

// the numeric handle is defined next to its kernels
struct MFHandle;
MFHandle* mf_new();
void mf_delete(MFHandle* h);
MFSymbolic& mf_sym(MFHandle* h);

}  // namespace sucem

struct sucem_lu {
  sucem::MFHandle* h = nullptr;
};

using sucem::cuda_fail;
using sucem::fail;

extern "C" {

int sucem_lu_analyse(int64_t n, const int32_t* indptr, const int32_t* indices, const double* xyz,
                     int leaf_size, sucem_lu** out) {
  if (!indptr || !indices || !out) return fail("null argument", SUCEM_ERR_ARG);
  *out = nullptr;
  sucem_lu* lu = new (std::nothrow) sucem_lu();
  if (!lu) return fail("out of host memory", SUCEM_ERR_MEMORY);
  lu->h = sucem::mf_new();
  std::string err;
  try {
    err = sucem::mf_analyse(sucem::mf_sym(lu->h), n, indptr, indices, xyz, leaf_size);
  } catch (const std::bad_alloc&) {
    err = "out of host memory";
  }
  if (!err.empty()) {
    sucem::mf_delete(lu->h);
    delete lu;
    return fail(err, SUCEM_ERR_ARG);
  }
  *out = lu;
  return SUCEM_OK;
}

int sucem_lu_analyse_cells(int64_t n, const int32_t* indptr, const int32_t* indices, int64_t nt,
                           int ndof_cell, const int32_t* cell_dofs, const double* cell_xyz,
                           int leaf_size, sucem_lu** out) {
  if (!indptr || !indices || !cell_dofs || !cell_xyz || !out)
    return fail("null argument", SUCEM_ERR_ARG);
  *out = nullptr;
  sucem_lu* lu = new (std::nothrow) sucem_lu();
  if (!lu) return fail("out of host memory", SUCEM_ERR_MEMORY);
  lu->h = sucem::mf_new();
  std::string err;
  try {
    err = sucem::mf_analyse_cells(sucem::mf_sym(lu->h), n, indptr, indices, nt, ndof_cell,
                                  cell_dofs, cell_xyz, leaf_size);
  } catch (const std::bad_alloc&) {
    err = "out of host memory";
  }
  if (!err.empty()) {
    sucem::mf_delete(lu->h);
    delete lu;
    return fail(err, SUCEM_ERR_ARG);
  }
  *out = lu;
  return SUCEM_OK;
}

void sucem_lu_destroy(sucem_lu* lu) {
  if (!lu) return;
  sucem::mf_delete(lu->h);
  delete lu;
}

int sucem_lu_info(const sucem_lu* lu, double* out) {
  if (!lu || !out) return fail("null argument", SUCEM_ERR_ARG);
  const sucem::MFSymbolic& s = sucem::mf_sym(lu->h);
  out[0] = (double)s.n;
  out[1] = (double)s.nnz;
  out[2] = (double)s.nodes.size();
  out[3] = (double)(s.max_level + 1);
  out[4] = (double)s.arena;
  out[5] = s.flops;
  out[6] = (double)s.max_front;
  return SUCEM_OK;
}

int sucem_lu_fronts(const sucem_lu* lu, int64_t* out) {
  if (!lu || !out) return fail("null argument", SUCEM_ERR_ARG);
  const sucem::MFSymbolic& s = sucem::mf_sym(lu->h);
  for (size_t i = 0; i < s.nodes.size(); ++i) {
    out[3 * i] = s.nodes[i].level;
    out[3 * i + 1] = s.nodes[i].k;
    out[3 * i + 2] = s.nodes[i].f;
  }
  return SUCEM_OK;
}

int sucem_lu_copy_perm(const sucem_lu* lu, int64_t* perm) {
  if (!lu || !perm) return fail("null argument", SUCEM_ERR_ARG);
  const sucem::MFSymbolic& s = sucem::mf_sym(lu->h);
  for (int64_t i = 0; i < s.n; ++i) perm[i] = s.perm[i];
  return SUCEM_OK;
}

int sucem_lu_factor(sucem_lu* lu, int dtype, const void* vals, double pivot_tol, void* stream) {
  if (!lu || !vals) return fail("null argument", SUCEM_ERR_ARG);
  if (dtype < SUCEM_F32 || dtype > SUCEM_C128) return fail("bad dtype", SUCEM_ERR_ARG);
  cudaStream_t st = (cudaStream_t)stream;
  // the pivot threshold pivot_tol * max|a_ij| is formed on the device, so a
  // factorisation is fully asynchronous on its stream
  cudaError_t e = sucem::mf_factor(*lu->h, dtype, vals, pivot_tol, st);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_lu_factor");
  return SUCEM_OK;
}

int sucem_lu_solve(sucem_lu* lu, int io_dtype, const void* b, void* x, void* stream) {
  if (!lu || !b || !x) return fail("null argument", SUCEM_ERR_ARG);
  // the first solve after a factorisation waits for it and refuses a factor
  // whose tensor-core update gave up waiting (its flag is device-side)
  if (sucem::mf_factor_status(*lu->h) == -1)
    return fail("the factorisation is invalid: a bounded wait of its tensor-core update gave up",
                SUCEM_ERR_STATE);
  cudaError_t e = sucem::mf_solve(*lu->h, io_dtype, b, x, (cudaStream_t)stream);
  if (e == cudaErrorNotReady) return fail("factor before solving", SUCEM_ERR_STATE);
  if (e == cudaErrorInvalidValue)
    return fail("solve dtype must match the factor (or its double-precision twin)", SUCEM_ERR_ARG);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_lu_solve");
  return SUCEM_OK;
}

int sucem_lu_perturbed(sucem_lu* lu) { return lu ? sucem::mf_perturbed(*lu->h) : 0; }

int sucem_lu_status(sucem_lu* lu) {
  if (!lu) return fail("null argument", SUCEM_ERR_ARG);
  const int st = sucem::mf_factor_status(*lu->h);
  if (st == -2) return fail("not factored (or the factorisation failed)", SUCEM_ERR_STATE);
  if (st == -1)
    return fail("the factorisation is invalid: a bounded wait of its tensor-core update gave up",
                SUCEM_ERR_STATE);
  return SUCEM_OK;
}

int sucem_lu_inject_timeout(sucem_lu* lu) {
  if (!lu) return fail("null argument", SUCEM_ERR_ARG);
  cudaError_t e = sucem::mf_mark_timed_out(*lu->h);
  if (e == cudaErrorNotReady) return fail("factor before injecting", SUCEM_ERR_STATE);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_lu_inject_timeout");
  return SUCEM_OK;
}

int sucem_selftest_bounded_wait(int polls, int* gave_up) {
  if (!gave_up || polls < 1) return fail("gave_up must be non-null and polls >= 1", SUCEM_ERR_ARG);
  cudaError_t e = sucem::mf_wait_selftest(polls, gave_up);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_selftest_bounded_wait");
  return SUCEM_OK;
}

int sucem_lu_configure(sucem_lu* lu, int superpanel, int panel_min_k) {
  if (!lu) return fail("null argument", SUCEM_ERR_ARG);
  cudaError_t e = sucem::mf_configure(*lu->h, superpanel, panel_min_k);
  if (e == cudaErrorInvalidValue)
    return fail("superpanel must be 0 or a positive multiple of 64, panel_min_k >= 0", SUCEM_ERR_ARG);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_lu_configure");
  return SUCEM_OK;
}

int sucem_lu_kernel_stats(sucem_lu* lu, double* out) {
  if (!lu || !out) return fail("null argument", SUCEM_ERR_ARG);
  sucem::mf_tc_stats(*lu->h, out);
  return SUCEM_OK;
}

}  // extern "C"
