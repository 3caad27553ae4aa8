// Current point sources: point location and N1curl basis evaluation on the
// GPU, the replacement of calc_pointsource_contrib
// (sucemfem/Sources/point_source.py:49-94: CGAL point location, then FIAT
// evaluate_basis_all, contribution N_i(p) . J).
//
// Cell rule: among the cells whose closure contains the point (barycentric
// coordinates >= -1e-12) the lowest cell index is taken.  Points on a
// shared face/edge/vertex are thereby resolved deterministically; the
// reference takes whichever cell its CGAL search returns first.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "../../include/sucem_gb300.h"
#include "device.h"
#include "handle.h"
#include "n1curl_tables.h"

namespace sucem {
int fail(const std::string& msg, int code);
int cuda_fail(cudaError_t e, const char* where);
void count_launch(int k);

namespace {

__constant__ double c_nb1[6][3][10];
__constant__ double c_nb2[20][3][10];

__device__ void jac(const double* xyz, int4 v, double J[3][3], double x0[3]) {
  for (int r = 0; r < 3; ++r) x0[r] = xyz[3 * (int64_t)v.x + r];
  const int vv[3] = {v.y, v.z, v.w};
  for (int i = 0; i < 3; ++i)
    for (int r = 0; r < 3; ++r) J[r][i] = xyz[3 * (int64_t)vv[i] + r] - x0[r];
}

__device__ void inv3(const double J[3][3], double Ji[3][3]) {
  const double m00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double m01 = J[1][0] * J[2][2] - J[1][2] * J[2][0];
  const double m02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double det = J[0][0] * m00 - J[0][1] * m01 + J[0][2] * m02;
  const double id = 1.0 / det;
  Ji[0][0] = m00 * id;
  Ji[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) * id;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  Ji[1][0] = -m01 * id;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  Ji[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) * id;
  Ji[2][0] = m02 * id;
  Ji[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) * id;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
}

// one thread per cell, loop over points; lowest containing cell wins
__global__ void locate_kernel(int64_t nt, const int4* __restrict__ cells,
                              const double* __restrict__ xyz, const double* __restrict__ pts,
                              int npts, int* __restrict__ cell_out) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nt) return;
  const int4 v = cells[c];
  double J[3][3], Ji[3][3], x0[3];
  jac(xyz, v, J, x0);
  inv3(J, Ji);
  for (int p = 0; p < npts; ++p) {
    const double d0 = pts[3 * p] - x0[0], d1 = pts[3 * p + 1] - x0[1], d2 = pts[3 * p + 2] - x0[2];
    const double l1 = Ji[0][0] * d0 + Ji[0][1] * d1 + Ji[0][2] * d2;
    const double l2 = Ji[1][0] * d0 + Ji[1][1] * d1 + Ji[1][2] * d2;
    const double l3 = Ji[2][0] * d0 + Ji[2][1] * d1 + Ji[2][2] * d2;
    const double l0 = 1.0 - l1 - l2 - l3;
    const double tol = -1e-12;
    if (l0 >= tol && l1 >= tol && l2 >= tol && l3 >= tol) atomicMin(&cell_out[p], (int)c);
  }
}

// one warp per point, lane = local basis function
template <int ND>
__global__ void evaluate_kernel(int64_t nt, const int4* __restrict__ cells,
                                const double* __restrict__ xyz,
                                const double* __restrict__ pts, const double* __restrict__ vals,
                                int npts, const int* __restrict__ cell_in,
                                double* __restrict__ contrib) {
  const int p = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (p >= npts) return;
  const int c = cell_in[p];
  if (c < 0 || c >= nt) return;  // not located: host reports it
  double J[3][3], Ji[3][3], x0[3];
  jac(xyz, cells[c], J, x0);
  inv3(J, Ji);
  double d[3] = {pts[3 * p] - x0[0], pts[3 * p + 1] - x0[1], pts[3 * p + 2] - x0[2]};
  double X[3];
  for (int r = 0; r < 3; ++r) X[r] = Ji[r][0] * d[0] + Ji[r][1] * d[1] + Ji[r][2] * d[2];
  if (lane >= ND) return;
  const double mono[10] = {1.0,         X[0],        X[1],        X[2],        X[0] * X[0],
                           X[1] * X[1], X[2] * X[2], X[0] * X[1], X[0] * X[2], X[1] * X[2]};
  double nh[3];
  for (int q = 0; q < 3; ++q) {
    double s = 0;
    for (int m = 0; m < 10; ++m) s += (ND == 6 ? c_nb1[lane % 6][q][m] : c_nb2[lane][q][m]) * mono[m];
    nh[q] = s;
  }
  // physical N = J^-T N_hat  ->  N_i = sum_q Ji[q][i] nh[q]
  double n[3];
  for (int i = 0; i < 3; ++i) n[i] = Ji[0][i] * nh[0] + Ji[1][i] * nh[1] + Ji[2][i] * nh[2];
  // value is complex: vals[p][i] = (re, im)
  const double* v = vals + 6 * (int64_t)p;
  const double re = n[0] * v[0] + n[1] * v[2] + n[2] * v[4];
  const double im = n[0] * v[1] + n[1] * v[3] + n[2] * v[5];
  contrib[2 * ((int64_t)p * ND + lane)] = re;
  contrib[2 * ((int64_t)p * ND + lane) + 1] = im;
}

bool g_tables_loaded[64] = {false};

}  // namespace
}  // namespace sucem

extern "C" int sucem_point_sources(const sucem_space* sp, const double* pts,
                                   const double* values, int npts, int32_t* cells_out,
                                   double* contrib, void* stream) {
  using namespace sucem;
  const DeviceSpace* d = sp ? sp->s.dev : nullptr;
  if (!d) return fail("space is not on a device", SUCEM_ERR_STATE);
  if (npts < 0) return fail("negative point count", SUCEM_ERR_ARG);
  if (npts == 0) return SUCEM_OK;
  if (!pts || !values || !cells_out || !contrib) return fail("null argument", SUCEM_ERR_ARG);
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !g_tables_loaded[dev]) {
    cudaError_t e = cudaMemcpyToSymbol(c_nb1, NB1, sizeof(NB1));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_nb2, NB2, sizeof(NB2));
    if (e != cudaSuccess) return cuda_fail(e, "sucem_point_sources tables");
    g_tables_loaded[dev] = true;
  }
  cudaError_t e = cudaMemsetAsync(cells_out, 0x7f, sizeof(int32_t) * npts, s);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_point_sources memset");
  // 0x7f7f7f7f (>= nt for any supported mesh) marks a point outside the mesh
  const int threads = 256;
  locate_kernel<<<(unsigned)((d->nt + threads - 1) / threads), threads, 0, s>>>(
      d->nt, d->cells, d->xyz, pts, npts, cells_out);
  const unsigned eb = (unsigned)(((int64_t)npts * 32 + threads - 1) / threads);
  if (d->nd == 6)
    evaluate_kernel<6><<<eb, threads, 0, s>>>(d->nt, d->cells, d->xyz, pts, values, npts, cells_out,
                                              contrib);
  else
    evaluate_kernel<20><<<eb, threads, 0, s>>>(d->nt, d->cells, d->xyz, pts, values, npts, cells_out,
                                               contrib);
  e = cudaGetLastError();
  count_launch(2);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_point_sources");
}
