// Field evaluation on the GPU: point location and N1curl basis evaluation
// for the current point sources (replacing calc_pointsource_contrib,
// sucemfem/Sources/point_source.py:49-94: CGAL point location, then FIAT
// evaluate_basis_all, contribution N_i(p) . J), the field at arbitrary
// points (Reconstruct.reconstruct_points,
// sucemfem/PostProcessing/PostProcessing.py:27-60) and the real power flux
// through the boundary (SurfaceFlux.calc_flux,
// sucemfem/PostProcessing/power_flux.py:11-60).
//
// Cell rule: among the cells whose closure contains the point (barycentric
// coordinates >= -1e-12) the lowest cell index is taken.  Points on a
// shared face/edge/vertex are thereby resolved deterministically; the
// reference takes whichever cell its CGAL search returns first.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <vector>

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

// one thread per point: the cells of the point's grid bin are tested
// (barycentric coordinates >= -1e-12); the lowest containing cell wins,
// 0x7f7f7f7f when none contains it
struct Grid {
  const int32_t* ptr;
  const int32_t* cells;
  int n[3];
  double lo[3], inv[3];
};

__global__ void locate_kernel(Grid g, const int4* __restrict__ cells,
                              const double* __restrict__ xyz, const double* __restrict__ pts,
                              int npts, int* __restrict__ cell_out) {
  const int p = (int)((int64_t)blockIdx.x * blockDim.x + threadIdx.x);
  if (p >= npts) return;
  const double P[3] = {pts[3 * p], pts[3 * p + 1], pts[3 * p + 2]};
  int b[3];
  for (int r = 0; r < 3; ++r) {
    const double f = (P[r] - g.lo[r]) * g.inv[r];
    b[r] = f < 0 ? -1 : (f >= g.n[r] ? g.n[r] : (int)f);
  }
  int best = 0x7f7f7f7f;
  if (b[0] >= 0 && b[0] < g.n[0] && b[1] >= 0 && b[1] < g.n[1] && b[2] >= 0 && b[2] < g.n[2]) {
    const int64_t bin = ((int64_t)b[2] * g.n[1] + b[1]) * g.n[0] + b[0];
    for (int32_t k = g.ptr[bin]; k < g.ptr[bin + 1]; ++k) {
      const int c = g.cells[k];
      if (c >= best) continue;
      double J[3][3], Ji[3][3], x0[3];
      jac(xyz, cells[c], J, x0);
      inv3(J, Ji);
      const double d0 = P[0] - x0[0], d1 = P[1] - x0[1], d2 = P[2] - x0[2];
      const double l1 = Ji[0][0] * d0 + Ji[0][1] * d1 + Ji[0][2] * d2;
      const double l2 = Ji[1][0] * d0 + Ji[1][1] * d1 + Ji[1][2] * d2;
      const double l3 = Ji[2][0] * d0 + Ji[2][1] * d1 + Ji[2][2] * d2;
      const double l0 = 1.0 - l1 - l2 - l3;
      const double tol = -1e-12;
      if (l0 >= tol && l1 >= tol && l2 >= tol && l3 >= tol) best = c;
    }
  }
  cell_out[p] = best;
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

// ---- surface power flux ----
// 3 x 3 collapsed Gauss-Jacobi rule on the reference triangle (Gauss-Jacobi
// (alpha = 1) in the collapsed direction, Gauss-Legendre in the other): exact
// to degree 5 (the flux integrand has degree 2 * order - 1), and the rule the
// reference's form compiler integrates its far-field forms with
constexpr int kFaceQ = 9;
// UFC local faces: face f is opposite vertex f
__constant__ int c_face_vert[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
__constant__ double c_fw[kFaceQ];
// reference basis value (0..2) and curl (3..5) at the quadrature points of
// every local face, per order
__constant__ double c_fq1[4][kFaceQ][6][6];
__constant__ double c_fq2[4][kFaceQ][20][6];
// reference coordinates of the quadrature points of every local face
__constant__ double c_fX[4][kFaceQ][3];
bool g_face_loaded[64] = {false};

template <int ND>
void face_tables(const double (*nb)[3][10], double (*out)[kFaceQ][ND][6], double* w,
                 double (*Xo)[kFaceQ][3]) {
  // Gauss-Jacobi (1, 0) and Gauss-Legendre nodes and weights on [-1, 1]
  const double ga[3] = {-0.8228240809745921, -0.1810662711185305, 0.5753189235216941};
  const double gwa[3] = {0.8037276549558384, 0.9169644254383448, 0.2793079196058167};
  const double gb[3] = {-0.7745966692414834, 0.0, 0.7745966692414834};
  const double gwb[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
  const double rv[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  const int fv[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
  for (int f = 0; f < 4; ++f)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const int q = 3 * i + j;
        const double u = 0.5 * (ga[i] + 1.0), v = 0.5 * (gb[j] + 1.0);
        const double s = u, t = v * (1.0 - u);
        w[q] = 0.125 * gwa[i] * gwb[j];  // the Jacobi weight carries (1 - u)
        double X[3];
        for (int r = 0; r < 3; ++r)
          X[r] = rv[fv[f][0]][r] + s * (rv[fv[f][1]][r] - rv[fv[f][0]][r]) +
                 t * (rv[fv[f][2]][r] - rv[fv[f][0]][r]);
        for (int r = 0; r < 3; ++r) Xo[f][q][r] = X[r];
        const double mono[10] = {1.0,         X[0],        X[1],        X[2],        X[0] * X[0],
                                 X[1] * X[1], X[2] * X[2], X[0] * X[1], X[0] * X[2], X[1] * X[2]};
        for (int a = 0; a < ND; ++a) {
          double d[3][3];  // d[p][r] = dN_p / dX_r
          for (int p = 0; p < 3; ++p) {
            const double* c = nb[a][p];
            double val = 0;
            for (int m = 0; m < 10; ++m) val += c[m] * mono[m];
            out[f][q][a][p] = val;
            d[p][0] = c[1] + 2 * c[4] * X[0] + c[7] * X[1] + c[8] * X[2];
            d[p][1] = c[2] + 2 * c[5] * X[1] + c[7] * X[0] + c[9] * X[2];
            d[p][2] = c[3] + 2 * c[6] * X[2] + c[8] * X[0] + c[9] * X[1];
          }
          out[f][q][a][3] = d[2][1] - d[1][2];
          out[f][q][a][4] = d[0][2] - d[2][0];
          out[f][q][a][5] = d[1][0] - d[0][1];
        }
      }
}

__device__ __forceinline__ double2 ld_c(const double2* x, int64_t i) { return x[i]; }
__device__ __forceinline__ double2 ld_c(const float2* x, int64_t i) {
  const float2 v = x[i];
  return make_double2(v.x, v.y);
}

// one thread per cell: the flux through its exterior facets (in local face
// order), written to part[c] (0 for interior cells)
template <int ND, typename T>
__global__ void surface_flux_kernel(int64_t nt, const int4* __restrict__ cells,
                                    const double* __restrict__ xyz,
                                    const uint8_t* __restrict__ ext_mask,
                                    const int32_t* __restrict__ cell_dofs,
                                    const T* __restrict__ x, const double* __restrict__ mu_r,
                                    double scale, double* __restrict__ part) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nt) return;
  const int mask = ext_mask[c];
  double acc = 0.0;
  if (mask) {
    const int4 v = cells[c];
    double J[3][3], Ji[3][3], x0[3];
    jac(xyz, v, J, x0);
    inv3(J, Ji);
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                       J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                       J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    const int vid[4] = {v.x, v.y, v.z, v.w};
    double2 xe[ND];
    for (int a = 0; a < ND; ++a) xe[a] = ld_c(x, cell_dofs[c * ND + a]);
    const double inv_mu = mu_r ? 1.0 / mu_r[c] : 1.0;
    for (int f = 0; f < 4; ++f) {
      if (!(mask >> f & 1)) continue;
      double P[3][3];
      for (int k = 0; k < 3; ++k)
        for (int r = 0; r < 3; ++r) P[k][r] = xyz[3 * (int64_t)vid[c_face_vert[f][k]] + r];
      double cr[3] = {(P[1][1] - P[0][1]) * (P[2][2] - P[0][2]) - (P[1][2] - P[0][2]) * (P[2][1] - P[0][1]),
                      (P[1][2] - P[0][2]) * (P[2][0] - P[0][0]) - (P[1][0] - P[0][0]) * (P[2][2] - P[0][2]),
                      (P[1][0] - P[0][0]) * (P[2][1] - P[0][1]) - (P[1][1] - P[0][1]) * (P[2][0] - P[0][0])};
      // outward: away from the vertex opposite the face
      double o = 0;
      for (int r = 0; r < 3; ++r) o += cr[r] * (P[0][r] - xyz[3 * (int64_t)vid[f] + r]);
      const double sg = o < 0 ? -1.0 : 1.0;
      const double area2 = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
      double n[3];
      for (int r = 0; r < 3; ++r) n[r] = sg * cr[r] / area2;
      double s = 0;
      for (int q = 0; q < kFaceQ; ++q) {
        double eh[2][3] = {{0, 0, 0}, {0, 0, 0}}, ch[2][3] = {{0, 0, 0}, {0, 0, 0}};
        for (int a = 0; a < ND; ++a) {
          const double* t = ND == 6 ? c_fq1[f][q][a % 6] : c_fq2[f][q][a];
          for (int r = 0; r < 3; ++r) {
            eh[0][r] += xe[a].x * t[r];
            eh[1][r] += xe[a].y * t[r];
            ch[0][r] += xe[a].x * t[3 + r];
            ch[1][r] += xe[a].y * t[3 + r];
          }
        }
        // E = J^-T E_hat, curl E = J curl E_hat / det J  (Re, Im)
        double E[2][3], C[2][3];
        for (int k = 0; k < 2; ++k)
          for (int i = 0; i < 3; ++i) {
            E[k][i] = Ji[0][i] * eh[k][0] + Ji[1][i] * eh[k][1] + Ji[2][i] * eh[k][2];
            C[k][i] = (J[i][0] * ch[k][0] + J[i][1] * ch[k][1] + J[i][2] * ch[k][2]) / det * inv_mu;
          }
        // n . (E_r x (-curl E_i) + E_i x curl E_r)
        double g3[3];
        for (int i = 0; i < 3; ++i) {
          const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
          g3[i] = -(E[0][i1] * C[1][i2] - E[0][i2] * C[1][i1]) + (E[1][i1] * C[0][i2] - E[1][i2] * C[0][i1]);
        }
        s += c_fw[q] * (n[0] * g3[0] + n[1] * g3[1] + n[2] * g3[2]);
      }
      acc += s * area2;
    }
  }
  part[c] = acc * scale;
}

// one block: out[0] = sum of part[0:n) in a fixed order
__global__ void __launch_bounds__(1024) sum_kernel(int64_t n, const double* __restrict__ part,
                                                   double* __restrict__ out) {
  __shared__ double red[1024];
  double s = 0;
  for (int64_t i = threadIdx.x; i < n; i += 1024) s += part[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int h = 512; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = red[0];
}

// ---- field at points: one warp per point, lane = local basis function ----
template <int ND, typename T>
__global__ void reconstruct_kernel(int64_t nt, const int4* __restrict__ cells,
                                   const double* __restrict__ xyz,
                                   const int32_t* __restrict__ cell_dofs, const T* __restrict__ x,
                                   const double* __restrict__ pts, int npts,
                                   const int* __restrict__ cell_in, double* __restrict__ E) {
  const int p = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (p >= npts) return;
  const int c = cell_in[p];
  double* out = E + 6 * (int64_t)p;
  if (c < 0 || c >= nt) {
    if (lane < 6) out[lane] = __longlong_as_double(0x7ff8000000000000LL);  // NaN: outside
    return;
  }
  double J[3][3], Ji[3][3], x0[3];
  jac(xyz, cells[c], J, x0);
  inv3(J, Ji);
  const double d[3] = {pts[3 * p] - x0[0], pts[3 * p + 1] - x0[1], pts[3 * p + 2] - x0[2]};
  double X[3];
  for (int r = 0; r < 3; ++r) X[r] = Ji[r][0] * d[0] + Ji[r][1] * d[1] + Ji[r][2] * d[2];
  double e[6] = {0, 0, 0, 0, 0, 0};
  if (lane < ND) {
    const double mono[10] = {1.0,         X[0],        X[1],        X[2],        X[0] * X[0],
                             X[1] * X[1], X[2] * X[2], X[0] * X[1], X[0] * X[2], X[1] * X[2]};
    double nh[3];
    for (int q = 0; q < 3; ++q) {
      double s = 0;
      for (int m = 0; m < 10; ++m) s += (ND == 6 ? c_nb1[lane % 6][q][m] : c_nb2[lane][q][m]) * mono[m];
      nh[q] = s;
    }
    const double2 xv = ld_c(x, cell_dofs[(int64_t)c * ND + lane]);
    for (int i = 0; i < 3; ++i) {
      const double ni = Ji[0][i] * nh[0] + Ji[1][i] * nh[1] + Ji[2][i] * nh[2];
      e[2 * i] = xv.x * ni;
      e[2 * i + 1] = xv.y * ni;
    }
  }
  for (int k = 0; k < 6; ++k)
    for (int o = 16; o > 0; o >>= 1) e[k] += __shfl_down_sync(~0u, e[k], o);
  if (lane == 0)
    for (int k = 0; k < 6; ++k) out[k] = e[k];
}

// ---- near-to-far-field transform (surface equivalence) ----
// per exterior facet (one thread), per quadrature point: the physical point,
// the weight (rule weight x twice the facet area), the equivalent electric
// current J = n x H with H = j curl E / (k0 Z0) and the magnetic current
// M = -n x E: 16 doubles per point (x3, w, J re/im x3, M re/im x3)
template <int ND, typename T>
__global__ void ntff_points_kernel(int64_t nfac, const int32_t* __restrict__ facets,
                                   const int4* __restrict__ cells, const double* __restrict__ xyz,
                                   const int32_t* __restrict__ cell_dofs, const T* __restrict__ x,
                                   double inv_k0z0, double* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nfac) return;
  const int c = facets[2 * i], f = facets[2 * i + 1];
  const int4 v = cells[c];
  double J[3][3], Ji[3][3], x0[3];
  jac(xyz, v, J, x0);
  inv3(J, Ji);
  const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  const int vid[4] = {v.x, v.y, v.z, v.w};
  double P[3][3];
  for (int k = 0; k < 3; ++k)
    for (int r = 0; r < 3; ++r) P[k][r] = xyz[3 * (int64_t)vid[c_face_vert[f][k]] + r];
  double cr[3] = {(P[1][1] - P[0][1]) * (P[2][2] - P[0][2]) - (P[1][2] - P[0][2]) * (P[2][1] - P[0][1]),
                  (P[1][2] - P[0][2]) * (P[2][0] - P[0][0]) - (P[1][0] - P[0][0]) * (P[2][2] - P[0][2]),
                  (P[1][0] - P[0][0]) * (P[2][1] - P[0][1]) - (P[1][1] - P[0][1]) * (P[2][0] - P[0][0])};
  double o = 0;
  for (int r = 0; r < 3; ++r) o += cr[r] * (P[0][r] - xyz[3 * (int64_t)vid[f] + r]);
  const double sg = o < 0 ? -1.0 : 1.0;
  const double area2 = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
  double n[3];
  for (int r = 0; r < 3; ++r) n[r] = sg * cr[r] / area2;
  double2 xe[ND];
  for (int a = 0; a < ND; ++a) xe[a] = ld_c(x, cell_dofs[(int64_t)c * ND + a]);
  for (int q = 0; q < kFaceQ; ++q) {
    double eh[2][3] = {{0, 0, 0}, {0, 0, 0}}, ch[2][3] = {{0, 0, 0}, {0, 0, 0}};
    for (int a = 0; a < ND; ++a) {
      const double* t = ND == 6 ? c_fq1[f][q][a % 6] : c_fq2[f][q][a];
      for (int r = 0; r < 3; ++r) {
        eh[0][r] += xe[a].x * t[r];
        eh[1][r] += xe[a].y * t[r];
        ch[0][r] += xe[a].x * t[3 + r];
        ch[1][r] += xe[a].y * t[3 + r];
      }
    }
    double E[2][3], H[2][3];
    for (int i3 = 0; i3 < 3; ++i3) {
      for (int k = 0; k < 2; ++k)
        E[k][i3] = Ji[0][i3] * eh[k][0] + Ji[1][i3] * eh[k][1] + Ji[2][i3] * eh[k][2];
      const double cre = (J[i3][0] * ch[0][0] + J[i3][1] * ch[0][1] + J[i3][2] * ch[0][2]) / det;
      const double cim = (J[i3][0] * ch[1][0] + J[i3][1] * ch[1][1] + J[i3][2] * ch[1][2]) / det;
      H[0][i3] = -cim * inv_k0z0;  // H = j curl E / (k0 Z0)
      H[1][i3] = cre * inv_k0z0;
    }
    double* o16 = out + 16 * (i * kFaceQ + q);
    for (int r = 0; r < 3; ++r)
      o16[r] = x0[r] + J[r][0] * c_fX[f][q][0] + J[r][1] * c_fX[f][q][1] + J[r][2] * c_fX[f][q][2];
    o16[3] = c_fw[q] * area2;
    for (int r = 0; r < 3; ++r) {
      const int r1 = (r + 1) % 3, r2 = (r + 2) % 3;
      for (int k = 0; k < 2; ++k) {
        o16[4 + 2 * r + k] = n[r1] * H[k][r2] - n[r2] * H[k][r1];       // n x H
        o16[10 + 2 * r + k] = -(n[r1] * E[k][r2] - n[r2] * E[k][r1]);   // -n x E
      }
    }
  }
}

// one block per direction (theta, phi in radians): N = sum w J e^{j k0 r.rhat},
// L = sum w M e^{j k0 r.rhat} in a fixed order, then
// out[12 d ..] = E_theta, E_phi, L_theta, L_phi, N_theta, N_phi (complex)
__global__ void __launch_bounds__(256) ntff_dir_kernel(int64_t npts, const double* __restrict__ pts,
                                                       const double* __restrict__ theta,
                                                       const double* __restrict__ phi, double k0,
                                                       double z0, double* __restrict__ out) {
  __shared__ double red[12][256];
  const int d = blockIdx.x;
  double st, ct, sp, cp;
  sincos(theta[d], &st, &ct);
  sincos(phi[d], &sp, &cp);
  const double rh[3] = {st * cp, st * sp, ct};
  double acc[12];
  for (int k = 0; k < 12; ++k) acc[k] = 0;
  for (int64_t i = threadIdx.x; i < npts; i += 256) {
    const double* p = pts + 16 * i;
    double s, c;
    sincos(k0 * (rh[0] * p[0] + rh[1] * p[1] + rh[2] * p[2]), &s, &c);
    const double w = p[3];
    for (int r = 0; r < 3; ++r) {
      const double jr = p[4 + 2 * r], ji = p[5 + 2 * r], mr = p[10 + 2 * r], mi = p[11 + 2 * r];
      acc[2 * r] += w * (jr * c - ji * s);
      acc[2 * r + 1] += w * (jr * s + ji * c);
      acc[6 + 2 * r] += w * (mr * c - mi * s);
      acc[7 + 2 * r] += w * (mr * s + mi * c);
    }
  }
  for (int k = 0; k < 12; ++k) red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h)
      for (int k = 0; k < 12; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double th[3] = {ct * cp, ct * sp, -st}, ph[3] = {-sp, cp, 0.0};
    double Nt[2] = {0, 0}, Np[2] = {0, 0}, Lt[2] = {0, 0}, Lp[2] = {0, 0};
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 2; ++k) {
        Nt[k] += th[r] * red[2 * r + k][0];
        Np[k] += ph[r] * red[2 * r + k][0];
        Lt[k] += th[r] * red[6 + 2 * r + k][0];
        Lp[k] += ph[r] * red[6 + 2 * r + k][0];
      }
    // r_fac = j k0 e^{-j k0} / (4 pi)
    double sk, ck;
    sincos(k0, &sk, &ck);
    const double fr = k0 * sk / (4 * 3.141592653589793), fi = k0 * ck / (4 * 3.141592653589793);
    const double ar = Lp[0] + z0 * Nt[0], ai = Lp[1] + z0 * Nt[1];   // E_theta = -r_fac a
    const double br = Lt[0] - z0 * Np[0], bi = Lt[1] - z0 * Np[1];   // E_phi = r_fac b
    double* o = out + 12 * (int64_t)d;
    o[0] = -(fr * ar - fi * ai);
    o[1] = -(fr * ai + fi * ar);
    o[2] = fr * br - fi * bi;
    o[3] = fr * bi + fi * br;
    o[4] = Lt[0];
    o[5] = Lt[1];
    o[6] = Lp[0];
    o[7] = Lp[1];
    o[8] = Nt[0];
    o[9] = Nt[1];
    o[10] = Np[0];
    o[11] = Np[1];
  }
}

// the location grid of a space: about two cells per bin, every cell listed
// in each bin its (slightly padded) bounding box overlaps
cudaError_t build_grid(const Space& hs, DeviceSpace* d) {
  if (d->bin_ptr) return cudaSuccess;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int64_t v = 0; v < hs.nv; ++v)
    for (int r = 0; r < 3; ++r) {
      lo[r] = std::min(lo[r], hs.coords[3 * v + r]);
      hi[r] = std::max(hi[r], hs.coords[3 * v + r]);
    }
  double ext[3], vol = 1.0;
  for (int r = 0; r < 3; ++r) {
    ext[r] = std::max(hi[r] - lo[r], 1e-300);
    const double pad = 1e-9 * ext[r] + 1e-300;
    lo[r] -= pad;
    hi[r] += pad;
    ext[r] = hi[r] - lo[r];
    vol *= ext[r];
  }
  const double target = std::max(1.0, (double)hs.nt / 2.0);
  const double h = std::cbrt(vol / target);
  int n[3];
  for (int r = 0; r < 3; ++r) n[r] = std::max(1, std::min(1024, (int)std::ceil(ext[r] / h)));
  const int64_t nbins = (int64_t)n[0] * n[1] * n[2];
  std::vector<int32_t> cnt(nbins + 1, 0);
  auto range = [&](int64_t c, int b0[3], int b1[3]) {
    double cl[3] = {1e300, 1e300, 1e300}, ch[3] = {-1e300, -1e300, -1e300};
    for (int k = 0; k < 4; ++k)
      for (int r = 0; r < 3; ++r) {
        const double x = hs.coords[3 * (int64_t)hs.cells[4 * c + k] + r];
        cl[r] = std::min(cl[r], x);
        ch[r] = std::max(ch[r], x);
      }
    for (int r = 0; r < 3; ++r) {
      const double pad = 1e-9 * ext[r];
      b0[r] = std::max(0, std::min(n[r] - 1, (int)((cl[r] - pad - lo[r]) / ext[r] * n[r])));
      b1[r] = std::max(0, std::min(n[r] - 1, (int)((ch[r] + pad - lo[r]) / ext[r] * n[r])));
    }
  };
  for (int pass = 0; pass < 2; ++pass) {
    std::vector<int32_t> fill;
    if (pass == 1) {
      for (int64_t i = 0; i < nbins; ++i) cnt[i + 1] += cnt[i];
      fill.assign(cnt.begin(), cnt.end() - 1);
    }
    std::vector<int32_t> out(pass == 1 ? cnt[nbins] : 0);
    for (int64_t c = 0; c < hs.nt; ++c) {
      int b0[3], b1[3];
      range(c, b0, b1);
      for (int z = b0[2]; z <= b1[2]; ++z)
        for (int y = b0[1]; y <= b1[1]; ++y)
          for (int x = b0[0]; x <= b1[0]; ++x) {
            const int64_t bin = ((int64_t)z * n[1] + y) * n[0] + x;
            if (pass == 0)
              cnt[bin + 1]++;
            else
              out[fill[bin]++] = (int32_t)c;
          }
    }
    if (pass == 1) {
      cudaError_t e = cudaMalloc((void**)&d->bin_ptr, cnt.size() * sizeof(int32_t));
      if (e == cudaSuccess)
        e = cudaMemcpy(d->bin_ptr, cnt.data(), cnt.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = cudaMalloc((void**)&d->bin_cells, std::max<size_t>(1, out.size()) * sizeof(int32_t));
      if (e == cudaSuccess && !out.empty())
        e = cudaMemcpy(d->bin_cells, out.data(), out.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
      if (e != cudaSuccess) {
        if (d->bin_ptr) cudaFree(d->bin_ptr);
        if (d->bin_cells) cudaFree(d->bin_cells);
        d->bin_ptr = d->bin_cells = nullptr;
        return e;
      }
    }
  }
  for (int r = 0; r < 3; ++r) {
    d->grid_n[r] = n[r];
    d->grid_lo[r] = lo[r];
    d->grid_inv[r] = n[r] / ext[r];
  }
  return cudaSuccess;
}

Grid grid_of(const DeviceSpace* d) {
  Grid g;
  g.ptr = d->bin_ptr;
  g.cells = d->bin_cells;
  for (int r = 0; r < 3; ++r) {
    g.n[r] = d->grid_n[r];
    g.lo[r] = d->grid_lo[r];
    g.inv[r] = d->grid_inv[r];
  }
  return g;
}

cudaError_t load_point_tables(int dev) {
  if (dev < 64 && g_tables_loaded[dev]) return cudaSuccess;
  cudaError_t e = cudaMemcpyToSymbol(c_nb1, NB1, sizeof(NB1));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_nb2, NB2, sizeof(NB2));
  if (e == cudaSuccess && dev < 64) g_tables_loaded[dev] = true;
  return e;
}

cudaError_t load_face_tables(int dev) {
  if (dev < 64 && g_face_loaded[dev]) return cudaSuccess;
  static double t1[4][kFaceQ][6][6], t2[4][kFaceQ][20][6], w[kFaceQ], X[4][kFaceQ][3];
  face_tables<6>(NB1, t1, w, X);
  face_tables<20>(NB2, t2, w, X);
  cudaError_t e = cudaMemcpyToSymbol(c_fq1, t1, sizeof(t1));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_fq2, t2, sizeof(t2));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_fw, w, sizeof(w));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_fX, X, sizeof(X));
  if (e == cudaSuccess && dev < 64) g_face_loaded[dev] = true;
  return e;
}

}  // namespace
}  // namespace sucem

extern "C" int sucem_point_sources(const sucem_space* sp, const double* pts,
                                   const double* values, int npts, int32_t* cells_out,
                                   double* contrib, void* stream) {
  using namespace sucem;
  const DeviceSpace* d = sp ? sp->s.dev : nullptr;
  if (!d) return fail("space is not on a device", SUCEM_ERR_STATE);
  if (d->nd > 20) return fail("supported for basis orders 1 and 2 only", SUCEM_ERR_ARG);
  if (npts < 0) return fail("negative point count", SUCEM_ERR_ARG);
  if (npts == 0) return SUCEM_OK;
  if (!pts || !values || !cells_out || !contrib) return fail("null argument", SUCEM_ERR_ARG);
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaError_t e = load_point_tables(dev);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_point_sources tables");
  e = build_grid(sp->s, const_cast<DeviceSpace*>(d));
  if (e != cudaSuccess) return cuda_fail(e, "sucem_point_sources grid");
  // 0x7f7f7f7f (>= nt for any supported mesh) marks a point outside the mesh
  const int threads = 256;
  locate_kernel<<<(unsigned)((npts + threads - 1) / threads), threads, 0, s>>>(
      grid_of(d), d->cells, d->xyz, pts, npts, cells_out);
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

extern "C" int sucem_reconstruct_points(const sucem_space* sp, int dtype, const void* x,
                                        const double* pts, int npts, int32_t* cells_out,
                                        double* E, void* stream) {
  using namespace sucem;
  const DeviceSpace* d = sp ? sp->s.dev : nullptr;
  if (!d) return fail("space is not on a device", SUCEM_ERR_STATE);
  if (d->nd > 20) return fail("supported for basis orders 1 and 2 only", SUCEM_ERR_ARG);
  if (dtype != SUCEM_C64 && dtype != SUCEM_C128) return fail("dtype must be complex", SUCEM_ERR_ARG);
  if (npts < 0) return fail("negative point count", SUCEM_ERR_ARG);
  if (npts == 0) return SUCEM_OK;
  if (!x || !pts || !cells_out || !E) return fail("null argument", SUCEM_ERR_ARG);
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaError_t e = load_point_tables(dev);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_reconstruct_points tables");
  e = build_grid(sp->s, const_cast<DeviceSpace*>(d));
  if (e != cudaSuccess) return cuda_fail(e, "sucem_reconstruct_points grid");
  const int threads = 256;
  locate_kernel<<<(unsigned)((npts + threads - 1) / threads), threads, 0, s>>>(
      grid_of(d), d->cells, d->xyz, pts, npts, cells_out);
  const unsigned eb = (unsigned)(((int64_t)npts * 32 + threads - 1) / threads);
  if (d->nd == 6 && dtype == SUCEM_C128)
    reconstruct_kernel<6, double2><<<eb, threads, 0, s>>>(d->nt, d->cells, d->xyz, d->cell_dofs,
                                                          (const double2*)x, pts, npts, cells_out, E);
  else if (d->nd == 6)
    reconstruct_kernel<6, float2><<<eb, threads, 0, s>>>(d->nt, d->cells, d->xyz, d->cell_dofs,
                                                         (const float2*)x, pts, npts, cells_out, E);
  else if (dtype == SUCEM_C128)
    reconstruct_kernel<20, double2><<<eb, threads, 0, s>>>(d->nt, d->cells, d->xyz, d->cell_dofs,
                                                           (const double2*)x, pts, npts, cells_out, E);
  else
    reconstruct_kernel<20, float2><<<eb, threads, 0, s>>>(d->nt, d->cells, d->xyz, d->cell_dofs,
                                                          (const float2*)x, pts, npts, cells_out, E);
  e = cudaGetLastError();
  count_launch(2);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_reconstruct_points");
}

extern "C" int sucem_surface_flux(const sucem_space* sp, int dtype, const void* x, double k0,
                                  const double* mu_r, double* part, double* out, void* stream) {
  using namespace sucem;
  const DeviceSpace* d = sp ? sp->s.dev : nullptr;
  if (!d) return fail("space is not on a device", SUCEM_ERR_STATE);
  if (d->nd > 20) return fail("supported for basis orders 1 and 2 only", SUCEM_ERR_ARG);
  if (dtype != SUCEM_C64 && dtype != SUCEM_C128) return fail("dtype must be complex", SUCEM_ERR_ARG);
  if (!(k0 > 0)) return fail("k0 must be positive", SUCEM_ERR_ARG);
  if (!x || !part || !out) return fail("null argument", SUCEM_ERR_ARG);
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaError_t e = load_face_tables(dev);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_surface_flux tables");
  // Consts.py: Z0 = mu0 * c0
  const double z0 = 3.141592653589793 * 4e-7 * 299792458.0;
  const double scale = 1.0 / (k0 * z0);
  const int threads = 128;
  const unsigned blocks = (unsigned)((d->nt + threads - 1) / threads);
  if (d->nd == 6 && dtype == SUCEM_C128)
    surface_flux_kernel<6, double2><<<blocks, threads, 0, s>>>(
        d->nt, d->cells, d->xyz, d->ext_mask, d->cell_dofs, (const double2*)x, mu_r, scale, part);
  else if (d->nd == 6)
    surface_flux_kernel<6, float2><<<blocks, threads, 0, s>>>(
        d->nt, d->cells, d->xyz, d->ext_mask, d->cell_dofs, (const float2*)x, mu_r, scale, part);
  else if (dtype == SUCEM_C128)
    surface_flux_kernel<20, double2><<<blocks, threads, 0, s>>>(
        d->nt, d->cells, d->xyz, d->ext_mask, d->cell_dofs, (const double2*)x, mu_r, scale, part);
  else
    surface_flux_kernel<20, float2><<<blocks, threads, 0, s>>>(
        d->nt, d->cells, d->xyz, d->ext_mask, d->cell_dofs, (const float2*)x, mu_r, scale, part);
  sum_kernel<<<1, 1024, 0, s>>>(d->nt, part, out);
  e = cudaGetLastError();
  count_launch(2);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_surface_flux");
}

extern "C" int sucem_ntff(const sucem_space* sp, int dtype, const void* x, double k0, int ndir,
                          const double* theta, const double* phi, double* out, void* stream) {
  using namespace sucem;
  DeviceSpace* d = sp ? sp->s.dev : nullptr;
  if (!d) return fail("space is not on a device", SUCEM_ERR_STATE);
  if (d->nd > 20) return fail("supported for basis orders 1 and 2 only", SUCEM_ERR_ARG);
  if (dtype != SUCEM_C64 && dtype != SUCEM_C128) return fail("dtype must be complex", SUCEM_ERR_ARG);
  if (!(k0 > 0)) return fail("k0 must be positive", SUCEM_ERR_ARG);
  if (ndir < 0) return fail("negative direction count", SUCEM_ERR_ARG);
  if (ndir == 0) return SUCEM_OK;
  if (!x || !theta || !phi || !out) return fail("null argument", SUCEM_ERR_ARG);
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaError_t e = load_face_tables(dev);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_ntff tables");
  if (!d->ext_facets) {
    // exterior facets in (cell, local face) order, and the point scratch
    const Space& hs = sp->s;
    std::vector<int32_t> fl;
    for (int64_t c = 0; c < (int64_t)hs.ext_mask.size(); ++c)
      for (int f = 0; f < 4; ++f)
        if (hs.ext_mask[c] >> f & 1) {
          fl.push_back((int32_t)c);
          fl.push_back(f);
        }
    d->n_ext = (int64_t)fl.size() / 2;
    if (d->n_ext == 0) return fail("the mesh has no exterior facets", SUCEM_ERR_ARG);
    e = cudaMalloc((void**)&d->ext_facets, fl.size() * sizeof(int32_t));
    if (e == cudaSuccess)
      e = cudaMemcpy(d->ext_facets, fl.data(), fl.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
      e = cudaMalloc((void**)&d->ntff_pts, (size_t)d->n_ext * kFaceQ * 16 * sizeof(double));
    if (e != cudaSuccess) {
      if (d->ext_facets) cudaFree(d->ext_facets);
      d->ext_facets = nullptr;
      return cuda_fail(e, "sucem_ntff allocation");
    }
  }
  const double z0 = 3.141592653589793 * 4e-7 * 299792458.0;
  const double inv = 1.0 / (k0 * z0);
  const int threads = 128;
  const unsigned blocks = (unsigned)((d->n_ext + threads - 1) / threads);
  if (d->nd == 6 && dtype == SUCEM_C128)
    ntff_points_kernel<6, double2><<<blocks, threads, 0, s>>>(
        d->n_ext, d->ext_facets, d->cells, d->xyz, d->cell_dofs, (const double2*)x, inv, d->ntff_pts);
  else if (d->nd == 6)
    ntff_points_kernel<6, float2><<<blocks, threads, 0, s>>>(
        d->n_ext, d->ext_facets, d->cells, d->xyz, d->cell_dofs, (const float2*)x, inv, d->ntff_pts);
  else if (dtype == SUCEM_C128)
    ntff_points_kernel<20, double2><<<blocks, threads, 0, s>>>(
        d->n_ext, d->ext_facets, d->cells, d->xyz, d->cell_dofs, (const double2*)x, inv, d->ntff_pts);
  else
    ntff_points_kernel<20, float2><<<blocks, threads, 0, s>>>(
        d->n_ext, d->ext_facets, d->cells, d->xyz, d->cell_dofs, (const float2*)x, inv, d->ntff_pts);
  ntff_dir_kernel<<<ndir, 256, 0, s>>>(d->n_ext * kFaceQ, d->ntff_pts, theta, phi, k0, z0, out);
  e = cudaGetLastError();
  count_launch(2);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_ntff");
}
