// Variational post-processing on the GPU: the EM functional of
// CalcEMFunctional (sucemfem/PostProcessing/PostProcessing.py:62-173),
//   I = int_marked  curl E . curl g / mu_r - k0^2 eps_r E . g  dx
// (bilinear, no conjugation), evaluated element by element from the
// reference tensors (no global matrix), and the interpolation of plane-wave
// testing functions onto the boundary DOFs (SurfaceInterpolant,
// sucemfem/Interpolation/Interpolation.py:26-82, with the
// TransformTestingExpression of sucemfem/PostProcessing/
// variational_ntff.py:31-66): DOF = t . f(p) for the dual functional
// (point p, tangent t) of each boundary DOF.
#include <cuda_runtime.h>

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

// dual functional of every boundary DOF (in boundary_dofs order): the
// reference point and tangent of the local DOF in the first cell holding
// it, mapped by that cell: p = x0 + J p_hat, t = J t_hat (6 doubles each)
void boundary_dual(const Space& hs, std::vector<double>& pt) {
  const int nd = hs.ndof_cell;
  if (hs.order > 2) {
    pt.clear();
    return;
  }
  const double(*dual)[6] = hs.order == 1 ? DUAL1 : DUAL2;
  std::vector<int64_t> owner(hs.n, -1);
  for (int64_t i = 0; i < hs.nt * nd; ++i)
    if (owner[hs.cell_dofs[i]] < 0) owner[hs.cell_dofs[i]] = i;
  pt.assign(hs.boundary_dofs.size() * 6, 0.0);
  for (size_t k = 0; k < hs.boundary_dofs.size(); ++k) {
    const int64_t o = owner[hs.boundary_dofs[k]];
    const int64_t c = o / nd;
    const int a = (int)(o % nd);
    const int32_t* cv = &hs.cells[c * 4];
    const double* x0 = &hs.coords[3 * (int64_t)cv[0]];
    for (int r = 0; r < 3; ++r) {
      double pr = x0[r], tr = 0;
      for (int i = 0; i < 3; ++i) {
        const double Jri = hs.coords[3 * (int64_t)cv[i + 1] + r] - x0[r];
        pr += Jri * dual[a][i];
        tr += Jri * dual[a][3 + i];
      }
      pt[6 * k + r] = pr;
      pt[6 * k + 3 + r] = tr;
    }
  }
}

namespace {

// one thread per cell: g_c^T (S_c / mu - k0^2 eps T_c) E_c, with
//   S_c = sum_m (J^T J)_m / |det J| KC[m],  T_c = sum_m |det J| (J^-1 J^-T)_m KM[m]
// over the metric entries m = 00, 11, 22, 01, 02, 12
template <int ND>
__global__ void em_functional_kernel(int64_t nt, const int4* __restrict__ cells,
                                     const double* __restrict__ xyz,
                                     const int32_t* __restrict__ cell_dofs,
                                     const double* __restrict__ kc, const double* __restrict__ km,
                                     const double* __restrict__ eps,
                                     const double* __restrict__ mu_inv,
                                     const uint8_t* __restrict__ mask,
                                     const double2* __restrict__ E, const double2* __restrict__ g,
                                     double k0sq, double2* __restrict__ part) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nt) return;
  if (mask && !mask[c]) {
    part[c] = make_double2(0.0, 0.0);
    return;
  }
  const int4 v = cells[c];
  const int vv[4] = {v.x, v.y, v.z, v.w};
  double J[3][3];
  for (int i = 0; i < 3; ++i)
    for (int r = 0; r < 3; ++r) J[r][i] = xyz[3 * (int64_t)vv[i + 1] + r] - xyz[3 * (int64_t)vv[0] + r];
  const double m00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const double m01 = J[1][0] * J[2][2] - J[1][2] * J[2][0];
  const double m02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const double det = J[0][0] * m00 - J[0][1] * m01 + J[0][2] * m02;
  const double id = 1.0 / det;
  double Ji[3][3];
  Ji[0][0] = m00 * id;
  Ji[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) * id;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  Ji[1][0] = -m01 * id;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  Ji[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) * id;
  Ji[2][0] = m02 * id;
  Ji[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) * id;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  const double ad = fabs(det);
  const int P[6] = {0, 1, 2, 0, 0, 1}, Q[6] = {0, 1, 2, 1, 2, 2};
  const double sm = mu_inv ? mu_inv[c] : 1.0, se = eps ? eps[c] : 1.0;
  double ws[6], wt[6];
  for (int m = 0; m < 6; ++m) {
    double gs = 0, gt = 0;
    for (int r = 0; r < 3; ++r) {
      gs += J[r][P[m]] * J[r][Q[m]];
      gt += Ji[P[m]][r] * Ji[Q[m]][r];
    }
    ws[m] = gs / ad * sm;
    wt[m] = -k0sq * gt * ad * se;
  }
  double2 e[ND], gg[ND];
  for (int a = 0; a < ND; ++a) {
    const int32_t dof = cell_dofs[c * ND + a];
    e[a] = E[dof];
    gg[a] = g[dof];
  }
  double sr = 0, si = 0;
  for (int a = 0; a < ND; ++a) {
    double hr = 0, hi = 0;  // (W E)_a
    for (int b = 0; b < ND; ++b) {
      double w = 0;
      for (int m = 0; m < 6; ++m)
        w += ws[m] * kc[(m * ND + a) * ND + b] + wt[m] * km[(m * ND + a) * ND + b];
      hr += w * e[b].x;
      hi += w * e[b].y;
    }
    sr += gg[a].x * hr - gg[a].y * hi;
    si += gg[a].x * hi + gg[a].y * hr;
  }
  part[c] = make_double2(sr, si);
}

// one block: out = sum of part[0:n) in a fixed order
__global__ void __launch_bounds__(1024) csum_kernel(int64_t n, const double2* __restrict__ part,
                                                    double2* __restrict__ out) {
  __shared__ double rr[1024], ri[1024];
  double a = 0, b = 0;
  for (int64_t i = threadIdx.x; i < n; i += 1024) {
    a += part[i].x;
    b += part[i].y;
  }
  rr[threadIdx.x] = a;
  ri[threadIdx.x] = b;
  __syncthreads();
  for (int h = 512; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      rr[threadIdx.x] += rr[threadIdx.x + h];
      ri[threadIdx.x] += ri[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = make_double2(rr[0], ri[0]);
}

// one thread per (boundary DOF, wave): g[w*n + dof] = j (t . cf_w) e^{j k0 rhat_w . p}
__global__ void plane_wave_kernel(int64_t nb, int64_t n, int npw,
                                  const int32_t* __restrict__ bdofs, const double* __restrict__ pt,
                                  const double* __restrict__ rhat, const double* __restrict__ cf,
                                  double k0, double2* __restrict__ g) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb * npw) return;
  const int w = (int)(i / nb);
  const int64_t b = i % nb;
  const double* p = pt + 6 * b;
  const double* r = rhat + 3 * w;
  const double* f = cf + 3 * w;
  const double amp = p[3] * f[0] + p[4] * f[1] + p[5] * f[2];
  double s, co;
  sincos(k0 * (r[0] * p[0] + r[1] * p[1] + r[2] * p[2]), &s, &co);
  g[(int64_t)w * n + bdofs[b]] = make_double2(-amp * s, amp * co);
}

}  // namespace
}  // namespace sucem

extern "C" int sucem_boundary_edge_cells(const sucem_space* sp, uint8_t* mask) {
  using namespace sucem;
  if (!sp || !mask) return fail("null argument", SUCEM_ERR_ARG);
  const Space& s = sp->s;
  // edges of the exterior facets, then every cell holding one of them
  std::vector<uint8_t> bedge(s.ne, 0);
  for (int64_t c = 0; c < s.nt; ++c)
    for (int f = 0; f < 4; ++f) {
      if (!(s.ext_mask[c] >> f & 1)) continue;
      for (int le = 0; le < 6; ++le) {
        // local edge le lies on face f unless it touches vertex f
        if (kEdgeVerts[le][0] != f && kEdgeVerts[le][1] != f) bedge[s.cell_edges[c * 6 + le]] = 1;
      }
    }
  for (int64_t c = 0; c < s.nt; ++c) {
    uint8_t m = 0;
    for (int le = 0; le < 6; ++le) m |= bedge[s.cell_edges[c * 6 + le]];
    mask[c] = m;
  }
  return SUCEM_OK;
}

extern "C" int sucem_em_functional(const sucem_space* sp, const double* E, const double* g,
                                   double k0, const double* eps_r, const double* mu_r_inv,
                                   const uint8_t* cell_mask, double* part, double* out,
                                   void* stream) {
  using namespace sucem;
  const DeviceSpace* d = sp ? sp->s.dev : nullptr;
  if (!d) return fail("space is not on a device", SUCEM_ERR_STATE);
  if (d->nd > 20) return fail("supported for basis orders 1 and 2 only", SUCEM_ERR_ARG);
  if (!E || !g || !part || !out) return fail("null argument", SUCEM_ERR_ARG);
  cudaStream_t s = (cudaStream_t)stream;
  const int threads = 128;
  const unsigned blocks = (unsigned)((d->nt + threads - 1) / threads);
  if (d->nd == 6)
    em_functional_kernel<6><<<blocks, threads, 0, s>>>(
        d->nt, d->cells, d->xyz, d->cell_dofs, d->kc_d, d->km_d, eps_r, mu_r_inv, cell_mask,
        (const double2*)E, (const double2*)g, k0 * k0, (double2*)part);
  else
    em_functional_kernel<20><<<blocks, threads, 0, s>>>(
        d->nt, d->cells, d->xyz, d->cell_dofs, d->kc_d, d->km_d, eps_r, mu_r_inv, cell_mask,
        (const double2*)E, (const double2*)g, k0 * k0, (double2*)part);
  csum_kernel<<<1, 1024, 0, s>>>(d->nt, (const double2*)part, (double2*)out);
  cudaError_t e = cudaGetLastError();
  count_launch(2);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_em_functional");
}

extern "C" int sucem_plane_wave_dofs(const sucem_space* sp, int npw, const double* rhat,
                                     const double* cf, double k0, double* g, void* stream) {
  using namespace sucem;
  DeviceSpace* d = sp ? sp->s.dev : nullptr;
  if (!d) return fail("space is not on a device", SUCEM_ERR_STATE);
  if (d->nd > 20) return fail("supported for basis orders 1 and 2 only", SUCEM_ERR_ARG);
  if (npw < 0) return fail("negative wave count", SUCEM_ERR_ARG);
  if (npw == 0 || d->n_boundary == 0) return SUCEM_OK;
  if (!rhat || !cf || !g) return fail("null argument", SUCEM_ERR_ARG);
  cudaStream_t s = (cudaStream_t)stream;
  if (!d->bdof_pt) {
    std::vector<double> pt;
    boundary_dual(sp->s, pt);
    cudaError_t e = cudaMalloc((void**)&d->bdof_pt, pt.size() * sizeof(double));
    if (e == cudaSuccess)
      e = cudaMemcpy(d->bdof_pt, pt.data(), pt.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      if (d->bdof_pt) cudaFree(d->bdof_pt);
      d->bdof_pt = nullptr;
      return cuda_fail(e, "sucem_plane_wave_dofs tables");
    }
  }
  const int64_t total = d->n_boundary * (int64_t)npw;
  const int threads = 256;
  plane_wave_kernel<<<(unsigned)((total + threads - 1) / threads), threads, 0, s>>>(
      d->n_boundary, d->n, npw, d->boundary_dofs, d->bdof_pt, rhat, cf, k0, (double2*)g);
  cudaError_t e = cudaGetLastError();
  count_launch(1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_plane_wave_dofs");
}
