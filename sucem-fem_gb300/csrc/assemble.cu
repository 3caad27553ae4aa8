// Row-gather assembly of the N1curl curl-curl (S), mass (T) and first-order
// ABC (B) matrices, the GPU replacement of dolfin.assemble for the forms of
// sucemfem/Forms.py:71-85 and sucemfem/BoundaryConditions/ABC.py:56-57.
// Orders 3 and 4 (45 and 84 DOFs per cell) use assemble_cells_kernel below
// instead of the row kernel.
//
// Two kernels (orders 1-2):
//  1. cell_geometry_kernel (one thread per cell) writes the cell's 12 metric
//     coefficients (6 for S, 6 for T, already scaled by 1/mu_r, eps_r) and,
//     for cells with exterior facets, 3 tangential coefficients per facet.
//  2. assemble_rows_kernel: one warp owns one mesh entity (an edge, or for
//     order 2 also a face) and therefore the dofs_per_entity CSR rows that
//     share its column list.  Lanes map to the columns of the incident
//     cells (order 2: one cell per step; order 1: five), contract the cell
//     coefficients with the reference tensors held in shared memory for
//     the entity's rows, and add the values into shared-memory row
//     accumulators at the precomputed column slots.  Each CSR value is then
//     written exactly once with coalesced stores: no zero-fill pass, no
//     atomics and a fixed summation order (bit-reproducible run to run).
//
// Element formulas (affine tet, J = [x1-x0 | x2-x0 | x3-x0], covariant
// Piola N = J^-T N_hat):
//   T_e[a][b] = eps   |det J|    sum_pq (J^-1 J^-T)_pq KM[a][b][p][q]
//   S_e[a][b] = 1/mu  / |det J|  sum_pq (J^T J)_pq    KC[a][b][p][q]
//   B_e[a][b] = sum_{exterior f} (|b|^2 KT_f0 - (a.b) KT_f1 + |a|^2 KT_f2)[a][b] / |a x b|
// with the symmetric 3x3 metrics stored as their 6 unique entries, a, b the
// physical edge vectors of face f and KT_f the tangential reference tensors
// ((n x u).(n x v) = tangential part of u.v; the tangential projector of the
// face pulled back by J^-1 is [a^ b^] G^-1 [a^ b^]^T with G the Gram matrix
// of a, b, so no normal vector and no cancellation is needed).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

#include "device.h"

namespace sucem {
void count_launch(int k);

namespace {

constexpr int kWarps = 8;  // warps per block of the row kernel

template <typename Real>
struct Cplx;
template <>
struct Cplx<float> {
  using T = float2;
};
template <>
struct Cplx<double> {
  using T = double2;
};

template <typename Real>
__device__ __forceinline__ void cell_jacobian(const float4* hi, const float4* lo, const double* xyz,
                                              int4 v, Real J[3][3]);

template <>
__device__ __forceinline__ void cell_jacobian<float>(const float4* hi, const float4* lo,
                                                     const double*, int4 v, float J[3][3]) {
  // hi/lo split coordinates: the differences keep ~FP64 accuracy in FP32 math
  const float4 h0 = __ldg(&hi[v.x]), l0 = __ldg(&lo[v.x]);
  const int vv[3] = {v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float4 h = __ldg(&hi[vv[i]]), l = __ldg(&lo[vv[i]]);
    J[0][i] = (h.x - h0.x) + (l.x - l0.x);
    J[1][i] = (h.y - h0.y) + (l.y - l0.y);
    J[2][i] = (h.z - h0.z) + (l.z - l0.z);
  }
}

template <>
__device__ __forceinline__ void cell_jacobian<double>(const float4*, const float4*,
                                                      const double* xyz, int4 v, double J[3][3]) {
  const double* x0 = xyz + 3 * (int64_t)v.x;
  const int vv[3] = {v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double* xi = xyz + 3 * (int64_t)vv[i];
#pragma unroll
    for (int r = 0; r < 3; ++r) J[r][i] = __ldg(xi + r) - __ldg(x0 + r);
  }
}

__device__ __forceinline__ int sym_p(int m) { return m < 3 ? m : (m == 5 ? 1 : 0); }
__device__ __forceinline__ int sym_q(int m) { return m < 3 ? m : (m == 3 ? 1 : 2); }

// ---- kernel 1: per-cell coefficients ----
template <typename Real>
__global__ void cell_geometry_kernel(int64_t nt, const int4* __restrict__ cells,
                                     const float4* __restrict__ hi, const float4* __restrict__ lo,
                                     const double* __restrict__ xyz,
                                     const uint8_t* __restrict__ ext_mask,
                                     const int32_t* __restrict__ bidx,
                                     const Real* __restrict__ eps_r,
                                     const Real* __restrict__ mu_inv, Real* __restrict__ g,
                                     Real* __restrict__ h, bool with_b) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nt) return;
  const int4 v = __ldg(&cells[c]);
  Real J[3][3];
  cell_jacobian<Real>(hi, lo, xyz, v, J);
  const Real m00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const Real m01 = J[1][0] * J[2][2] - J[1][2] * J[2][0];
  const Real m02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const Real det = J[0][0] * m00 - J[0][1] * m01 + J[0][2] * m02;
  const Real adet = fabs(det);
  const Real id = Real(1) / det;
  Real Ji[3][3];
  Ji[0][0] = m00 * id;
  Ji[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]) * id;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
  Ji[1][0] = -m01 * id;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
  Ji[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]) * id;
  Ji[2][0] = m02 * id;
  Ji[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]) * id;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
  const Real sS = (mu_inv ? __ldg(mu_inv + c) : Real(1)) / adet;
  const Real sT = (eps_r ? __ldg(eps_r + c) : Real(1)) * adet;
  Real out[12];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const int pp = sym_p(m), qq = sym_q(m);
    out[m] = (J[0][pp] * J[0][qq] + J[1][pp] * J[1][qq] + J[2][pp] * J[2][qq]) * sS;
    out[6 + m] = (Ji[pp][0] * Ji[qq][0] + Ji[pp][1] * Ji[qq][1] + Ji[pp][2] * Ji[qq][2]) * sT;
  }
#pragma unroll
  for (int m = 0; m < 12; ++m) g[c * 12 + m] = out[m];
  if (!with_b) return;
  const int hb = __ldg(&bidx[c]);
  if (hb < 0) return;
  const int mask = __ldg(&ext_mask[c]);
#pragma unroll
  for (int f = 0; f < 4; ++f) {
    Real c0 = 0, c1 = 0, c2 = 0;
    if (mask >> f & 1) {
      Real a[3], b[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        if (f == 0) {
          a[r] = J[r][1] - J[r][0];
          b[r] = J[r][2] - J[r][0];
        } else if (f == 1) {
          a[r] = J[r][1];
          b[r] = J[r][2];
        } else if (f == 2) {
          a[r] = J[r][0];
          b[r] = J[r][2];
        } else {
          a[r] = J[r][0];
          b[r] = J[r][1];
        }
      }
      const Real cx = a[1] * b[2] - a[2] * b[1];
      const Real cy = a[2] * b[0] - a[0] * b[2];
      const Real cz = a[0] * b[1] - a[1] * b[0];
      const Real ita = Real(1) / sqrt(cx * cx + cy * cy + cz * cz);
      c0 = (b[0] * b[0] + b[1] * b[1] + b[2] * b[2]) * ita;
      c1 = -(a[0] * b[0] + a[1] * b[1] + a[2] * b[2]) * ita;
      c2 = (a[0] * a[0] + a[1] * a[1] + a[2] * a[2]) * ita;
    }
    h[(int64_t)hb * 12 + f * 3 + 0] = c0;
    h[(int64_t)hb * 12 + f * 3 + 1] = c1;
    h[(int64_t)hb * 12 + f * 3 + 2] = c2;
  }
}

struct RowPtrs {
  const int32_t* ent_ptr;
  const int32_t* inc_cell;
  const uint8_t* inc_rec;
  const int32_t* indptr;
  const int32_t* bidx;
  const uint8_t* ext_mask;
  int64_t n_ent;
  int max_row;
};

template <typename Real>
__device__ __forceinline__ void load12(const Real* p, Real out[12]);
template <>
__device__ __forceinline__ void load12<float>(const float* p, float out[12]) {
  const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float4 t = q[i];
    out[4 * i] = t.x;
    out[4 * i + 1] = t.y;
    out[4 * i + 2] = t.z;
    out[4 * i + 3] = t.w;
  }
}
template <>
__device__ __forceinline__ void load12<double>(const double* p, double out[12]) {
  const double2* q = reinterpret_cast<const double2*>(p);
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const double2 t = q[i];
    out[2 * i] = t.x;
    out[2 * i + 1] = t.y;
  }
}

// ORDER: 1 or 2.  WITH_B: accumulate the ABC matrix.  MODE 0: separate
// real outputs; MODE 1: fused complex A = S - k0^2 T + j k0 B.
//
// One warp per entity.  Its lanes take ICH = 32/ND incident cells at a time
// (order 2: one cell, lane b = cell column b; order 1: five cells x six
// columns).  Each lane contracts the cell's coefficients with the reference
// tensors for the entity's rows and adds the result into its accumulator
// copy (copy = which of the ICH cells of the step it handles).  Within a copy
// the columns of one cell are distinct slots, so plain shared-memory
// read-add-write is race free; copies are summed in a fixed order when the
// rows are written, so results are bit-reproducible.
template <int ORDER, typename Real, bool WITH_B, int MODE>
__global__ void __launch_bounds__(kWarps * 32)
    assemble_rows_kernel(RowPtrs p, const Real* __restrict__ gcell, const Real* __restrict__ hcell,
                         const Real* __restrict__ kab, const Real* __restrict__ kt, Real* S,
                         Real* T, Real* B, typename Cplx<Real>::T* A, Real k0) {
  constexpr int ND = ORDER == 1 ? 6 : 20;
  constexpr int DPE = ORDER == 1 ? 1 : 2;
  constexpr int REC = ORDER == 1 ? 8 : 24;
  constexpr int ICH = 32 / ND;                 // incident cells per sweep step
  // accumulated matrices: mode 0 -> S, T (, B); mode 1 -> Re A, Im A
  constexpr int NMAT = MODE == 1 ? 2 : (WITH_B ? 3 : 2);
  constexpr int KSZ = ND * ND * 12;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  Real* sK = reinterpret_cast<Real*>(smem_raw);  // [a][b][12]: KC[0..5], KM[0..5]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int R = p.max_row;
  const int copy_len = DPE * NMAT * R;        // one copy: [DPE][NMAT][R]
  const int acc_len = ICH * copy_len;
  Real* acc = sK + KSZ + warp * acc_len;      // [ICH][DPE][NMAT][R]

  for (int i = threadIdx.x; i < KSZ; i += blockDim.x) sK[i] = kab[i];
  for (int i = lane; i < acc_len; i += 32) acc[i] = Real(0);
  __syncthreads();
  const Real k0sq = k0 * k0;
  const int sub = lane / ND, b = lane - sub * ND;   // cell of the step, cell column
  const bool lane_on = sub < ICH;
  Real* my_copy = acc + (lane_on ? sub : 0) * copy_len;

  const int64_t nwarps = (int64_t)gridDim.x * kWarps;
  for (int64_t e = (int64_t)blockIdx.x * kWarps + warp; e < p.n_ent; e += nwarps) {
    const int i0 = __ldg(&p.ent_ptr[e]), i1 = __ldg(&p.ent_ptr[e + 1]);
    const int64_t r0 = (int64_t)DPE * e;
    const int off = __ldg(&p.indptr[r0]);
    const int L = __ldg(&p.indptr[r0 + 1]) - off;
    for (int k0i = i0; k0i < i1; k0i += ICH) {
      const int inc = k0i + sub;
      if (lane_on && inc < i1) {
        const int c = __ldg(&p.inc_cell[inc]);
        const uint8_t* rec = p.inc_rec + (int64_t)inc * REC;
        const int le = __ldg(rec);
        const int slot = __ldg(rec + 1 + b);
        Real g[12];
        load12<Real>(gcell + (int64_t)c * 12, g);
        int hb = -1, mask = 0;
        if (WITH_B) {
          hb = __ldg(&p.bidx[c]);
          if (hb >= 0) mask = __ldg(&p.ext_mask[c]);
        }
#pragma unroll
        for (int j = 0; j < DPE; ++j) {
          const int a = DPE * le + j;
          Real kk[12];
          load12<Real>(sK + (a * ND + b) * 12, kk);
          Real s = 0, tm = 0;
#pragma unroll
          for (int m = 0; m < 6; ++m) {
            s = fma(g[m], kk[m], s);
            tm = fma(g[6 + m], kk[6 + m], tm);
          }
          Real* ar = my_copy + j * NMAT * R + slot;
          if (MODE == 1) {
            ar[0] += s - k0sq * tm;
          } else {
            ar[0] += s;
            ar[R] += tm;
          }
          if (WITH_B && hb >= 0) {
            const Real* hh = hcell + (int64_t)hb * 12;
            Real bv = 0;
#pragma unroll
            for (int f = 0; f < 4; ++f) {
              if (!(mask >> f & 1)) continue;
#pragma unroll
              for (int m = 0; m < 3; ++m)
                bv = fma(__ldg(&hh[f * 3 + m]), __ldg(&kt[((f * 3 + m) * ND + a) * ND + b]), bv);
            }
            if (MODE == 1)
              ar[R] += k0 * bv;
            else
              ar[2 * R] += bv;
          }
        }
      }
      __syncwarp();
    }
    // ---- write the entity's rows (sum of the copies), reset the copies ----
#pragma unroll
    for (int j = 0; j < DPE; ++j) {
      const int64_t base = (int64_t)off + (int64_t)j * L;
      for (int col = lane; col < L; col += 32) {
        Real v[NMAT];
#pragma unroll
        for (int q = 0; q < NMAT; ++q) v[q] = 0;
#pragma unroll
        for (int cc = 0; cc < ICH; ++cc) {
          Real* ar = acc + cc * copy_len + j * NMAT * R + col;
#pragma unroll
          for (int q = 0; q < NMAT; ++q) {
            v[q] += ar[q * R];
            ar[q * R] = 0;
          }
        }
        if (MODE == 0) {
          if (S) S[base + col] = v[0];
          if (T) T[base + col] = v[1];
          if (WITH_B && B) B[base + col] = v[NMAT - 1];
        } else {
          typename Cplx<Real>::T z;
          z.x = v[0];
          z.y = v[1];
          A[base + col] = z;
        }
      }
    }
    __syncwarp();
  }
}

// Orders 3-4: one block per cell (grid-stride over the cells), a thread per
// local entry (a, b): the cell's 12 coefficients contracted with the
// reference tensors ([a][b][12], read through L1/L2) and added atomically
// at the entry's precomputed CSR position (the outputs are zeroed first).
// Every value is exact up to the order in which the cells' contributions
// are summed, which is not fixed.
template <int ND, typename Real, bool WITH_B, int MODE>
__global__ void __launch_bounds__(256)
    assemble_cells_kernel(int64_t nt, const int32_t* __restrict__ pos,
                          const int32_t* __restrict__ bidx, const uint8_t* __restrict__ ext_mask,
                          const Real* __restrict__ gcell, const Real* __restrict__ hcell,
                          const Real* __restrict__ kab, const Real* __restrict__ kt, Real* S,
                          Real* T, Real* B, typename Cplx<Real>::T* A, Real k0) {
  constexpr int NN = ND * ND;
  const Real k0sq = k0 * k0;
  for (int64_t c = blockIdx.x; c < nt; c += gridDim.x) {
    Real g[12];
    load12<Real>(gcell + c * 12, g);
    int hb = -1, mask = 0;
    if (WITH_B) {
      hb = __ldg(&bidx[c]);
      if (hb >= 0) mask = __ldg(&ext_mask[c]);
    }
    const int32_t* pc = pos + c * NN;
    for (int e = threadIdx.x; e < NN; e += blockDim.x) {
      Real kk[12];
      load12<Real>(kab + (int64_t)e * 12, kk);
      Real sv = 0, tm = 0;
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        sv = fma(g[m], kk[m], sv);
        tm = fma(g[6 + m], kk[6 + m], tm);
      }
      Real bv = 0;
      if (WITH_B && hb >= 0) {
        const Real* hh = hcell + (int64_t)hb * 12;
#pragma unroll
        for (int f = 0; f < 4; ++f) {
          if (!(mask >> f & 1)) continue;
#pragma unroll
          for (int m = 0; m < 3; ++m)
            bv = fma(__ldg(&hh[f * 3 + m]), __ldg(&kt[(f * 3 + m) * NN + e]), bv);
        }
      }
      const int64_t q = __ldg(&pc[e]);
      if (MODE == 1) {
        atomicAdd(&A[q].x, sv - k0sq * tm);
        if (WITH_B && bv != 0) atomicAdd(&A[q].y, k0 * bv);
      } else {
        if (S) atomicAdd(&S[q], sv);
        if (T) atomicAdd(&T[q], tm);
        if (WITH_B && B && bv != 0) atomicAdd(&B[q], bv);
      }
    }
  }
}

template <typename Real>
cudaError_t ensure_scratch(DeviceSpace& d, Real** g, Real** h) {
  void** pg = sizeof(Real) == 4 ? (void**)&d.g_f : (void**)&d.g_d;
  void** ph = sizeof(Real) == 4 ? (void**)&d.h_f : (void**)&d.h_d;
  if (!*pg) {
    cudaError_t e = cudaMalloc(pg, sizeof(Real) * 12 * std::max<int64_t>(d.nt, 1));
    if (e != cudaSuccess) return e;
  }
  if (!*ph) {
    cudaError_t e = cudaMalloc(ph, sizeof(Real) * 12 * std::max<int64_t>(d.nb, 1));
    if (e != cudaSuccess) return e;
  }
  *g = (Real*)*pg;
  *h = (Real*)*ph;
  return cudaSuccess;
}

template <int ORDER, typename Real, bool WITH_B, int MODE>
cudaError_t launch_t(DeviceSpace& d, const AssembleArgs& a, cudaStream_t stream) {
  constexpr int ND = ORDER == 1 ? 6 : 20;
  constexpr int DPE = ORDER == 1 ? 1 : 2;
  constexpr int NMAT = MODE == 1 ? 2 : (WITH_B ? 3 : 2);
  constexpr int ICH = 32 / ND;
  Real *g = nullptr, *h = nullptr;
  cudaError_t err = ensure_scratch<Real>(d, &g, &h);
  if (err != cudaSuccess) return err;
  {
    const int threads = 256;
    const int64_t blocks = (d.nt + threads - 1) / threads;
    cell_geometry_kernel<Real><<<(unsigned)blocks, threads, 0, stream>>>(
        d.nt, d.cells, d.xyz_hi, d.xyz_lo, d.xyz, d.ext_mask, d.bidx, (const Real*)a.eps_r,
        (const Real*)a.mu_r_inv, g, h, WITH_B);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  }
  RowPtrs p;
  p.ent_ptr = d.ent_ptr;
  p.inc_cell = d.inc_cell;
  p.inc_rec = d.inc_rec;
  p.indptr = d.indptr;
  p.bidx = d.bidx;
  p.ext_mask = d.ext_mask;
  p.n_ent = d.n_ent;
  p.max_row = d.max_row;
  const size_t smem =
      sizeof(Real) * ((size_t)ND * ND * 12 + (size_t)kWarps * ICH * DPE * NMAT * d.max_row);
  auto kern = assemble_rows_kernel<ORDER, Real, WITH_B, MODE>;
  err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarps * 32, smem);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int64_t want = (d.n_ent + kWarps - 1) / kWarps;
  int64_t grid = std::min<int64_t>(want, (int64_t)nsm * per_sm);
  if (grid < 1) grid = 1;
  const Real* kab = sizeof(Real) == 4 ? (const Real*)d.kab_f : (const Real*)d.kab_d;
  const Real* kt = sizeof(Real) == 4 ? (const Real*)d.kt_f : (const Real*)d.kt_d;
  kern<<<(unsigned)grid, kWarps * 32, smem, stream>>>(p, g, h, kab, kt, (Real*)a.S, (Real*)a.T,
                                                      (Real*)a.B, (typename Cplx<Real>::T*)a.A,
                                                      (Real)a.k0);
  count_launch(2);
  return cudaGetLastError();
}

template <int ND, typename Real, bool WITH_B, int MODE>
cudaError_t launch_cells_t(DeviceSpace& d, const AssembleArgs& a, cudaStream_t stream) {
  Real *g = nullptr, *h = nullptr;
  cudaError_t err = ensure_scratch<Real>(d, &g, &h);
  if (err != cudaSuccess) return err;
  {
    const int threads = 256;
    const int64_t blocks = (d.nt + threads - 1) / threads;
    cell_geometry_kernel<Real><<<(unsigned)blocks, threads, 0, stream>>>(
        d.nt, d.cells, d.xyz_hi, d.xyz_lo, d.xyz, d.ext_mask, d.bidx, (const Real*)a.eps_r,
        (const Real*)a.mu_r_inv, g, h, WITH_B);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  }
  const size_t vbytes = (size_t)d.nnz * sizeof(Real);
  if (MODE == 1) {
    err = cudaMemsetAsync(a.A, 0, 2 * vbytes, stream);
  } else {
    if (a.S) err = cudaMemsetAsync(a.S, 0, vbytes, stream);
    if (err == cudaSuccess && a.T) err = cudaMemsetAsync(a.T, 0, vbytes, stream);
    if (err == cudaSuccess && WITH_B && a.B) err = cudaMemsetAsync(a.B, 0, vbytes, stream);
  }
  if (err != cudaSuccess) return err;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(d.nt, (int64_t)nsm * 8));
  const Real* kab = sizeof(Real) == 4 ? (const Real*)d.kab_f : (const Real*)d.kab_d;
  const Real* kt = sizeof(Real) == 4 ? (const Real*)d.kt_f : (const Real*)d.kt_d;
  assemble_cells_kernel<ND, Real, WITH_B, MODE><<<(unsigned)grid, 256, 0, stream>>>(
      d.nt, d.cell_pos, d.bidx, d.ext_mask, g, h, kab, kt, (Real*)a.S, (Real*)a.T, (Real*)a.B,
      (typename Cplx<Real>::T*)a.A, (Real)a.k0);
  count_launch(2);
  return cudaGetLastError();
}

template <int ND, typename Real>
cudaError_t dispatch_cells(DeviceSpace& d, const AssembleArgs& a, cudaStream_t stream) {
  if (!d.cell_pos) return cudaErrorInvalidValue;
  if (a.mode == 1) return launch_cells_t<ND, Real, true, 1>(d, a, stream);
  if (a.B) return launch_cells_t<ND, Real, true, 0>(d, a, stream);
  return launch_cells_t<ND, Real, false, 0>(d, a, stream);
}

template <int ORDER, typename Real>
cudaError_t dispatch_mode(DeviceSpace& d, const AssembleArgs& a, cudaStream_t stream) {
  if (a.mode == 1) return launch_t<ORDER, Real, true, 1>(d, a, stream);
  if (a.B) return launch_t<ORDER, Real, true, 0>(d, a, stream);
  return launch_t<ORDER, Real, false, 0>(d, a, stream);
}

}  // namespace

cudaError_t launch_assemble(DeviceSpace& d, const AssembleArgs& a, cudaStream_t stream) {
  if (d.order == 3)
    return a.real_bytes == 4 ? dispatch_cells<45, float>(d, a, stream)
                             : dispatch_cells<45, double>(d, a, stream);
  if (d.order == 4)
    return a.real_bytes == 4 ? dispatch_cells<84, float>(d, a, stream)
                             : dispatch_cells<84, double>(d, a, stream);
  if (d.order == 1) {
    return a.real_bytes == 4 ? dispatch_mode<1, float>(d, a, stream)
                             : dispatch_mode<1, double>(d, a, stream);
  }
  return a.real_bytes == 4 ? dispatch_mode<2, float>(d, a, stream)
                           : dispatch_mode<2, double>(d, a, stream);
}

}  // namespace sucem
