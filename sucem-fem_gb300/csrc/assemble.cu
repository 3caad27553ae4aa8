// Row-gather assembly of the N1curl curl-curl (S), mass (T) and first-order
// ABC (B) matrices, the GPU replacement of dolfin.assemble for the forms of
// sucemfem/Forms.py:71-85 and sucemfem/BoundaryConditions/ABC.py:56-57.
//
// One warp owns one mesh entity (an edge, or for order 2 also a face) and
// therefore the dofs_per_entity CSR rows that share its column list.  It
// walks the entity's incident cells in cell order, recomputes each cell's
// affine geometry (one lane per incident cell), contracts it with the
// reference tensors, accumulates the rows in shared memory and writes every
// CSR value exactly once with coalesced stores.  No atomics, no zero-fill
// pass and a fixed summation order (bit-reproducible run to run).
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

#include <cstdio>

#include "device.h"

namespace sucem {

namespace {

constexpr int kWarps = 8;  // warps per block

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

struct KernelPtrs {
  const int4* cells;
  const float4* xyz_hi;
  const float4* xyz_lo;
  const double* xyz;
  const uint8_t* ext_mask;
  const int32_t* ent_ptr;
  const int32_t* inc_cell;
  const uint8_t* inc_rec;
  const int32_t* indptr;
  int64_t n_ent;
  int max_row;
};

template <typename Real>
__device__ __forceinline__ void cell_jacobian(const KernelPtrs& p, int4 v, Real J[3][3]);

template <>
__device__ __forceinline__ void cell_jacobian<float>(const KernelPtrs& p, int4 v, float J[3][3]) {
  // hi/lo split coordinates: the differences keep ~FP64 accuracy in FP32 math
  const float4 h0 = __ldg(&p.xyz_hi[v.x]), l0 = __ldg(&p.xyz_lo[v.x]);
  const int vv[3] = {v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float4 h = __ldg(&p.xyz_hi[vv[i]]), l = __ldg(&p.xyz_lo[vv[i]]);
    J[0][i] = (h.x - h0.x) + (l.x - l0.x);
    J[1][i] = (h.y - h0.y) + (l.y - l0.y);
    J[2][i] = (h.z - h0.z) + (l.z - l0.z);
  }
}

template <>
__device__ __forceinline__ void cell_jacobian<double>(const KernelPtrs& p, int4 v, double J[3][3]) {
  const double* x0 = p.xyz + 3 * (int64_t)v.x;
  const int vv[3] = {v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double* xi = p.xyz + 3 * (int64_t)vv[i];
#pragma unroll
    for (int r = 0; r < 3; ++r) J[r][i] = __ldg(xi + r) - __ldg(x0 + r);
  }
}

__device__ __forceinline__ int sym_p(int m) { return m < 3 ? m : (m == 5 ? 1 : 0); }
__device__ __forceinline__ int sym_q(int m) { return m < 3 ? m : (m == 3 ? 1 : 2); }

template <typename Real>
__device__ __forceinline__ Real load_coef(const Real* a, int c) {
  return a ? __ldg(a + c) : Real(1);
}

// ORDER: 1 or 2.  WITH_B: accumulate the ABC matrix.  MODE 0: separate
// real outputs; MODE 1: fused complex A = S - k0^2 T + j k0 B.
template <int ORDER, typename Real, bool WITH_B, int MODE>
__global__ void __launch_bounds__(kWarps * 32)
    assemble_rows_kernel(KernelPtrs p, const Real* __restrict__ eps_r,
                         const Real* __restrict__ mu_inv, const Real* __restrict__ kc,
                         const Real* __restrict__ km, const Real* __restrict__ kf, Real* S,
                         Real* T, Real* B, typename Cplx<Real>::T* A, Real k0) {
  constexpr int ND = ORDER == 1 ? 6 : 20;
  constexpr int DPE = ORDER == 1 ? 1 : 2;
  constexpr int REC = ORDER == 1 ? 8 : 24;
  constexpr int NMAT = WITH_B ? 3 : 2;
  constexpr int KSZ = 6 * ND * ND;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  Real* sKC = reinterpret_cast<Real*>(smem_raw);
  Real* sKM = sKC + KSZ;
  Real* warp_base = sKM + KSZ;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int acc_len = DPE * NMAT * p.max_row;
  const int per_warp = 32 * 12 + (WITH_B ? 32 * 12 : 0) + acc_len;
  Real* gbuf = warp_base + warp * per_warp;   // [32][12]
  Real* hbuf = gbuf + 32 * 12;                // [32][4 faces][3] (WITH_B)
  Real* acc = hbuf + (WITH_B ? 32 * 12 : 0);  // [DPE][NMAT][max_row]
  __shared__ int masks[kWarps][32];

  for (int i = threadIdx.x; i < KSZ; i += blockDim.x) {
    sKC[i] = kc[i];
    sKM[i] = km[i];
  }
  for (int i = lane; i < acc_len; i += 32) acc[i] = Real(0);
  __syncthreads();

  const int64_t nwarps = (int64_t)gridDim.x * kWarps;
  for (int64_t e = (int64_t)blockIdx.x * kWarps + warp; e < p.n_ent; e += nwarps) {
    const int i0 = __ldg(&p.ent_ptr[e]), i1 = __ldg(&p.ent_ptr[e + 1]);
    const int64_t r0 = (int64_t)DPE * e;
    const int off = __ldg(&p.indptr[r0]);
    const int L = __ldg(&p.indptr[r0 + 1]) - off;

    for (int c0 = i0; c0 < i1; c0 += 32) {
      const int nk = min(32, i1 - c0);
      // ---- phase 1: geometry of incident cell (one lane per incidence) ----
      if (lane < nk) {
        const int c = __ldg(&p.inc_cell[c0 + lane]);
        const int4 v = __ldg(&p.cells[c]);
        Real J[3][3];
        cell_jacobian<Real>(p, v, J);
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
        const Real sS = load_coef(mu_inv, c) / adet;
        const Real sT = load_coef(eps_r, c) * adet;
        Real* g = gbuf + lane * 12;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
          const int pp = sym_p(m), qq = sym_q(m);
          g[m] = (J[0][pp] * J[0][qq] + J[1][pp] * J[1][qq] + J[2][pp] * J[2][qq]) * sS;
          g[6 + m] = (Ji[pp][0] * Ji[qq][0] + Ji[pp][1] * Ji[qq][1] + Ji[pp][2] * Ji[qq][2]) * sT;
        }
        int mask = 0;
        if (WITH_B) {
          // ABC block of exterior face f from its edge vectors a, b:
          // (|b|^2 KT[f][0] - (a.b) KT[f][1] + |a|^2 KT[f][2]) / |a x b|
          mask = __ldg(&p.ext_mask[c]);
          Real* h = hbuf + lane * 12;
#pragma unroll
          for (int f = 0; f < 4; ++f) {
            if (!(mask >> f & 1)) continue;
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
            h[f * 3 + 0] = (b[0] * b[0] + b[1] * b[1] + b[2] * b[2]) * ita;
            h[f * 3 + 1] = -(a[0] * b[0] + a[1] * b[1] + a[2] * b[2]) * ita;
            h[f * 3 + 2] = (a[0] * a[0] + a[1] * a[1] + a[2] * a[2]) * ita;
          }
        }
        masks[warp][lane] = mask;
      }
      __syncwarp();
      // ---- phase 2: contract and accumulate (lane = local column dof) ----
      for (int k = 0; k < nk; ++k) {
        const uint8_t* rec = p.inc_rec + (int64_t)(c0 + k) * REC;
        const int le = __ldg(rec);
        const Real* g = gbuf + k * 12;
        if (lane < ND) {
          const int slot = __ldg(rec + 1 + lane);
          const int mask = WITH_B ? masks[warp][k] : 0;
#pragma unroll
          for (int j = 0; j < DPE; ++j) {
            const int a = DPE * le + j;
            Real s = 0, t = 0;
#pragma unroll
            for (int m = 0; m < 6; ++m) {
              s += g[m] * sKC[(m * ND + a) * ND + lane];
              t += g[6 + m] * sKM[(m * ND + a) * ND + lane];
            }
            Real* ar = acc + j * NMAT * p.max_row;
            ar[slot] += s;
            ar[p.max_row + slot] += t;
            if (WITH_B && mask) {
              const Real* h = hbuf + k * 12;
              Real bsum = 0;
#pragma unroll
              for (int f = 0; f < 4; ++f) {
                if (!(mask >> f & 1)) continue;
#pragma unroll
                for (int m = 0; m < 3; ++m)
                  bsum += h[f * 3 + m] * __ldg(&kf[((f * 3 + m) * ND + a) * ND + lane]);
              }
              ar[2 * p.max_row + slot] += bsum;
            }
          }
        }
        __syncwarp();
      }
    }
    // ---- phase 3: write the entity's rows, reset the accumulators ----
#pragma unroll
    for (int j = 0; j < DPE; ++j) {
      Real* ar = acc + j * NMAT * p.max_row;
      const int64_t base = (int64_t)off + (int64_t)j * L;
      for (int col = lane; col < L; col += 32) {
        const Real s = ar[col], t = ar[p.max_row + col];
        const Real b = WITH_B ? ar[2 * p.max_row + col] : Real(0);
        if (MODE == 0) {
          if (S) S[base + col] = s;
          if (T) T[base + col] = t;
          if (WITH_B && B) B[base + col] = b;
        } else {
          typename Cplx<Real>::T z;
          z.x = s - k0 * k0 * t;
          z.y = k0 * b;
          A[base + col] = z;
        }
        ar[col] = 0;
        ar[p.max_row + col] = 0;
        if (WITH_B) ar[2 * p.max_row + col] = 0;
      }
    }
    __syncwarp();
  }
}

template <int ORDER, typename Real, bool WITH_B, int MODE>
cudaError_t launch_t(const DeviceSpace& d, const AssembleArgs& a, cudaStream_t stream) {
  constexpr int ND = ORDER == 1 ? 6 : 20;
  constexpr int DPE = ORDER == 1 ? 1 : 2;
  constexpr int NMAT = WITH_B ? 3 : 2;
  KernelPtrs p;
  p.cells = d.cells;
  p.xyz_hi = d.xyz_hi;
  p.xyz_lo = d.xyz_lo;
  p.xyz = d.xyz;
  p.ext_mask = d.ext_mask;
  p.ent_ptr = d.ent_ptr;
  p.inc_cell = d.inc_cell;
  p.inc_rec = d.inc_rec;
  p.indptr = d.indptr;
  p.n_ent = d.n_ent;
  p.max_row = d.max_row;
  const size_t per_warp = 32 * 12 + (WITH_B ? 32 * 12 : 0) + (size_t)DPE * NMAT * d.max_row;
  const size_t smem = sizeof(Real) * (2 * 6 * ND * ND + kWarps * per_warp);
  auto kern = assemble_rows_kernel<ORDER, Real, WITH_B, MODE>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (err != cudaSuccess) return err;
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarps * 32, smem);
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  int64_t want = (d.n_ent + kWarps - 1) / kWarps;
  int64_t grid = std::min<int64_t>(want, (int64_t)nsm * per_sm);
  if (grid < 1) grid = 1;
  const Real* kc = sizeof(Real) == 4 ? (const Real*)d.kc_f : (const Real*)d.kc_d;
  const Real* km = sizeof(Real) == 4 ? (const Real*)d.km_f : (const Real*)d.km_d;
  const Real* kf = sizeof(Real) == 4 ? (const Real*)d.kt_f : (const Real*)d.kt_d;
  kern<<<(unsigned)grid, kWarps * 32, smem, stream>>>(
      p, (const Real*)a.eps_r, (const Real*)a.mu_r_inv, kc, km, kf, (Real*)a.S, (Real*)a.T,
      (Real*)a.B, (typename Cplx<Real>::T*)a.A, (Real)a.k0);
  return cudaGetLastError();
}

template <int ORDER, typename Real>
cudaError_t dispatch_mode(const DeviceSpace& d, const AssembleArgs& a, cudaStream_t stream) {
  if (a.mode == 1) return launch_t<ORDER, Real, true, 1>(d, a, stream);
  if (a.B) return launch_t<ORDER, Real, true, 0>(d, a, stream);
  return launch_t<ORDER, Real, false, 0>(d, a, stream);
}

}  // namespace

cudaError_t launch_assemble(const DeviceSpace& d, const AssembleArgs& a, cudaStream_t stream) {
  if (d.order == 1) {
    return a.real_bytes == 4 ? dispatch_mode<1, float>(d, a, stream)
                             : dispatch_mode<1, double>(d, a, stream);
  }
  return a.real_bytes == 4 ? dispatch_mode<2, float>(d, a, stream)
                           : dispatch_mode<2, double>(d, a, stream);
}

}  // namespace sucem
