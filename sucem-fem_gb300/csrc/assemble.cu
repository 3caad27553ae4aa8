// Assembly of the N1curl curl-curl (S), mass (T) and first-order ABC (B)
// matrices, the GPU replacement of dolfin.assemble for the forms of
// sucemfem/Forms.py:71-85 and sucemfem/BoundaryConditions/ABC.py:56-57.
// Orders 3 and 4 (45 and 84 DOFs per cell) use assemble_cell_entries_kernel
// below instead of the entity kernel.
//
// Two kernels (orders 1-2):
//  1. cell_geometry_kernel (one thread per cell) writes the cell's 12 metric
//     coefficients (6 for S, 6 for T, already scaled by 1/mu_r, eps_r, and
//     for the fused complex matrix the T part by -k0^2) and, for cells with
//     exterior facets, 3 tangential coefficients per facet (scaled by k0 for
//     the fused matrix).
//  2. assemble_entities_kernel: one lane owns one mesh entity (an edge, or
//     for order 2 also a face) and therefore the dofs_per_entity CSR rows
//     that share its column list; a warp takes 32 of them (see the kernel).
//     Each CSR value is written exactly once with coalesced stores: no
//     zero-fill pass, no atomics and a fixed summation order
//     (bit-reproducible run to run).
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
#include "n1curl_contract.h"

namespace sucem {
void count_launch(int k);

namespace {

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

// programmatic dependent launch between the two kernels of an order-1/2
// assembly: the geometry kernel lets the entity kernel start launching at
// once; the entity kernel clears its accumulators and loads its schedule
// before it waits (griddepcontrol.wait) for the coefficients.  No-ops for a
// plain launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }

// ---- kernel 1: per-cell coefficients ----
// Computed in Real, written as Out (the assembly's precision).  HILO (Real
// double, Out float): each coefficient is written as float hi + lo, the 12
// hi values then the 12 rests (24 per cell, and likewise the 12 tangential
// coefficients of a boundary cell), for the compensated single-precision
// contraction.
template <typename Real, typename Out, bool HILO>
__global__ void cell_geometry_kernel(int64_t nt, const int4* __restrict__ cells,
                                     const float4* __restrict__ hi, const float4* __restrict__ lo,
                                     const double* __restrict__ xyz,
                                     const uint8_t* __restrict__ ext_mask,
                                     const int32_t* __restrict__ bidx,
                                     const Out* __restrict__ eps_r,
                                     const Out* __restrict__ mu_inv, Out* __restrict__ g,
                                     Out* __restrict__ h, bool with_b, Real tscale,
                                     Real hscale) {
  pdl_trigger();
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
  const Real sS = (mu_inv ? Real(__ldg(mu_inv + c)) : Real(1)) / adet;
  const Real sT = (eps_r ? Real(__ldg(eps_r + c)) : Real(1)) * adet * tscale;
  Real out[12];
#pragma unroll
  for (int m = 0; m < 6; ++m) {
    const int pp = sym_p(m), qq = sym_q(m);
    out[m] = (J[0][pp] * J[0][qq] + J[1][pp] * J[1][qq] + J[2][pp] * J[2][qq]) * sS;
    out[6 + m] = (Ji[pp][0] * Ji[qq][0] + Ji[pp][1] * Ji[qq][1] + Ji[pp][2] * Ji[qq][2]) * sT;
  }
  if (HILO) {
#pragma unroll
    for (int m = 0; m < 12; ++m) {
      const Out gh = Out(out[m]);
      g[c * 24 + m] = gh;
      g[c * 24 + 12 + m] = Out(out[m] - Real(gh));
    }
  } else {
#pragma unroll
    for (int m = 0; m < 12; ++m) g[c * 12 + m] = Out(out[m]);
  }
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
      const Real ita = hscale / sqrt(cx * cx + cy * cy + cz * cz);
      c0 = (b[0] * b[0] + b[1] * b[1] + b[2] * b[2]) * ita;
      c1 = -(a[0] * b[0] + a[1] * b[1] + a[2] * b[2]) * ita;
      c2 = (a[0] * a[0] + a[1] * a[1] + a[2] * a[2]) * ita;
    }
    const Real cc[3] = {c0, c1, c2};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const Out hv = Out(cc[q]);
      if (HILO) {
        h[(int64_t)hb * 24 + f * 3 + q] = hv;
        h[(int64_t)hb * 24 + 12 + f * 3 + q] = Out(cc[q] - Real(hv));
      } else {
        h[(int64_t)hb * 12 + f * 3 + q] = hv;
      }
    }
  }
}

template <typename Real>
__device__ __forceinline__ void load12(const Real* p, Real out[12]);
template <>
__device__ __forceinline__ void load12<float>(const float* p, float out[12]) {
  const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float4 t = __ldg(q + i);
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
    const double2 t = __ldg(q + i);
    out[2 * i] = t.x;
    out[2 * i + 1] = t.y;
  }
}

// ---- entity-per-lane assembly of orders 1-2 ----
//
// One warp owns a task of 32 entities (edges, or faces of order 2), one per
// lane; a lane's entity owns DPE consecutive CSR rows (DPE = order) that
// share one column list of L slots.  The task's steps (see Space: local
// entity index le major, trip[le] steps each) give every lane one incident
// cell per step.  For step le the element-matrix rows of local entity le
// are the same straight-line code on every lane (contract::Rows, reference
// constants inlined), so the contraction needs no table loads; the lane
// adds its DPE x ND values (and, in separate mode, S and T apart) to its
// own accumulator row in shared memory at the column slots of the step
// record.  A lane's accumulator is private: no atomics and a fixed
// summation order (bit-reproducible).  The slots of one slot index of all
// lanes sit in distinct banks (per-lane stride odd in units of the slot
// vector).  At the end the warp writes each lane's rows in turn with
// coalesced stores: every CSR value is written once and nothing is
// zero-filled first.
//
// Boundary entities (on an exterior facet) are in tasks of their own that
// also accumulate the ABC matrix B from the cells' tangential coefficients
// h and the face tables KT (read through L1: the cells concerned are few).
// The host packs consecutive tasks into blocks (up to a per-variant number)
// within a shared-memory budget: a task's accumulators take 32 x P slot
// vectors, P its longest row, so blocks of short rows hold more tasks.

template <int V, typename Real>
struct SlotVec;  // V values of one slot, moved with the widest shared access
template <>
struct SlotVec<1, float> {
  static __device__ __forceinline__ void add(float* p, const float* v) { p[0] += v[0]; }
};
template <>
struct SlotVec<2, float> {
  static __device__ __forceinline__ void add(float* p, const float* v) {
    float2 t = *reinterpret_cast<float2*>(p);
    t.x += v[0];
    t.y += v[1];
    *reinterpret_cast<float2*>(p) = t;
  }
};
template <>
struct SlotVec<4, float> {
  static __device__ __forceinline__ void add(float* p, const float* v) {
    float4 t = *reinterpret_cast<float4*>(p);
    t.x += v[0];
    t.y += v[1];
    t.z += v[2];
    t.w += v[3];
    *reinterpret_cast<float4*>(p) = t;
  }
};
template <>
struct SlotVec<1, double> {
  static __device__ __forceinline__ void add(double* p, const double* v) { p[0] += v[0]; }
};
template <>
struct SlotVec<2, double> {
  static __device__ __forceinline__ void add(double* p, const double* v) {
    double2 t = *reinterpret_cast<double2*>(p);
    t.x += v[0];
    t.y += v[1];
    *reinterpret_cast<double2*>(p) = t;
  }
};
template <>
struct SlotVec<4, double> {
  static __device__ __forceinline__ void add(double* p, const double* v) {
    SlotVec<2, double>::add(p, v);
    SlotVec<2, double>::add(p + 2, v + 2);
  }
};

struct EntArgs {
  const int32_t* task_ent;     // n_tasks*32
  const int4* task_meta;       // n_tasks
  const uint32_t* step_words;  // step blocks
  const int32_t* indptr;       // n+1
  const int32_t* bidx;         // nt
  const uint8_t* ext_mask;     // nt
  const int32_t* blocks;       // first task of each block (+ end)
  int64_t n_int_blocks;        // blocks [0, n_int_blocks) take interior tasks
};

// Block shape per kernel variant (EntCfg::BLOCK_WARPS / BLOCK_BYTES): the
// fused single-precision kernel (< 85 registers) takes blocks of 8 warps
// within 68 KB, so three blocks share an SM's shared memory and registers,
// i.e. 24 warps where the rows are short enough (order-2 faces: 8 tasks of
// 33 slots) and fewer for the longest rows (3 tasks of 75 slots); the
// register-heavy variants (double precision, compensated separate
// matrices) take blocks of 2 warps within 40 KB.

template <int ORDER, typename Real, int MODE>
struct EntCfg {
  static constexpr int ND = ORDER == 1 ? 6 : 20;
  static constexpr int DPE = ORDER;
  static constexpr int PL = (ND + 3) / 4;              // slot planes of a step block
  static constexpr int WPS = (1 + PL) * 32;            // words per step block
  static constexpr int NMAT = MODE == 1 ? 1 : 2;       // fused A, or S and T
  // separate single-precision matrices: compensated throughout (element
  // sums by contract::Dot2, accumulation in double-float hi + lo slots)
  static constexpr bool DD = MODE == 0 && sizeof(Real) == 4;
  // values per slot of the main accumulator: [S0 S1 T0 T1] / [A0 A1]; DD:
  // per row j [S hi, S lo, T hi, T lo]
  static constexpr int V = DD ? 4 * DPE : DPE * NMAT;
  static constexpr int VB = DD ? 2 * DPE : DPE;        // B / Im accumulator (DD: hi, lo per row)
  // cell coefficients per cell: 12, or 24 (float hi + lo) when DD
  static constexpr int NG = DD ? 24 : 12;
  static constexpr bool LIGHT = MODE == 1 && sizeof(Real) == 4;
  static constexpr int BLOCK_WARPS = LIGHT ? 8 : 2;          // most tasks per block
  static constexpr int BLOCK_BYTES = (LIGHT ? 68 : 40) << 10;  // shared memory budget
};

// (hi, lo) += (xh, xl): TwoSum of the leading parts, rests added to lo
__device__ __forceinline__ void dd_add(float& hi, float& lo, float xh, float xl) {
  const float s = __fadd_rn(hi, xh);
  const float z = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, z)), __fsub_rn(xh, z));
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(xl, e));
}

struct StepRec {
  int cell;
  uint32_t sl[5];
};

template <int PL>
__device__ __forceinline__ StepRec load_step(const uint32_t* blk, int lane) {
  StepRec r;
  r.cell = (int)__ldg(blk + lane);
#pragma unroll
  for (int q = 0; q < PL; ++q) r.sl[q] = __ldg(blk + 32 * (1 + q) + lane);
  return r;
}

template <typename Real, int NG>
__device__ __forceinline__ void load_g(const Real* gcell, int c, Real* g) {
  if (c >= 0) {
#pragma unroll
    for (int q = 0; q < NG / 12; ++q) load12<Real>(gcell + (int64_t)c * NG + 12 * q, g + 12 * q);
  } else {
#pragma unroll
    for (int m = 0; m < NG; ++m) g[m] = Real(0);
  }
}

__device__ __forceinline__ int slot_of(const StepRec& r, int b) {
  return (int)((r.sl[b >> 2] >> (8 * (b & 3))) & 0xffu);
}

// does exterior local face f of a cell contain the lane's entity (local
// index LE, edge or face)?
template <bool FACE, int LE>
__device__ __forceinline__ bool face_holds(int f) {
  if (FACE) return f == LE;
  constexpr int ev0 = LE == 0 ? 2 : LE == 1 ? 1 : LE == 2 ? 1 : 0;
  constexpr int ev1 = LE == 0 ? 3 : LE == 1 ? 3 : LE == 2 ? 2 : LE == 3 ? 3 : LE == 4 ? 2 : 1;
  return f != ev0 && f != ev1;
}

// one step of local entity LE: contract, then add into the lane's rows
template <int ORDER, typename Real, int MODE, bool FACE, int LE, bool BND>
__device__ __forceinline__ void ent_step(const StepRec& r, const Real* g, Real* acc, Real* bacc,
                                         const EntArgs& p, const Real* __restrict__ hcell,
                                         const Real* __restrict__ kt,
                                         const float* __restrict__ kt_lo) {
  using C = EntCfg<ORDER, Real, MODE>;
  constexpr int ND = C::ND, DPE = C::DPE;
  if constexpr (C::DD) {
    // compensated: each element sum (unrounded s + c) straight into its
    // double-float slot
    if (r.cell >= 0)
      contract::Rows<ORDER, FACE, LE>::split(
          g, [&](int j, int b, const contract::Dot2<float>& sd, const contract::Dot2<float>& td) {
            float4* q = reinterpret_cast<float4*>(acc + (slot_of(r, b) * DPE + j) * 4);
            float4 t = *q;
            dd_add(t.x, t.y, sd.s, sd.c);
            dd_add(t.z, t.w, td.s, td.c);
            *q = t;
          });
  } else {
    Real v[ND][C::V];
#pragma unroll
    for (int b = 0; b < ND; ++b)
#pragma unroll
      for (int q = 0; q < C::V; ++q) v[b][q] = Real(0);
    if constexpr (MODE == 1) {
      contract::Rows<ORDER, FACE, LE>::fused(g, [&](int j, int b, Real x) { v[b][j] = x; });
    } else {
      contract::Rows<ORDER, FACE, LE>::split(
          g, [&](int j, int b, const contract::Dot2<Real>& sd, const contract::Dot2<Real>& td) {
            v[b][j] = sd.s;
            v[b][DPE + j] = td.s;
          });
    }
    if (r.cell < 0) return;
#pragma unroll
    for (int b = 0; b < ND; ++b) SlotVec<C::V, Real>::add(acc + slot_of(r, b) * C::V, v[b]);
  }
  if (!BND || r.cell < 0) return;
  const int hb = __ldg(&p.bidx[r.cell]);
  if (hb < 0) return;
  const int mask = __ldg(&p.ext_mask[r.cell]);
  const Real* hh = hcell + (int64_t)hb * (C::DD ? 24 : 12);
  for (int f = 0; f < 4; ++f) {
    if (!(mask >> f & 1) || !face_holds<FACE, LE>(f)) continue;
#pragma unroll
    for (int j = 0; j < DPE; ++j) {
      const int a = FACE ? 12 + 2 * LE + j : DPE * LE + j;
      const int64_t k0i = ((int64_t)(f * 3 + 0) * ND + a) * ND;
      const int64_t k1i = ((int64_t)(f * 3 + 1) * ND + a) * ND;
      const int64_t k2i = ((int64_t)(f * 3 + 2) * ND + a) * ND;
#pragma unroll 4
      for (int b = 0; b < ND; ++b) {
        if constexpr (C::DD) {
          // h as hi + lo pairs (stride 12), KT as float hi + lo
          contract::Dot2<float> bd;
          bd.add(hh, 3 * f, 0.0, __ldg(kt + k0i + b), __ldg(kt_lo + k0i + b));
          bd.add(hh, 3 * f + 1, 0.0, __ldg(kt + k1i + b), __ldg(kt_lo + k1i + b));
          bd.add(hh, 3 * f + 2, 0.0, __ldg(kt + k2i + b), __ldg(kt_lo + k2i + b));
          float* q = bacc + (slot_of(r, b) * DPE + j) * 2;
          dd_add(q[0], q[1], bd.s, bd.c);
        } else {
          const Real bv = fma(__ldg(hh + 3 * f + 2), __ldg(kt + k2i + b),
                              fma(__ldg(hh + 3 * f + 1), __ldg(kt + k1i + b),
                                  __ldg(hh + 3 * f) * __ldg(kt + k0i + b)));
          bacc[slot_of(r, b) * C::VB + j] += bv;
        }
      }
    }
  }
}

// the steps of local entities LE .. NLE-1; the next step's record and cell
// coefficients and the record after it are loaded one step ahead
template <int ORDER, typename Real, int MODE, bool FACE, int LE, int NLE, bool BND>
__device__ __forceinline__ void ent_steps(const uint8_t* trip, int& s, int nsteps,
                                          const uint32_t* blk0, int lane, StepRec& r0, Real* g0,
                                          StepRec& r1, Real* acc, Real* bacc, const EntArgs& p,
                                          const Real* __restrict__ gcell,
                                          const Real* __restrict__ hcell,
                                          const Real* __restrict__ kt,
                                          const float* __restrict__ kt_lo) {
  if constexpr (LE < NLE) {
    using C = EntCfg<ORDER, Real, MODE>;
    for (int t = 0; t < trip[LE]; ++t, ++s) {
      Real g1[C::NG];
      load_g<Real, C::NG>(gcell, s + 1 < nsteps ? r1.cell : -1, g1);
      StepRec r2;
      r2.cell = -1;
      if (s + 2 < nsteps) r2 = load_step<C::PL>(blk0 + (int64_t)(s + 2) * C::WPS, lane);
      ent_step<ORDER, Real, MODE, FACE, LE, BND>(r0, g0, acc, bacc, p, hcell, kt, kt_lo);
      r0 = r1;
#pragma unroll
      for (int m = 0; m < C::NG; ++m) g0[m] = g1[m];
      r1 = r2;
    }
    ent_steps<ORDER, Real, MODE, FACE, LE + 1, NLE, BND>(trip, s, nsteps, blk0, lane, r0, g0, r1,
                                                        acc, bacc, p, gcell, hcell, kt, kt_lo);
  }
}

template <int ORDER, typename Real, int MODE, bool BND>
__device__ __forceinline__ void ent_task(int64_t task, const int4 meta, int P, int lane,
                                         Real* acc, Real* bacc, const EntArgs& p,
                                         const Real* __restrict__ gcell,
                                         const Real* __restrict__ hcell,
                                         const Real* __restrict__ kt,
                                         const float* __restrict__ kt_lo, Real* S, Real* T,
                                         Real* B, typename Cplx<Real>::T* A) {
  using C = EntCfg<ORDER, Real, MODE>;
  constexpr int DPE = C::DPE;
  // the lane's entity and its rows' CSR offset and length: loaded first so
  // that their latency hides under the steps (the write phase needs them)
  const int my_ent = __ldg(&p.task_ent[task * 32 + lane]);
  int my_off = 0, my_len = 0;
  if (my_ent >= 0) {
    my_off = __ldg(&p.indptr[(int64_t)DPE * my_ent]);
    my_len = __ldg(&p.indptr[(int64_t)DPE * my_ent + 1]) - my_off;
  }
  // clear the warp's accumulators (each lane's P slots; 16-byte stores, the
  // regions start 16-byte aligned and hold a multiple of 16 bytes)
  {
    float4* a0 = reinterpret_cast<float4*>(acc - (int64_t)lane * P * C::V);
    const int n4 = 32 * P * C::V * (int)sizeof(Real) / 16;
    for (int i = lane; i < n4; i += 32) a0[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (BND) {
      float4* b0 = reinterpret_cast<float4*>(bacc - (int64_t)lane * P * C::VB);
      const int m4 = 32 * P * C::VB * (int)sizeof(Real) / 16;
      for (int i = lane; i < m4; i += 32) b0[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  __syncwarp();
  uint8_t trip[8];
  *reinterpret_cast<int*>(&trip[0]) = meta.y;
  *reinterpret_cast<int*>(&trip[4]) = meta.z;
  int nsteps = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) nsteps += trip[i];
  const uint32_t* blk0 = p.step_words + (int64_t)meta.x * C::WPS;
  StepRec r0, r1;
  r0.cell = r1.cell = -1;
  if (nsteps > 0) r0 = load_step<C::PL>(blk0, lane);
  if (nsteps > 1) r1 = load_step<C::PL>(blk0 + C::WPS, lane);
  pdl_wait();  // the cell coefficients are the geometry kernel's output
  Real g0[C::NG];
  load_g<Real, C::NG>(gcell, r0.cell, g0);
  int s = 0;
  bool done = false;
  if constexpr (ORDER == 2) {
    if (meta.w & 1) {
      ent_steps<ORDER, Real, MODE, true, 0, 4, BND>(trip, s, nsteps, blk0, lane, r0, g0, r1, acc,
                                                    bacc, p, gcell, hcell, kt, kt_lo);
      done = true;
    }
  }
  if (!done)
    ent_steps<ORDER, Real, MODE, false, 0, 6, BND>(trip, s, nsteps, blk0, lane, r0, g0, r1, acc,
                                                   bacc, p, gcell, hcell, kt, kt_lo);
  __syncwarp();
  // write each lane's rows, one entity at a time, coalesced
  const Real* acc0 = acc - (int64_t)lane * P * C::V;
  const Real* bacc0 = BND ? bacc - (int64_t)lane * P * C::VB : nullptr;
  for (int l = 0; l < 32; ++l) {
    const int k = __shfl_sync(0xffffffffu, my_ent, l);
    const int off = __shfl_sync(0xffffffffu, my_off, l);
    const int L = __shfl_sync(0xffffffffu, my_len, l);
    if (k < 0) continue;
    const Real* al = acc0 + (int64_t)l * P * C::V;
    const Real* bl = BND ? bacc0 + (int64_t)l * P * C::VB : nullptr;
    // lanes over the slots, both rows of a slot per lane: row j of the
    // entity starts at off + j * L
    for (int sl = lane; sl < L; sl += 32)
#pragma unroll
    for (int j = 0; j < DPE; ++j) {
      const int idx = j * L + sl;
      if constexpr (C::DD) {
        const float* q = al + (sl * DPE + j) * 4;
        if (S) S[(int64_t)off + idx] = __fadd_rn(q[0], q[1]);
        if (T) T[(int64_t)off + idx] = __fadd_rn(q[2], q[3]);
        if (B) B[(int64_t)off + idx] = BND ? __fadd_rn(bl[(sl * DPE + j) * 2], bl[(sl * DPE + j) * 2 + 1]) : 0.f;
      } else {
        const Real bval = BND ? bl[sl * C::VB + j] : Real(0);
        if (MODE == 1) {
          typename Cplx<Real>::T z;
          z.x = al[sl * C::V + j];
          z.y = bval;
          A[(int64_t)off + idx] = z;
        } else {
          if (S) S[(int64_t)off + idx] = al[sl * C::V + j];
          if (T) T[(int64_t)off + idx] = al[sl * C::V + DPE + j];
          if (B) B[(int64_t)off + idx] = bval;
        }
      }
    }
  }
}

template <int ORDER, typename Real, int MODE, bool WITH_B>
__global__ void __launch_bounds__(EntCfg<ORDER, Real, MODE>::BLOCK_WARPS * 32)
    assemble_entities_kernel(EntArgs p, const Real* __restrict__ gcell,
                             const Real* __restrict__ hcell, const Real* __restrict__ kt,
                             const float* __restrict__ kt_lo, Real* S, Real* T, Real* B,
                             typename Cplx<Real>::T* A) {
  using C = EntCfg<ORDER, Real, MODE>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Real* sm = reinterpret_cast<Real*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t t0 = __ldg(&p.blocks[blockIdx.x]), t1 = __ldg(&p.blocks[blockIdx.x + 1]);
  const int64_t task = t0 + warp;
  if (task >= t1) return;
  const bool bnd = WITH_B && (int64_t)blockIdx.x >= p.n_int_blocks;
  const int words = bnd ? C::V + C::VB : C::V;  // per slot and lane
  // this warp's accumulators follow those of the block's earlier tasks
  int64_t off = 0;
  for (int i = 0; i < warp; ++i) off += 32LL * ((__ldg(&p.task_meta[t0 + i].w) >> 8) & 0xffff) * words;
  const int4 meta = __ldg(&p.task_meta[task]);
  const int P = (meta.w >> 8) & 0xffff;
  Real* base = sm + off;
  if constexpr (WITH_B) {
    if (bnd) {
      ent_task<ORDER, Real, MODE, true>(task, meta, P, lane, base + (int64_t)lane * P * C::V,
                                        base + 32LL * P * C::V + (int64_t)lane * P * C::VB, p,
                                        gcell, hcell, kt, kt_lo, S, T, B, A);
      return;
    }
  }
  ent_task<ORDER, Real, MODE, false>(task, meta, P, lane, base + (int64_t)lane * P * C::V,
                                     nullptr, p, gcell, hcell, kt, kt_lo, S, T, B, A);
}

// Orders 3-4: a thread per CSR entry (grid-stride; thread t takes entry
// perm[t], each row's entries ordered by list length so that a warp's lanes
// walk lists of similar length), gathering the cell entries listed for it
// (ascending cell order): each is the cell's 12
// coefficients contracted with the reference tensors ([a][b][12], read
// through L1/L2), plus the tangential term of the cell's exterior faces.
// S, T and B are summed separately in that fixed order and every output
// entry is written once (no atomics, no zeroing pass), so the matrices are
// the same bits on every run.
template <int ND, typename Real, bool WITH_B, int MODE>
__global__ void __launch_bounds__(256)
    assemble_cell_entries_kernel(int64_t nnz, const int32_t* __restrict__ perm,
                                 const int32_t* __restrict__ ptr,
                                 const int32_t* __restrict__ src,
                                 const int32_t* __restrict__ bidx,
                                 const uint8_t* __restrict__ ext_mask,
                                 const Real* __restrict__ gcell, const Real* __restrict__ hcell,
                                 const Real* __restrict__ kab, const Real* __restrict__ kt,
                                 Real* S, Real* T, Real* B, typename Cplx<Real>::T* A, Real k0) {
  constexpr int NN = ND * ND;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nnz;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = __ldg(&perm[t]);
    Real sv = 0, tm = 0, bv = 0;
    const int j1 = __ldg(&ptr[q + 1]);
    for (int j = __ldg(&ptr[q]); j < j1; ++j) {
      const int sc = __ldg(&src[j]);
      const int c = sc / NN, e = sc - c * NN;
      Real g[12], kk[12];
      load12<Real>(gcell + (int64_t)c * 12, g);
      load12<Real>(kab + (int64_t)e * 12, kk);
      Real sc_s = 0, sc_t = 0;
#pragma unroll
      for (int m = 0; m < 6; ++m) {
        sc_s = fma(g[m], kk[m], sc_s);
        sc_t = fma(g[6 + m], kk[6 + m], sc_t);
      }
      sv += sc_s;
      tm += sc_t;
      if (WITH_B) {
        const int hb = __ldg(&bidx[c]);
        if (hb >= 0) {
          const int mask = __ldg(&ext_mask[c]);
          const Real* hh = hcell + (int64_t)hb * 12;
          Real sc_b = 0;
#pragma unroll
          for (int f = 0; f < 4; ++f) {
            if (!(mask >> f & 1)) continue;
#pragma unroll
            for (int m = 0; m < 3; ++m)
              sc_b = fma(__ldg(&hh[f * 3 + m]), __ldg(&kt[(f * 3 + m) * NN + e]), sc_b);
          }
          bv += sc_b;
        }
      }
    }
    if (MODE == 1) {
      typename Cplx<Real>::T v;
      v.x = sv - k0 * k0 * tm;
      v.y = k0 * bv;
      A[q] = v;
    } else {
      if (S) S[q] = sv;
      if (T) T[q] = tm;
      if (WITH_B && B) B[q] = bv;
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

// Blocks of the entity kernel for a slot size (bytes per accumulator slot
// and lane: interior tasks, boundary tasks): consecutive tasks share a block
// while their accumulators fit `budget` bytes and at most `warps` tasks;
// interior tasks first, then (with B) boundary tasks.  Built once per layout
// and kept with the space.
cudaError_t task_blocks(DeviceSpace& d, int slot_int, int slot_bnd, bool with_b, int warps,
                        int budget, const DeviceSpace::TaskBlocks** out) {
  const int key = slot_int | (slot_bnd << 8) | ((with_b ? 1 : 0) << 16) | (warps << 17) |
                  ((budget >> 10) << 21);
  auto it = d.task_blocks.find(key);
  if (it != d.task_blocks.end()) {
    *out = &it->second;
    return cudaSuccess;
  }
  DeviceSpace::TaskBlocks tb;
  std::vector<int32_t> first;
  const int64_t n_int = with_b ? d.n_tasks_interior : d.n_tasks;
  auto pack = [&](int64_t lo, int64_t hi, int slot) {
    int64_t t = lo;
    while (t < hi) {
      first.push_back((int32_t)t);
      int64_t used = 0;
      int n = 0;
      while (t < hi && n < warps) {
        const int64_t need = 32LL * d.task_P[t] * slot;
        if (n > 0 && used + need > budget) break;
        used += need;
        ++n;
        ++t;
      }
      tb.smem = std::max(tb.smem, used);
    }
  };
  pack(0, n_int, slot_int);
  tb.n_int = (int64_t)first.size();
  if (with_b) pack(n_int, d.n_tasks, slot_bnd);
  tb.n_bnd = (int64_t)first.size() - tb.n_int;
  first.push_back((int32_t)d.n_tasks);
  cudaError_t e = cudaMalloc((void**)&tb.first, first.size() * sizeof(int32_t));
  if (e == cudaSuccess)
    e = cudaMemcpy(tb.first, first.data(), first.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (tb.first) cudaFree(tb.first);
    return e;
  }
  *out = &(d.task_blocks[key] = tb);
  return cudaSuccess;
}

template <int ORDER, typename Real, bool WITH_B, int MODE>
cudaError_t launch_t(DeviceSpace& d, const AssembleArgs& a, cudaStream_t stream) {
  using C = EntCfg<ORDER, Real, MODE>;
  if (!d.task_meta || d.n_tasks == 0) return cudaErrorInvalidValue;
  Real *g = nullptr, *h = nullptr;
  cudaError_t err = ensure_scratch<Real>(d, &g, &h);
  if (err != cudaSuccess) return err;
  {
    const int threads = 256;
    const int64_t blocks = (d.nt + threads - 1) / threads;
    if constexpr (C::NG == 24) {
      // separate single-precision matrices: coefficients from FP64
      // geometry as float hi + lo (see contract::Dot2)
      if (!d.g2_f) {
        err = cudaMalloc((void**)&d.g2_f, sizeof(float) * 24 * std::max<int64_t>(d.nt, 1));
        if (err != cudaSuccess) return err;
      }
      if (!d.h2_f) {
        err = cudaMalloc((void**)&d.h2_f, sizeof(float) * 24 * std::max<int64_t>(d.nb, 1));
        if (err != cudaSuccess) return err;
      }
      g = reinterpret_cast<Real*>(d.g2_f);
      h = reinterpret_cast<Real*>(d.h2_f);
      cell_geometry_kernel<double, float, true><<<(unsigned)blocks, threads, 0, stream>>>(
          d.nt, d.cells, d.xyz_hi, d.xyz_lo, d.xyz, d.ext_mask, d.bidx, (const float*)a.eps_r,
          (const float*)a.mu_r_inv, (float*)g, (float*)h, WITH_B, 1.0, 1.0);
    } else {
      const Real tscale = MODE == 1 ? Real(-a.k0 * a.k0) : Real(1);
      const Real hscale = MODE == 1 ? Real(a.k0) : Real(1);
      cell_geometry_kernel<Real, Real, false><<<(unsigned)blocks, threads, 0, stream>>>(
          d.nt, d.cells, d.xyz_hi, d.xyz_lo, d.xyz, d.ext_mask, d.bidx, (const Real*)a.eps_r,
          (const Real*)a.mu_r_inv, g, h, WITH_B, tscale, hscale);
    }
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  }
  const DeviceSpace::TaskBlocks* tb = nullptr;
  err = task_blocks(d, (int)(C::V * sizeof(Real)), (int)((C::V + C::VB) * sizeof(Real)), WITH_B,
                    C::BLOCK_WARPS, C::BLOCK_BYTES, &tb);
  if (err != cudaSuccess) return err;
  EntArgs p;
  p.task_ent = d.task_ent;
  p.task_meta = d.task_meta;
  p.step_words = d.step_words;
  p.indptr = d.indptr;
  p.bidx = d.bidx;
  p.ext_mask = d.ext_mask;
  p.blocks = tb->first;
  p.n_int_blocks = tb->n_int;
  const int64_t grid = tb->n_int + tb->n_bnd;
  if (grid < 1) return cudaSuccess;
  if (tb->smem > (227 << 10)) return cudaErrorInvalidConfiguration;  // rows too long
  auto kern = assemble_entities_kernel<ORDER, Real, MODE, WITH_B>;
  err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tb->smem);
  if (err != cudaSuccess) return err;
  const Real* kt = sizeof(Real) == 4 ? (const Real*)d.kt_f : (const Real*)d.kt_d;
  {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(C::BLOCK_WARPS * 32);
    cfg.dynamicSmemBytes = (size_t)tb->smem;
    cfg.stream = stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    err = cudaLaunchKernelEx(&cfg, kern, p, (const Real*)g, (const Real*)h, kt,
                             (const float*)d.kt_lo_f, (Real*)a.S, (Real*)a.T, (Real*)a.B,
                             (typename Cplx<Real>::T*)a.A);
    if (err != cudaSuccess) return err;
  }
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
    cell_geometry_kernel<Real, Real, false><<<(unsigned)blocks, threads, 0, stream>>>(
        d.nt, d.cells, d.xyz_hi, d.xyz_lo, d.xyz, d.ext_mask, d.bidx, (const Real*)a.eps_r,
        (const Real*)a.mu_r_inv, g, h, WITH_B, Real(1), Real(1));
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  }
  const int64_t grid = std::max<int64_t>(1, (d.nnz + 255) / 256);
  const Real* kab = sizeof(Real) == 4 ? (const Real*)d.kab_f : (const Real*)d.kab_d;
  const Real* kt = sizeof(Real) == 4 ? (const Real*)d.kt_f : (const Real*)d.kt_d;
  assemble_cell_entries_kernel<ND, Real, WITH_B, MODE><<<(unsigned)grid, 256, 0, stream>>>(
      d.nnz, d.entry_perm, d.entry_ptr, d.entry_src, d.bidx, d.ext_mask, g, h, kab, kt, (Real*)a.S, (Real*)a.T,
      (Real*)a.B, (typename Cplx<Real>::T*)a.A, (Real)a.k0);
  count_launch(2);
  return cudaGetLastError();
}

template <int ND, typename Real>
cudaError_t dispatch_cells(DeviceSpace& d, const AssembleArgs& a, cudaStream_t stream) {
  if (!d.entry_ptr || !d.entry_src || !d.entry_perm) return cudaErrorInvalidValue;
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
