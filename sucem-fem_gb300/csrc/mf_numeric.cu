// Numeric multifrontal LU on the GPU (factor and solve), level by level
// over the assembly tree built by mf_symbolic.cpp.  Scalars: float, double,
// complex float (float2), complex double (double2).
//
// Factor: the arena of dense row-major fronts is zeroed, the matrix values
// are scattered into it, then for every tree level (leaves first): the
// children's Schur complements are added into their parents (extend-add,
// one launch per child slot so no two writers meet), and every front of the
// level is partially factorised with a blocked right-looking LU (panel
// width 64, 32 for complex double): diagonal-block LU (one block per front), the two triangular
// panel solves, and the trailing update, a batched register-tiled GEMM.
// Solve: forward (unit-lower L) and backward (U) substitution level by
// level; the off-diagonal block products are spread over many blocks.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <map>
#include <cstdio>
#include <cstring>

#include "../../include/sucem_gb300.h"
#include "mf.h"

#include <type_traits>

namespace sucem {
int fail(const std::string& msg, int code);
int cuda_fail(cudaError_t e, const char* where);
void count_launch(int k);

namespace {


// single precision (real and complex): trailing and panel updates on the
// tensor cores (mf_tc.cuh); double precision keeps the CUDA-core kernels
template <typename S>
constexpr bool kTensorCore = std::is_same<S, float2>::value || std::is_same<S, float>::value;
// algorithmic flops of one multiply-add
template <typename S>
constexpr double kMacFlops = std::is_same<S, float2>::value ? 8.0 : 2.0;

// ---- scalar helpers ----
__device__ __forceinline__ float s_zero(float) { return 0.f; }
__device__ __forceinline__ double s_zero(double) { return 0.0; }
__device__ __forceinline__ float2 s_zero(float2) { return make_float2(0.f, 0.f); }
__device__ __forceinline__ double2 s_zero(double2) { return make_double2(0.0, 0.0); }

__device__ __forceinline__ float s_fms(float c, float a, float b) { return fmaf(-a, b, c); }
__device__ __forceinline__ double s_fms(double c, double a, double b) { return fma(-a, b, c); }
__device__ __forceinline__ float2 s_fms(float2 c, float2 a, float2 b) {
  c.x = fmaf(-a.x, b.x, c.x);
  c.x = fmaf(a.y, b.y, c.x);
  c.y = fmaf(-a.x, b.y, c.y);
  c.y = fmaf(-a.y, b.x, c.y);
  return c;
}
__device__ __forceinline__ double2 s_fms(double2 c, double2 a, double2 b) {
  c.x = fma(-a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(-a.x, b.y, c.y);
  c.y = fma(-a.y, b.x, c.y);
  return c;
}
__device__ __forceinline__ float s_one(float) { return 1.f; }
__device__ __forceinline__ double s_one(double) { return 1.0; }
__device__ __forceinline__ float2 s_one(float2) { return make_float2(1.f, 0.f); }
__device__ __forceinline__ double2 s_one(double2) { return make_double2(1.0, 0.0); }
__device__ __forceinline__ float s_mul(float a, float b) { return a * b; }
__device__ __forceinline__ double s_mul(double a, double b) { return a * b; }
__device__ __forceinline__ float2 s_mul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 s_mul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float s_add(float a, float b) { return a + b; }
__device__ __forceinline__ double s_add(double a, double b) { return a + b; }
__device__ __forceinline__ float2 s_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 s_add(double2 a, double2 b) {
  return make_double2(a.x + b.x, a.y + b.y);
}
__device__ __forceinline__ float s_div(float a, float b) { return a / b; }
__device__ __forceinline__ double s_div(double a, double b) { return a / b; }
__device__ __forceinline__ float2 s_div(float2 a, float2 b) {
  const float d = b.x * b.x + b.y * b.y;
  return make_float2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double2 s_div(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double s_abs(float a) { return fabsf(a); }
__device__ __forceinline__ double s_abs(double a) { return fabs(a); }
__device__ __forceinline__ double s_abs(float2 a) { return hypotf(a.x, a.y); }
__device__ __forceinline__ double s_abs(double2 a) { return hypot(a.x, a.y); }
__device__ __forceinline__ float s_real(float, double v) { return (float)v; }
__device__ __forceinline__ double s_real(double, double v) { return v; }
__device__ __forceinline__ float2 s_real(float2, double v) { return make_float2((float)v, 0.f); }
__device__ __forceinline__ double2 s_real(double2, double v) { return make_double2(v, 0.0); }
// squared magnitude in the working precision and the reciprocal of a pivot
// from it: 1/p = conj(p) / |p|^2, with a correctly rounded 1/|p|^2
__device__ __forceinline__ float s_mag2s(float v) { return v * v; }
__device__ __forceinline__ double s_mag2s(double v) { return v * v; }
__device__ __forceinline__ float s_mag2s(float2 v) { return fmaf(v.x, v.x, v.y * v.y); }
__device__ __forceinline__ double s_mag2s(double2 v) { return fma(v.x, v.x, v.y * v.y); }
__device__ __forceinline__ float s_recip(float v, float) { return __frcp_rn(v); }
__device__ __forceinline__ double s_recip(double v, double) { return 1.0 / v; }
__device__ __forceinline__ float2 s_recip(float2 v, float m2) {
  const float r = __frcp_rn(m2);
  return make_float2(v.x * r, -v.y * r);
}
__device__ __forceinline__ double2 s_recip(double2 v, double m2) {
  const double r = 1.0 / m2;
  return make_double2(v.x * r, -v.y * r);
}
// barrier over the first `threads` threads that reach it (a multiple of 32)
// programmatic dependent launch (the solve's kernels are launched with it):
// a kernel may start while the kernel before it on its stream finishes; it
// reads nothing that kernel wrote before pdl_wait(), and lets the next
// kernel start launching (pdl_trigger) only once its own wait is over, so
// at most one launch waits ahead.  Both are no-ops for a plain launch.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }
// one 128-byte line of a row segment into L2 per lane (lanes beyond the
// segment idle)
__device__ __forceinline__ void prefetch_l2(const void* base, int bytes, int lane) {
  if (lane * 128 < bytes)
    asm volatile("prefetch.global.L2 [%0];" ::"l"((const char*)base + lane * 128));
}

__device__ __forceinline__ void named_barrier(int id, int threads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}
__device__ __forceinline__ void s_atomic_sub(float* p, float v) { atomicAdd(p, -v); }
__device__ __forceinline__ void s_atomic_sub(double* p, double v) { atomicAdd(p, -v); }
__device__ __forceinline__ void s_atomic_sub(float2* p, float2 v) {
  atomicAdd(&p->x, -v.x);
  atomicAdd(&p->y, -v.y);
}
__device__ __forceinline__ void s_atomic_sub(double2* p, double2 v) {
  atomicAdd(&p->x, -v.x);
  atomicAdd(&p->y, -v.y);
}
// shuffle down within groups of `width` lanes (a power of two)
__device__ __forceinline__ float s_shfl_down_w(float v, int o, int width) {
  return __shfl_down_sync(~0u, v, o, width);
}
__device__ __forceinline__ double s_shfl_down_w(double v, int o, int width) {
  return __shfl_down_sync(~0u, v, o, width);
}
__device__ __forceinline__ float2 s_shfl_down_w(float2 v, int o, int width) {
  return make_float2(__shfl_down_sync(~0u, v.x, o, width), __shfl_down_sync(~0u, v.y, o, width));
}
__device__ __forceinline__ double2 s_shfl_down_w(double2 v, int o, int width) {
  return make_double2(__shfl_down_sync(~0u, v.x, o, width), __shfl_down_sync(~0u, v.y, o, width));
}

template <typename S>
__device__ __forceinline__ S s_shfl_down(S v, int o);
template <>
__device__ __forceinline__ float s_shfl_down(float v, int o) { return __shfl_down_sync(~0u, v, o); }
template <>
__device__ __forceinline__ double s_shfl_down(double v, int o) { return __shfl_down_sync(~0u, v, o); }
template <>
__device__ __forceinline__ float2 s_shfl_down(float2 v, int o) {
  return make_float2(__shfl_down_sync(~0u, v.x, o), __shfl_down_sync(~0u, v.y, o));
}
template <>
__device__ __forceinline__ double2 s_shfl_down(double2 v, int o) {
  return make_double2(__shfl_down_sync(~0u, v.x, o), __shfl_down_sync(~0u, v.y, o));
}
// c ? a : b without a branch
__device__ __forceinline__ float s_sel(bool c, float a, float b) { return c ? a : b; }
__device__ __forceinline__ double s_sel(bool c, double a, double b) { return c ? a : b; }
__device__ __forceinline__ float2 s_sel(bool c, float2 a, float2 b) {
  return make_float2(c ? a.x : b.x, c ? a.y : b.y);
}
__device__ __forceinline__ double2 s_sel(bool c, double2 a, double2 b) {
  return make_double2(c ? a.x : b.x, c ? a.y : b.y);
}

template <typename S>
__device__ __forceinline__ S s_shfl(S v, int src);
template <>
__device__ __forceinline__ float s_shfl(float v, int s) { return __shfl_sync(~0u, v, s); }
template <>
__device__ __forceinline__ double s_shfl(double v, int s) { return __shfl_sync(~0u, v, s); }
template <>
__device__ __forceinline__ float2 s_shfl(float2 v, int s) {
  return make_float2(__shfl_sync(~0u, v.x, s), __shfl_sync(~0u, v.y, s));
}
template <>
__device__ __forceinline__ double2 s_shfl(double2 v, int s) {
  return make_double2(__shfl_sync(~0u, v.x, s), __shfl_sync(~0u, v.y, s));
}

// ---- per-node device metadata ----
struct DNode {
  int64_t off;  // front offset in the arena
  int64_t start;
  int32_t f, k;
  int64_t u_off;   // offset of U (new indices) in d_U
  int64_t ea_off;  // offset of the extend-add map in d_ea
  int32_t parent;
  int32_t child_slot;  // 0 or 1: position among the parent's children
};

#include "mf_tc.cuh"

// Self-test of the bounded mbarrier wait the tensor-core kernel relies on:
// one thread initialises a barrier that nothing will arrive at and waits
// for its first phase with the kernel's own wait, limited to `polls`; the
// wait must give up (status 1) and the kernel must return normally.
__global__ void wait_selftest_kernel(int polls, int* __restrict__ status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::smem_u32(&bar)));
  const bool done = tc::wait_parity(tc::smem_u32(&bar), 0, false, polls);
  *status = done ? 0 : 1;
}

// ---- factor kernels ----
template <typename S>
__global__ void scatter_kernel(int64_t m, const int32_t* __restrict__ src,
                               const int64_t* __restrict__ dst, const S* __restrict__ vals,
                               S* __restrict__ arena) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) arena[dst[i]] = vals[src[i]];
}

// children (of nodes in this level) with the given child slot add their
// Schur complement into the parent front; one block row per (child, row)
template <typename S>
__global__ void extend_add_kernel(const int32_t* __restrict__ kids, int nkids,
                                  const DNode* __restrict__ nodes, const int32_t* __restrict__ ea,
                                  S* __restrict__ arena) {
  pdl_wait();  // launched with programmatic dependent launch (launch_pdl)
  pdl_trigger();
  const int ci = blockIdx.y;
  if (ci >= nkids) return;
  const DNode c = nodes[kids[ci]];
  const int u = c.f - c.k;
  if (u <= 0 || c.parent < 0) return;
  const DNode p = nodes[c.parent];
  const int32_t* map = ea + c.ea_off;
  for (int r = blockIdx.x; r < u; r += gridDim.x) {
    const S* src = arena + c.off + (int64_t)(c.k + r) * c.f + c.k;
    S* dst = arena + p.off + (int64_t)map[r] * p.f;
    for (int j = threadIdx.x; j < u; j += blockDim.x) {
      S* d = dst + map[j];
      *d = s_add(*d, src[j]);
    }
  }
}

// largest |a_ij| of the values (non-negative doubles order like their bits)
__device__ __forceinline__ double mag2(float v) { return (double)v * v; }
__device__ __forceinline__ double mag2(double v) { return v * v; }
__device__ __forceinline__ double mag2(float2 v) { return (double)v.x * v.x + (double)v.y * v.y; }
__device__ __forceinline__ double mag2(double2 v) { return v.x * v.x + v.y * v.y; }
template <typename S>
__global__ void max_abs_kernel(int64_t m, const S* __restrict__ v,
                               unsigned long long* __restrict__ out) {
  double best = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * blockDim.x)
    best = fmax(best, mag2(v[i]));
  for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_down_sync(~0u, best, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(sqrt(best)));
}

// LU (no pivoting, static pivot replacement) of the nb x nb diagonal block;
// pivots with |p| below rel_tol * max|a_ij| are replaced by that value.
// Rows live in registers, LPR lanes per row (column q + LPR*s in slot s of
// lane q), warp w owning rows [w*RPW, (w+1)*RPW).  Step i: the lanes of row
// i publish it through shared memory (permuted so each lane's columns are
// contiguous, double-buffered) and the owner of a_ii its reciprocal; one
// named barrier over the warps that still own rows below i; the multiplier
// of every lower row is shuffled from the lane holding column i.  A warp
// whose rows are all final stores them and leaves, so the barrier shrinks
// with the remaining triangle.
template <typename S, int NBT>
__global__ void __launch_bounds__(256) diag_lu_kernel(const int32_t* __restrict__ list,
                                                      int count, const DNode* __restrict__ nodes,
                                                      S* __restrict__ arena, int p0,
                                                      const unsigned long long* __restrict__ amax,
                                                      double rel_tol, int* __restrict__ n_perturbed) {
  pdl_wait();  // launched with programmatic dependent launch (launch_pdl)
  pdl_trigger();
  constexpr int LPR = 256 / NBT;  // lanes per row
  constexpr int CPL = NBT / LPR;  // columns per lane
  constexpr int RPW = 32 / LPR;   // rows per warp
  constexpr int NW = 8;
  using R = decltype(s_mag2s(S()));
  __shared__ __align__(16) S rowbuf[2][LPR][CPL + 2];
  __shared__ S pinv[2];
  const int fi = blockIdx.x;
  if (fi >= count) return;
  const DNode nd = nodes[list[fi]];
  const int nb = min(NBT, nd.k - p0);
  if (nb <= 0) return;
  const double am = __longlong_as_double((long long)*amax);
  const double tau = rel_tol * (am > 0 ? am : 1.0);
  const R tau2 = (R)(tau * tau);
  S* base = arena + nd.off + (int64_t)p0 * nd.f + p0;
  const S zero = s_zero(S()), one = s_one(S());
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = lane % LPR, grp = lane - q;
  const int r = warp * RPW + lane / LPR;
  S v[CPL];
#pragma unroll
  for (int s = 0; s < CPL; ++s) {
    const int c = q + LPR * s;
    v[s] = (r < nb && c < nb) ? base[(int64_t)r * nd.f + c] : (r == c ? one : zero);
  }
  // the column groups are unrolled (register slots stay static), the steps
  // inside a group are not (keeps the kernel within the instruction cache)
#pragma unroll
  for (int sj = 0; sj < CPL; ++sj) {
#pragma unroll 1
    for (int jq = 0; jq < LPR; ++jq) {
      const int i = LPR * sj + jq;
      if (i >= nb || i / RPW > warp) goto finished;
      const int par = i & 1;
      if (r == i) {
        if (q == jq) {
          S piv = v[sj];
          R m2 = s_mag2s(piv);
          if (m2 < tau2) {
            piv = s_real(piv, tau);
            m2 = tau2;
            v[sj] = piv;
            atomicAdd(n_perturbed, 1);
          }
          pinv[par] = s_recip(piv, m2);
        }
#pragma unroll
        for (int s = sj; s < CPL; ++s) rowbuf[par][q][s] = v[s];
      }
      named_barrier(1, (NW - i / RPW) * 32);
      const S ci = s_shfl(v[sj], grp | jq);
      if (r > i) {
        const S l = s_mul(ci, pinv[par]);
        if (q == jq) v[sj] = l;
#pragma unroll
        for (int s = sj; s < CPL; ++s)
          if (q + LPR * s > i) v[s] = s_fms(v[s], l, rowbuf[par][q][s]);
      }
    }
  }
finished:
  if (r < nb) {
#pragma unroll
    for (int s = 0; s < CPL; ++s) {
      const int c = q + LPR * s;
      if (c < nb) base[(int64_t)r * nd.f + c] = v[s];
    }
  }
}

// panel solves by substitution: rows below the diagonal block
// (X U11 = A21, non-unit upper) and columns right of it (L11 X = A12, unit
// lower), 64 rows (or columns) per block.  Four lanes share a row: lane q
// holds the entries q, q+4, ... in registers; at step j the owner of entry j
// finishes it and hands it to the other three by a shuffle, so no block
// barrier is needed inside the substitution.
// Dynamic shared memory: D[NBT][NBT+1] (the factored block), T[64][NBT+1],
// then the NBT pivot reciprocals.
template <typename S, int NBT>
__global__ void __launch_bounds__(256) panel_trsm_kernel(const int32_t* __restrict__ list,
                                                         int count,
                                                         const DNode* __restrict__ nodes,
                                                         S* __restrict__ arena, int p0) {
  pdl_wait();  // launched with programmatic dependent launch (launch_pdl)
  pdl_trigger();
  constexpr int CPT = NBT / 4;
  extern __shared__ __align__(16) unsigned char trsm_smem[];
  S(*D)[NBT + 1] = reinterpret_cast<S(*)[NBT + 1]>(trsm_smem);
  S(*T)[NBT + 1] = D + NBT;
  const int fi = blockIdx.y;
  if (fi >= count) return;
  const DNode nd = nodes[list[fi]];
  const int nb = min(NBT, nd.k - p0);
  if (nb <= 0) return;
  const int rest = nd.f - p0 - nb;
  if (rest <= 0) return;
  const int tiles = (rest + 63) / 64;
  int tile = blockIdx.x;
  const bool rows = tile < tiles;
  if (!rows) tile -= tiles;
  if (tile >= tiles) return;
  const int first = p0 + nb + tile * 64;
  const int cnt = min(64, nd.f - first);
  S* F = arena + nd.off;
  const S zero = s_zero(S()), one = s_one(S());
  {
    // all loads of the block issued before the first shared-memory store
    constexpr int ND = NBT * NBT / 256, NT = 64 * NBT / 256;
    S dv[ND], tv[NT];
#pragma unroll
    for (int it = 0; it < ND; ++it) {
      const int t = it * 256 + threadIdx.x, r = t / NBT, c = t % NBT;
      dv[it] = (r < nb && c < nb) ? F[(int64_t)(p0 + r) * nd.f + p0 + c] : (r == c ? one : zero);
    }
#pragma unroll
    for (int it = 0; it < NT; ++it) {
      const int t = it * 256 + threadIdx.x;
      if (rows) {
        const int r = t / NBT, c = t % NBT;
        tv[it] = (r < cnt && c < nb) ? F[(int64_t)(first + r) * nd.f + p0 + c] : zero;
      } else {
        const int m = t / 64, c = t % 64;
        tv[it] = (m < nb && c < cnt) ? F[(int64_t)(p0 + m) * nd.f + first + c] : zero;
      }
    }
#pragma unroll
    for (int it = 0; it < ND; ++it) {
      const int t = it * 256 + threadIdx.x;
      D[t / NBT][t % NBT] = dv[it];
    }
#pragma unroll
    for (int it = 0; it < NT; ++it) {
      const int t = it * 256 + threadIdx.x;
      if (rows)
        T[t / NBT][t % NBT] = tv[it];
      else
        T[t % 64][t / 64] = tv[it];
    }
  }
  __syncthreads();
  S* rinv = reinterpret_cast<S*>(T + 64);  // reciprocals of the pivots
  if (rows) {
    if (threadIdx.x < NBT) {
      const S p = D[threadIdx.x][threadIdx.x];
      rinv[threadIdx.x] = s_recip(p, s_mag2s(p));
    }
    __syncthreads();
  }
  const int r = threadIdx.x >> 2, q = threadIdx.x & 3;
  const int lane = threadIdx.x & 31, grp = lane & ~3;
  S v[CPT];
#pragma unroll
  for (int s = 0; s < CPT; ++s) v[s] = T[r][q + 4 * s];
  // groups of four steps unrolled (register indices stay static), the
  // steps inside a group not (keeps the kernel within the instruction cache)
  if (rows) {
    // x_j = (a_j - sum_{i<j} x_i U_ij) / U_jj, right-looking over j
#pragma unroll
    for (int sj = 0; sj < CPT; ++sj)
#pragma unroll 1
      for (int jq = 0; jq < 4; ++jq) {
        const int j = 4 * sj + jq;
        if (j >= nb) break;
        if (q == jq) v[sj] = s_mul(v[sj], rinv[j]);
        const S xj = s_shfl(v[sj], grp | jq);
#pragma unroll
        for (int s = sj; s < CPT; ++s)
          if (q + 4 * s > j) v[s] = s_fms(v[s], xj, D[j][q + 4 * s]);
      }
  } else {
    // x_i = a_i - sum_{m<i} L_im x_m (unit diagonal)
#pragma unroll
    for (int sm = 0; sm < CPT; ++sm)
#pragma unroll 1
      for (int mq = 0; mq < 4; ++mq) {
        const int m = 4 * sm + mq;
        if (m >= nb) break;
        const S xm = s_shfl(v[sm], grp | mq);
#pragma unroll
        for (int s = sm; s < CPT; ++s)
          if (q + 4 * s > m) v[s] = s_fms(v[s], D[q + 4 * s][m], xm);
      }
  }
#pragma unroll
  for (int s = 0; s < CPT; ++s) T[r][q + 4 * s] = v[s];
  __syncthreads();
  if (rows) {
    for (int t = threadIdx.x; t < 64 * NBT; t += 256) {
      const int rr = t / NBT, c = t % NBT;
      if (rr < cnt && c < nb) F[(int64_t)(first + rr) * nd.f + p0 + c] = T[rr][c];
    }
  } else {
    for (int t = threadIdx.x; t < NBT * 64; t += 256) {
      const int m = t / 64, c = t % 64;
      if (m < nb && c < cnt) F[(int64_t)(p0 + m) * nd.f + first + c] = T[c][m];
    }
  }
}

// trailing update C -= Lpanel * Upanel over the (f-p0-nb)^2 block outside
// [bnd, f)^2, 64x64 tile per block, 4x4 outputs per thread, K = nb <= NBT.
// Dynamic shared memory: As[NBT][65] (As[t][i] = L[i][t]) then Bs[NBT][64].
template <typename S, int NBT>
__global__ void __launch_bounds__(256) gemm_update_kernel(const int32_t* __restrict__ list,
                                                          int count,
                                                          const DNode* __restrict__ nodes,
                                                          S* __restrict__ arena, int p0,
                                                          int sp) {
  pdl_wait();  // launched with programmatic dependent launch (launch_pdl)
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char gemm_smem[];
  S(*As)[65] = reinterpret_cast<S(*)[65]>(gemm_smem);
  S(*Bs)[64] = reinterpret_cast<S(*)[64]>(gemm_smem + sizeof(S) * NBT * 65);
  const int fi = blockIdx.y;
  if (fi >= count) return;
  const DNode nd = nodes[list[fi]];
  const int nb = min(NBT, nd.k - p0);
  if (nb <= 0) return;
  const int lo = p0 + nb;
  const int rest = nd.f - lo;
  if (rest <= 0) return;
  const int tpd = (rest + 63) / 64;
  if ((int)blockIdx.x >= tpd * tpd) return;
  const int ti = blockIdx.x / tpd, tj = blockIdx.x % tpd;
  const int i0 = lo + ti * 64, j0 = lo + tj * 64;
  // the (k,f) x (k,f) Schur block is updated once, after all panels, by
  // schur_update_kernel with the full K = k (see factor_t)
  // the block [bnd, f) x [bnd, f) is left for a later update with a longer
  // K: the Schur block (bnd = k) or, with super-panels of width sp, the
  // trailing block of the current super-panel
  const int bnd = sp > 0 ? min(nd.k, (p0 / sp) * sp + sp) : nd.k;
  if (i0 >= bnd && j0 >= bnd) return;
  S* F = arena + nd.off;
  {
    constexpr int NL = 64 * NBT / 256;
    S av[NL], bv[NL];
#pragma unroll
    for (int it = 0; it < NL; ++it) {
      const int t = it * 256 + threadIdx.x;
      const int i = t / NBT, c = t % NBT;
      av[it] = (i0 + i < nd.f && c < nb) ? F[(int64_t)(i0 + i) * nd.f + p0 + c] : s_zero(S());
      const int r = t / 64, j = t % 64;
      bv[it] = (j0 + j < nd.f && r < nb) ? F[(int64_t)(p0 + r) * nd.f + j0 + j] : s_zero(S());
    }
#pragma unroll
    for (int it = 0; it < NL; ++it) {
      const int t = it * 256 + threadIdx.x;
      As[t % NBT][t / NBT] = av[it];
      Bs[t / 64][t % 64] = bv[it];
    }
  }
  __syncthreads();
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  S acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = s_zero(S());
  // issue the C loads early; they are consumed after the contraction
  S cv[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = i0 + ty + 16 * a;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = j0 + tx + 16 * b;
      cv[a][b] = (i < nd.f && j < nd.f && (i < bnd || j < bnd)) ? F[(int64_t)i * nd.f + j]
                                                                 : s_zero(S());
    }
  }
  for (int t = 0; t < nb; ++t) {
    S av[4], bv[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) av[a] = As[t][ty + 16 * a];
#pragma unroll
    for (int b = 0; b < 4; ++b) bv[b] = Bs[t][tx + 16 * b];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] = s_fms(acc[a][b], av[a], bv[b]);
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = i0 + ty + 16 * a;
    if (i >= nd.f) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = j0 + tx + 16 * b;
      if (j >= nd.f || (i >= bnd && j >= bnd)) continue;
      F[(int64_t)i * nd.f + j] = s_add(cv[a][b], acc[a][b]);
    }
  }
}

// Schur block of a front, F[k:f, k:f] -= F[k:f, 0:k] F[0:k, k:f], once after
// the pivot panels: one 64x64 tile per block, K = k in chunks of KC
// (dynamic shared memory As[KC][65], Bs[KC][64]).
template <typename S, int KC>
__global__ void __launch_bounds__(256) schur_update_kernel(const int32_t* __restrict__ list,
                                                           int count,
                                                           const DNode* __restrict__ nodes,
                                                           S* __restrict__ arena) {
  pdl_wait();  // launched with programmatic dependent launch (launch_pdl)
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char schur_smem[];
  S(*As)[65] = reinterpret_cast<S(*)[65]>(schur_smem);
  S(*Bs)[64] = reinterpret_cast<S(*)[64]>(schur_smem + sizeof(S) * KC * 65);
  const int fi = blockIdx.y;
  if (fi >= count) return;
  const DNode nd = nodes[list[fi]];
  const int u = nd.f - nd.k;
  if (u <= 0 || nd.k <= 0) return;
  const int tpd = (u + 63) / 64;
  if ((int)blockIdx.x >= tpd * tpd) return;
  const int i0 = nd.k + (blockIdx.x / tpd) * 64, j0 = nd.k + (blockIdx.x % tpd) * 64;
  S* F = arena + nd.off;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  S acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = s_zero(S());
  // chunk kc of L21 (rows i0.., columns kc..) and U12 (rows kc.., columns
  // j0..) through registers, the next chunk loaded while this one is used
  constexpr int NL = 64 * KC / 256;
  S av[NL], bv[NL];
  auto load = [&](int kc) {
#pragma unroll
    for (int it = 0; it < NL; ++it) {
      const int t = it * 256 + threadIdx.x;
      const int i = t / KC, c = t % KC;
      av[it] = (i0 + i < nd.f && kc + c < nd.k) ? F[(int64_t)(i0 + i) * nd.f + kc + c]
                                                : s_zero(S());
      const int r = t / 64, j = t % 64;
      bv[it] = (j0 + j < nd.f && kc + r < nd.k) ? F[(int64_t)(kc + r) * nd.f + j0 + j]
                                                : s_zero(S());
    }
  };
  load(0);
  for (int kc = 0; kc < nd.k; kc += KC) {
    __syncthreads();
#pragma unroll
    for (int it = 0; it < NL; ++it) {
      const int t = it * 256 + threadIdx.x;
      As[t % KC][t / KC] = av[it];
      Bs[t / 64][t % 64] = bv[it];
    }
    __syncthreads();
    if (kc + KC < nd.k) load(kc + KC);
    const int kn = min(KC, nd.k - kc);
    for (int t = 0; t < kn; ++t) {
      S a4[4], b4[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) a4[a] = As[t][ty + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) b4[b] = Bs[t][tx + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = s_fms(acc[a][b], a4[a], b4[b]);
    }
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = i0 + ty + 16 * a;
    if (i >= nd.f) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = j0 + tx + 16 * b;
      if (j >= nd.f) continue;
      S* c = F + (int64_t)i * nd.f + j;
      *c = s_add(*c, acc[a][b]);
    }
  }
}

// ---- solve kernels (x in the new ordering) ----
// acc - sum_{j in [lo,hi)} row[j] * y[j] over the lanes of a warp, four
// independent partial sums so four loads per lane are in flight; the result
// is complete in lane 0.  IDX: y is gathered through idx (y[idx[j]]).
template <typename S, bool IDX>
__device__ __forceinline__ S warp_row_dot(const S* __restrict__ row, const S* y,
                                          const int32_t* __restrict__ idx, int lo, int hi,
                                          int lane) {
  S a0 = s_zero(S()), a1 = s_zero(S()), a2 = s_zero(S()), a3 = s_zero(S());
  int j = lo + lane;
  for (; j + 96 < hi; j += 128) {
    const S r0 = row[j], r1 = row[j + 32], r2 = row[j + 64], r3 = row[j + 96];
    const S y0 = IDX ? y[idx[j]] : y[j];
    const S y1 = IDX ? y[idx[j + 32]] : y[j + 32];
    const S y2 = IDX ? y[idx[j + 64]] : y[j + 64];
    const S y3 = IDX ? y[idx[j + 96]] : y[j + 96];
    a0 = s_fms(a0, r0, y0);
    a1 = s_fms(a1, r1, y1);
    a2 = s_fms(a2, r2, y2);
    a3 = s_fms(a3, r3, y3);
  }
  for (; j < hi; j += 32) a0 = s_fms(a0, row[j], IDX ? y[idx[j]] : y[j]);
  S acc = s_add(s_add(a0, a1), s_add(a2, a3));
  for (int o = 16; o > 0; o >>= 1) acc = s_add(acc, s_shfl_down(acc, o));
  return acc;
}

// The solve walks the pivot block [0, k) of every front in sub-panels
// [c0, c1) of P = solve_panel<S>() columns (c0 = j * P for sub-step j), so
// the dense triangular work of a large front is spread over many blocks:
// a one-block triangular solve of the sub-panel's diagonal tile (held whole
// in shared memory), then the products of the sub-panel with the rows
// (forward) or columns (backward) outside it, a warp per row over the GPU.
template <typename S>
__host__ __device__ constexpr int solve_panel() {
  return sizeof(S) == 16 ? 64 : 128;
}
constexpr int kTrsvThreads = 1024;      // block size of the sub-panel solves
constexpr int kBwdChunk = 1024;         // columns per warp in the backward products

// forward, sub-step j: y[c0:c1] = L[c0:c1, c0:c1]^-1 y[c0:c1] (unit lower),
// by one whole block for one front: the strictly lower tile and y[c0:c1] are
// loaded into shared memory, then 32 rows at a time: their products with
// the solved rows (a warp per row), then the 32 x 32 diagonal part by one
// warp.  Shared memory (smem): Dt[P][P+1], ys[P].  Uniform over the block;
// the caller separates two calls with a barrier.
template <typename S, int PT = solve_panel<S>(), int THR = kTrsvThreads>
__device__ __forceinline__ void fwd_trsv_front(const DNode& nd, const S* __restrict__ arena,
                                               S* __restrict__ x, int j, unsigned char* smem) {
  constexpr int P = solve_panel<S>();
  // the tile: PT x PT (PT >= the rows of the sub-panel, P = 128 columns
  // per sub-step), THR threads
  S(*Dt)[PT + 1] = reinterpret_cast<S(*)[PT + 1]>(smem);
  S* ys = reinterpret_cast<S*>(smem + sizeof(S) * PT * (PT + 1));
  const int c0 = j * P;
  if (nd.k <= c0) return;
  const int m = min(nd.k, c0 + P) - c0;
  if (m > PT) return;  // not for this tile size (the launch plan never asks)
  const S* F = arena + nd.off + (int64_t)c0 * nd.f + c0;
  S* y = x + nd.start + c0;
#pragma unroll
  for (int it = 0; it < PT * PT / THR; ++it) {
    const int t = it * THR + threadIdx.x;
    const int i = t / PT, jj = t % PT;
    if (i < m && jj < i) Dt[i][jj] = F[(int64_t)i * nd.f + jj];
  }
  pdl_wait();  // y[c0:c1] is the previous kernels' output
  pdl_trigger();
  for (int t = threadIdx.x; t < m; t += THR) ys[t] = y[t];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = THR >> 5;
  for (int b0 = 0; b0 < m; b0 += 32) {
    const int mb = min(32, m - b0);
    if (b0 > 0) {
      for (int r = b0 + warp; r < b0 + mb; r += nw) {
        S acc = s_zero(S());
        for (int c = lane; c < b0; c += 32) acc = s_fms(acc, Dt[r][c], ys[c]);
        for (int o = 16; o > 0; o >>= 1) acc = s_add(acc, s_shfl_down(acc, o));
        if (lane == 0) ys[r] = s_add(ys[r], acc);
      }
      __syncthreads();
    }
    if (warp == 0) {
      // the chain, two columns per step: for the pair (jj, jj + 1) every
      // row below takes
      //   v -= (L[i][jj] - L[i][jj+1] L[jj+1][jj]) x_jj + L[i][jj+1] v_jj+1
      // with v_jj+1 as it stands before the pair (row jj + 1 itself takes
      // v -= L[jj+1][jj] x_jj), so both shuffles of a pair are issued
      // together and its coefficient is formed off the dependent path.  No
      // divergent branch: the lanes that keep v discard a product formed
      // from whatever the unused triangle of Dt holds.
      const int rl = min(lane, mb - 1);
      S v = lane < mb ? ys[b0 + lane] : s_zero(S());
#pragma unroll
      for (int jj = 0; jj < 32; jj += 2) {
        const S l_a = Dt[b0 + rl][b0 + jj], l_b = Dt[b0 + rl][b0 + jj + 1];
        const S m_a = s_fms(l_a, l_b, Dt[b0 + jj + 1][b0 + jj]);
        const S xa = s_shfl(v, jj), vb = s_shfl(v, jj + 1);
        const S t2 = s_fms(s_fms(v, m_a, xa), l_b, vb);
        const S t1 = s_fms(v, l_a, xa);
        v = s_sel(lane > jj + 1 && lane < mb, t2, s_sel(lane == jj + 1 && lane < mb, t1, v));
      }
      if (lane < mb) ys[b0 + lane] = v;
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < m; t += THR) y[t] = ys[t];
}

// forward, sub-step j, row q of the rows [c1, f) of the front outside the
// sub-panel (one warp): row r takes -= L[r, c0:c1] . y[c0:c1]; rows inside
// the pivot block update y (one writer, or atomically when ATOM: the
// look-ahead schedule runs two launches on the same rows concurrently),
// rows of the update set go to the ancestors' x[U[r - k]] (atomic, sibling
// fronts share ancestors)
template <typename S, bool ATOM>
__device__ __forceinline__ void fwd_gemv_row(const DNode& nd, const int32_t* __restrict__ U,
                                             const S* __restrict__ arena, S* __restrict__ x,
                                             int c0, int c1, int q, int lane) {
  S* y = x + nd.start;
  const int r = c1 + q;
  const S* row = arena + nd.off + (int64_t)r * nd.f;
  const S acc = warp_row_dot<S, false>(row, y, nullptr, c0, c1, lane);
  if (lane == 0) {
    if (r < nd.k && !ATOM)
      y[r] = s_add(y[r], acc);
    else if (r < nd.k)
      s_atomic_sub(&y[r], s_fms(s_zero(S()), acc, s_real(S(), 1.0)));
    else
      s_atomic_sub(&x[U[nd.u_off + r - nd.k]], s_fms(s_zero(S()), acc, s_real(S(), 1.0)));
  }
}

// backward, sub-step j, work item w of rows [c0, c1) x chunks of kBwdChunk
// of the columns [cb, ce) outside the sub-panel (one warp): row r takes
// -= U[r, cb:ce] . x over its chunk (own variables y[c] for c < k, the
// ancestors' x[U[c - k]] beyond); with several chunks (or ATOM: another
// launch adds to the same rows concurrently) the partial sums are added
// atomically
template <typename S, bool ATOM>
__device__ __forceinline__ void bwd_gemv_item(const DNode& nd, const int32_t* __restrict__ U,
                                              const S* __restrict__ arena, S* __restrict__ x,
                                              int c0, int c1, int cb, int ce, int nch, int w,
                                              int lane) {
  S* y = x + nd.start;
  const int rows = c1 - c0;
  const int r = c0 + w % rows, ch = w / rows;
  const int lo = cb + ch * kBwdChunk, hi = min(ce, lo + kBwdChunk);
  const S* row = arena + nd.off + (int64_t)r * nd.f;
  S acc = s_zero(S());
  if (lo < nd.k) acc = warp_row_dot<S, false>(row, y, nullptr, lo, min(hi, nd.k), lane);
  if (hi > nd.k)
    acc = s_add(acc, warp_row_dot<S, true>(row + nd.k, x, U + nd.u_off, max(lo, nd.k) - nd.k,
                                           hi - nd.k, lane));
  if (lane == 0) {
    if (nch == 1 && !ATOM)
      y[r] = s_add(y[r], acc);
    else
      s_atomic_sub(&y[r], s_fms(s_zero(S()), acc, s_real(S(), 1.0)));
  }
}

// backward, sub-step j: y[c0:c1] = U[c0:c1, c0:c1]^-1 y[c0:c1] (upper,
// non-unit), by one whole block for one front, the upper tile and y in
// shared memory, 32 rows at a time from the bottom; the reciprocals of the
// diagonal are formed in parallel before each 32-row chain.
// Shared memory (smem): Dt[P][P+1], ys[P].
template <typename S, int PT = solve_panel<S>(), int THR = kTrsvThreads>
__device__ __forceinline__ void bwd_trsv_front(const DNode& nd, const S* __restrict__ arena,
                                               S* __restrict__ x, int j, unsigned char* smem) {
  constexpr int P = solve_panel<S>();
  // the tile: PT x PT (PT >= the rows of the sub-panel, P = 128 columns
  // per sub-step), THR threads
  S(*Dt)[PT + 1] = reinterpret_cast<S(*)[PT + 1]>(smem);
  S* ys = reinterpret_cast<S*>(smem + sizeof(S) * PT * (PT + 1));
  const int c0 = j * P;
  if (nd.k <= c0) return;
  const int m = min(nd.k, c0 + P) - c0;
  if (m > PT) return;  // not for this tile size (the launch plan never asks)
  const S* F = arena + nd.off + (int64_t)c0 * nd.f + c0;
  S* y = x + nd.start + c0;
#pragma unroll
  for (int it = 0; it < PT * PT / THR; ++it) {
    const int t = it * THR + threadIdx.x;
    const int i = t / PT, jj = t % PT;
    if (i < m && jj >= i && jj < m) Dt[i][jj] = F[(int64_t)i * nd.f + jj];
  }
  pdl_wait();
  pdl_trigger();
  for (int t = threadIdx.x; t < m; t += THR) ys[t] = y[t];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = THR >> 5;
  const int nblk = (m + 31) / 32;
  for (int bi = nblk - 1; bi >= 0; --bi) {
    const int b0 = bi * 32, b1 = min(b0 + 32, m), mb = b1 - b0;
    if (b1 < m) {
      for (int r = b0 + warp; r < b1; r += nw) {
        S acc = s_zero(S());
        for (int c = b1 + lane; c < m; c += 32) acc = s_fms(acc, Dt[r][c], ys[c]);
        for (int o = 16; o > 0; o >>= 1) acc = s_add(acc, s_shfl_down(acc, o));
        if (lane == 0) ys[r] = s_add(ys[r], acc);
      }
      __syncthreads();
    }
    if (warp == 0) {
      const int rl = min(lane, mb - 1);
      const S rinv = lane < mb ? s_div(s_one(S()), Dt[b0 + lane][b0 + lane]) : s_zero(S());
      S v = lane < mb ? ys[b0 + lane] : s_zero(S());
      // two columns per step, from the bottom: for the pair (a, b = a - 1),
      // x_a = v_a / U[a][a], x_b = (v_b - U[b][a] x_a) / U[b][b], and every
      // row above takes
      //   v -= (U[i][a] - U[i][b] U[b][a] / U[b][b]) x_a + U[i][b] / U[b][b] v_b
      // with v_b as it stands before the pair, so both shuffles of a pair are
      // issued together; the branches below are uniform over the warp (mb)
#pragma unroll
      for (int a = 31; a >= 1; a -= 2) {
        const int b = a - 1;
        if (a < mb) {
          const S u_a = Dt[b0 + rl][b0 + a], u_b = Dt[b0 + rl][b0 + b];
          const S n_b = s_mul(u_b, s_shfl(rinv, b));
          const S m_a = s_fms(u_a, n_b, Dt[b0 + b][b0 + a]);
          v = s_sel(lane == a, s_mul(v, rinv), v);
          const S xa = s_shfl(v, a), vb = s_shfl(v, b);
          const S t2 = s_fms(s_fms(v, m_a, xa), n_b, vb);
          const S t1 = s_mul(s_fms(v, u_a, xa), rinv);
          v = s_sel(lane < b, t2, s_sel(lane == b, t1, v));
        } else if (b < mb) {  // the block's last row alone
          v = s_sel(lane == b, s_mul(v, rinv), v);
          const S xj = s_shfl(v, b);
          const S t = s_fms(v, Dt[b0 + rl][b0 + b], xj);
          v = s_sel(lane < b, t, v);
        }
      }
      if (lane < mb) ys[b0 + lane] = v;
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < m; t += THR) y[t] = ys[t];
}

// one block per listed front (dynamic shared memory Dt[P][P+1], ys[P])
// one block per listed front (dynamic shared memory Dt[PT][PT+1], ys[PT]);
// the 64-row variant (PT = 64, 256 threads) serves the fronts whose
// sub-panel holds at most 64 rows, several blocks to an SM
template <typename S, int PT = solve_panel<S>(), int THR = kTrsvThreads>
__global__ void __launch_bounds__(THR) fwd_trsv_kernel(const int32_t* __restrict__ list, int count,
                                const DNode* __restrict__ nodes, const S* __restrict__ arena,
                                S* __restrict__ x, int j) {
  extern __shared__ __align__(16) unsigned char trsv_smem[];
  if ((int)blockIdx.x >= count) return;
  fwd_trsv_front<S, PT, THR>(nodes[list[blockIdx.x]], arena, x, j, trsv_smem);
}

// a warp per row of the listed front blockIdx.y, rows [c1 + q_lo, c1 + q_hi)
// of the rows [c1, f) outside the sub-panel
template <typename S, bool ATOM>
__global__ void fwd_gemv_kernel(const int32_t* __restrict__ list, int count,
                                const DNode* __restrict__ nodes, const int32_t* __restrict__ U,
                                const S* __restrict__ arena, S* __restrict__ x, int j, int q_lo,
                                int q_hi) {
  constexpr int P = solve_panel<S>();
  const int fi = blockIdx.y;
  if (fi >= count) return;
  const DNode nd = nodes[list[fi]];
  const int c0 = j * P;
  if (nd.k <= c0) return;
  const int c1 = min(nd.k, c0 + P);
  const int rows = min(nd.f - c1, q_hi);
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  // the factor rows do not depend on the kernels before: the first one is
  // requested while they finish
  if (q_lo + warp < rows)
    prefetch_l2(arena + nd.off + (int64_t)(c1 + q_lo + warp) * nd.f + c0, (c1 - c0) * (int)sizeof(S),
                lane);
  pdl_wait();
  pdl_trigger();
  const int w = c1 - c0;
  if (w > 32) {
    for (int q = q_lo + warp; q < rows; q += nwarps)
      fwd_gemv_row<S, ATOM>(nd, U, arena, x, c0, c1, q, lane);
    return;
  }
  // a narrow sub-panel (the last one of a front, or a small front): groups
  // of lpr lanes take a row each (2 to 8 rows per warp), at most two
  // columns per lane
  const int lpr = w > 16 ? 16 : w > 8 ? 8 : 4, rpw = 32 / lpr;
  const int sub = lane % lpr, grp = lane / lpr;
  S* y = x + nd.start;
  for (int qb = q_lo + warp * rpw; qb < rows; qb += nwarps * rpw) {
    const int q = qb + grp;
    S acc = s_zero(S());
    if (q < rows) {
      const S* row = arena + nd.off + (int64_t)(c1 + q) * nd.f;
      for (int c = c0 + sub; c < c1; c += lpr) acc = s_fms(acc, row[c], y[c]);
    }
    for (int o = lpr / 2; o > 0; o >>= 1) acc = s_add(acc, s_shfl_down_w(acc, o, lpr));
    if (sub == 0 && q < rows) {
      const int r = c1 + q;
      if (r < nd.k && !ATOM)
        y[r] = s_add(y[r], acc);
      else if (r < nd.k)
        s_atomic_sub(&y[r], s_fms(s_zero(S()), acc, s_real(S(), 1.0)));
      else
        s_atomic_sub(&x[U[nd.u_off + r - nd.k]], s_fms(s_zero(S()), acc, s_real(S(), 1.0)));
    }
  }
}

// a warp per (row, kBwdChunk columns) of the listed front blockIdx.y, the
// columns [c1 + col_lo, c1 + col_hi) of the columns [c1, f) outside the
// sub-panel
template <typename S, bool ATOM>
__global__ void bwd_gemv_kernel(const int32_t* __restrict__ list, int count,
                                const DNode* __restrict__ nodes, const int32_t* __restrict__ U,
                                const S* __restrict__ arena, S* __restrict__ x, int j, int col_lo,
                                int col_hi) {
  constexpr int P = solve_panel<S>();
  const int fi = blockIdx.y;
  if (fi >= count) return;
  const DNode nd = nodes[list[fi]];
  const int c0 = j * P;
  if (nd.k <= c0) return;
  const int c1 = min(nd.k, c0 + P);
  const int cb = c1 + col_lo, ce = c1 + min(nd.f - c1, col_hi);
  if (cb >= ce) return;
  const int rows = c1 - c0, ncol = ce - cb;
  const int nch = (ncol + kBwdChunk - 1) / kBwdChunk;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  if (warp < rows * nch) {
    const int lo = cb + (warp / rows) * kBwdChunk;
    prefetch_l2(arena + nd.off + (int64_t)(c0 + warp % rows) * nd.f + lo,
                (min(ce, lo + kBwdChunk) - lo) * (int)sizeof(S), lane);
  }
  pdl_wait();
  pdl_trigger();
  for (int w = warp; w < rows * nch; w += nwarps)
    bwd_gemv_item<S, ATOM>(nd, U, arena, x, c0, c1, cb, ce, nch, w, lane);
}

template <typename S, int PT = solve_panel<S>(), int THR = kTrsvThreads>
__global__ void __launch_bounds__(THR) bwd_trsv_kernel(const int32_t* __restrict__ list, int count,
                                const DNode* __restrict__ nodes, const S* __restrict__ arena,
                                S* __restrict__ x, int j) {
  extern __shared__ __align__(16) unsigned char trsv_smem[];
  if ((int)blockIdx.x >= count) return;
  bwd_trsv_front<S, PT, THR>(nodes[list[blockIdx.x]], arena, x, j, trsv_smem);
}

template <typename S, typename T>
__global__ void permute_in_kernel(int64_t n, const int64_t* __restrict__ perm,
                                  const T* __restrict__ b, S* __restrict__ x);
template <typename S, typename T>
__global__ void permute_out_kernel(int64_t n, const int64_t* __restrict__ perm,
                                   const S* __restrict__ x, T* __restrict__ out);

__device__ __forceinline__ void cvt(float& d, float s) { d = s; }
__device__ __forceinline__ void cvt(float& d, double s) { d = (float)s; }
__device__ __forceinline__ void cvt(double& d, float s) { d = s; }
__device__ __forceinline__ void cvt(double& d, double s) { d = s; }
__device__ __forceinline__ void cvt(float2& d, float2 s) { d = s; }
__device__ __forceinline__ void cvt(float2& d, double2 s) { d = make_float2((float)s.x, (float)s.y); }
__device__ __forceinline__ void cvt(double2& d, float2 s) { d = make_double2(s.x, s.y); }
__device__ __forceinline__ void cvt(double2& d, double2 s) { d = s; }

template <typename S, typename T>
__global__ void permute_in_kernel(int64_t n, const int64_t* __restrict__ perm,
                                  const T* __restrict__ b, S* __restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cvt(x[i], b[perm[i]]);
}
template <typename S, typename T>
__global__ void permute_out_kernel(int64_t n, const int64_t* __restrict__ perm,
                                   const S* __restrict__ x, T* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) cvt(out[perm[i]], x[i]);
}

}  // namespace

// ---- host object ----
// one tensor-core trailing update: the fronts of a level whose super-panel
// ends with the panel at p0
struct TcLaunch {
  int p0 = 0, ntiles = 0, nchunks = 0;
  double flops = 0;                 // algorithmic flops (8 per complex MAC)
  int32_t* d_tiles = nullptr;       // tc::TD ints per tile (see tc::tile_of)
  int32_t* d_strips = nullptr;      // 8 ints per operand strip (see tc_presplit_kernel)
  int32_t* d_chunk_strip = nullptr; // the strip of every K-chunk image
};

struct MFLevel {
  std::vector<int32_t> nodes_by_k;  // node ids sorted by k descending
  std::vector<TcLaunch> tcl;        // complex64 only: trailing updates, ordered by p0
  std::vector<TcLaunch> tcp;        // complex64 only: panel updates, one per panel (or none)
  std::vector<int32_t> kids[2];     // children by slot
  int max_k = 0, max_rest = 0, max_u = 0;
  int32_t* d_nodes = nullptr;
  int32_t* d_kids[2] = {nullptr, nullptr};
  std::vector<int> k_sorted;        // k of nodes_by_k
  std::vector<int> f_sorted;        // f of nodes_by_k
};

struct MFDevice {
  int device = -1;
  int dtype = -1;                   // SUCEM_F32 ...
  size_t elem = 0;
  void* arena = nullptr;
  DNode* d_nodes = nullptr;
  int32_t* d_U = nullptr;
  int32_t* d_ea = nullptr;
  int32_t* d_src = nullptr;
  int64_t* d_dst = nullptr;
  int64_t* d_perm = nullptr;
  void* d_x = nullptr;              // solve work vector (new ordering)
  int* d_flag = nullptr;            // perturbed pivot count
  cudaStream_t cap_stream = nullptr;  // private stream for capturing the solve graph
  cudaStream_t cap_side = nullptr;    // its look-ahead side stream (see solve_launches)
  std::vector<cudaEvent_t> solve_ev;  // fork/join events of the solve capture
  std::vector<cudaEvent_t> tc_ev;   // start/stop events around tensor-core launches
  int tc_n = 0;                     // tensor-core launches in the last factorisation
  double tc_flops = 0;              // their algorithmic flops (8 per complex MAC)
  cudaGraphExec_t solve_exec = nullptr;
  int solve_n = 0;                  // kernel launches in the solve graph
  int tc_sp = 0;                    // super-panel width of the tensor-core path (complex64)
  int sm_count = 1;                 // multiprocessors of the device
  int tc_panel_k = 0;               // see kTcPanelMinK
  uint8_t* d_img = nullptr;         // split operand chunk images of one tensor-core launch
  std::vector<MFLevel> levels;
  bool factored = false;
  int perturbed = 0;
  // end of the last factorisation on its stream; the first solve after it
  // waits for it and reads d_flag once (a factor whose tensor-core wait gave
  // up is refused)
  cudaEvent_t factor_ev = nullptr;
  bool checked = false;
  bool valid = true;
};

struct MFHandle {
  MFSymbolic sym;
  MFDevice dev;
  // plan parameters chosen by the caller (sucem_lu_configure; 0 = default):
  // super-panel width and the pivot-block threshold of the tensor-core
  // panel updates
  int cfg_superpanel = 0;
  int cfg_panel_k = 0;
};

namespace {

size_t elem_size(int dtype) {
  switch (dtype) {
    case SUCEM_F32: return 4;
    case SUCEM_F64: return 8;
    case SUCEM_C64: return 8;
    case SUCEM_C128: return 16;
  }
  return 0;
}

template <typename T>
cudaError_t upv(T** d, const std::vector<T>& h) {
  *d = nullptr;
  if (h.empty()) return cudaSuccess;
  cudaError_t e = cudaMalloc((void**)d, h.size() * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
}

void free_dev(MFDevice& d) {
  void* ptrs[] = {d.arena, d.d_nodes, d.d_U, d.d_ea, d.d_src, d.d_dst, d.d_perm, d.d_x, d.d_flag,
                  d.d_img};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  d.d_img = nullptr;
  for (auto& L : d.levels) {
    if (L.d_nodes) cudaFree(L.d_nodes);
    for (auto* v : {&L.tcl, &L.tcp})
      for (auto& t : *v) {
        int32_t* q[] = {t.d_tiles, t.d_strips, t.d_chunk_strip};
        for (int32_t* p : q)
          if (p) cudaFree(p);
      }
    for (int s = 0; s < 2; ++s)
      if (L.d_kids[s]) cudaFree(L.d_kids[s]);
  }
  if (d.solve_exec) cudaGraphExecDestroy(d.solve_exec);
  for (cudaEvent_t ev : d.tc_ev) cudaEventDestroy(ev);
  if (d.cap_stream) cudaStreamDestroy(d.cap_stream);
  if (d.cap_side) cudaStreamDestroy(d.cap_side);
  for (cudaEvent_t ev : d.solve_ev) cudaEventDestroy(ev);
  if (d.factor_ev) cudaEventDestroy(d.factor_ev);
  d = MFDevice();
}

// single-precision factorisations work in super-panels of d.tc_sp columns on every
// level; for each level, the panels p0 at which some fronts' super-panel
// ends get one tensor-core launch over exactly those fronts (list on the
// device).  Narrower super-panels move panel work onto the tensor cores
// but re-read and re-write the trailing block once per super-panel; on the
// 20^3 order-2 box the factorisation takes 48.7, 46.1, 44.5, 45.3, 45.6,
// 46.4 ms for widths 128, 192, 256, 384, 512, 768 (the autotuner's timed
// trials; sucem_lu_configure sets the width per handle).
// SUCEM_LU_SUPERPANEL overrides the default (a multiple of 64).
constexpr int kTcSuperPanel = 512;
// levels of at least two fronts whose largest pivot block has at least this
// many columns apply the K = 64 panel updates on the tensor cores as well (a
// single front's panel has too few tiles to fill the GPU: enabling them
// there too measured 44.8 against 44.5 ms on the 20^3 order-2 box);
// SUCEM_LU_TC_PANEL_K overrides the column threshold
constexpr int kTcPanelMinK = 64;
constexpr int kTcPanel = 64;  // panel width of the complex64 factorisation

// the tiles of one tensor-core launch and the operand strips they read
struct TcPlan {
  std::vector<int32_t> tiles;                                  // tc::TD ints per tile
  std::vector<int32_t> strips;                                 // 8 ints per strip
  std::map<std::array<int64_t, 5>, int32_t> strip_of;          // (node, side, first, kk0, K)
  int32_t strip(int32_t node, int side, int64_t first, int64_t n, int64_t kk0, int64_t K) {
    const std::array<int64_t, 5> key = {node, side, first, kk0, K};
    auto it = strip_of.find(key);
    if (it != strip_of.end()) {
      // one strip serves tiles of different extents: stage the widest (the
      // extra rows/columns only reach outputs that the narrower tile skips)
      int32_t& m = strips[8 * it->second + 2];
      m = std::max<int32_t>(m, (int32_t)n);
      return it->second;
    }
    const int32_t id = (int32_t)(strips.size() / 8);
    const int32_t v[8] = {node, (int32_t)first, (int32_t)n, (int32_t)kk0, (int32_t)K, 0, side, 0};
    strips.insert(strips.end(), v, v + 8);
    strip_of.emplace(key, id);
    return id;
  }
};

// 128 x 128 tiles of rows [r0, r1) x columns [c0, c1) of front `node`, K
// range [kk0, kk0 + K), appended with their A and B strips
void add_tiles(TcPlan& pl, int32_t node, int64_t r0, int64_t r1, int64_t c0, int64_t c1,
               int64_t kk0, int64_t K) {
  if (r1 <= r0 || c1 <= c0 || K <= 0) return;
  for (int64_t r = r0; r < r1; r += tc::BM)
    for (int64_t c = c0; c < c1; c += tc::BN) {
      const int64_t nr = std::min<int64_t>(tc::BM, r1 - r), nc = std::min<int64_t>(tc::BN, c1 - c);
      const int32_t a = pl.strip(node, 0, r, nr, kk0, K), b = pl.strip(node, 1, c, nc, kk0, K);
      const int32_t v[tc::TD] = {node, (int32_t)r, (int32_t)c, (int32_t)nr, (int32_t)nc, (int32_t)kk0,
                                 (int32_t)K, a, b, 0, 0, 0};
      pl.tiles.insert(pl.tiles.end(), v, v + tc::TD);
    }
}

// uploads a launch's tiles and strips: numbers the strips' K-chunk images
// and points every tile at the first image of its A and its B strip
cudaError_t upload_plan(TcPlan& pl, TcLaunch& t) {
  std::vector<int32_t> chunk_strip;
  const int32_t nstrips = (int32_t)(pl.strips.size() / 8);
  for (int32_t i = 0; i < nstrips; ++i) {
    pl.strips[8 * i + 5] = (int32_t)chunk_strip.size();
    const int32_t nch = (pl.strips[8 * i + 4] + tc::KC - 1) / tc::KC;
    chunk_strip.insert(chunk_strip.end(), nch, i);
  }
  t.ntiles = (int)(pl.tiles.size() / tc::TD);
  for (int i = 0; i < t.ntiles; ++i) {
    int32_t* td = &pl.tiles[(size_t)tc::TD * i];
    td[7] = pl.strips[8 * td[7] + 5];
    td[8] = pl.strips[8 * td[8] + 5];
  }
  t.nchunks = (int)chunk_strip.size();
  cudaError_t e = upv(&t.d_tiles, pl.tiles);
  if (e == cudaSuccess) e = upv(&t.d_strips, pl.strips);
  if (e == cudaSuccess) e = upv(&t.d_chunk_strip, chunk_strip);
  return e;
}

cudaError_t plan_tc(MFDevice& d, const MFSymbolic& s, double mac_flops, size_t chunk_bytes,
                    int cfg_sp, int cfg_pk) {
  int max_chunks = 0;
  d.tc_sp = kTcSuperPanel;
  d.tc_panel_k = kTcPanelMinK;
  if (const char* v = getenv("SUCEM_LU_TC_PANEL_K")) d.tc_panel_k = atoi(v);
  if (cfg_pk > 0) d.tc_panel_k = cfg_pk;
  cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, d.device);
  if (const char* v = getenv("SUCEM_LU_SUPERPANEL")) {
    const int w = atoi(v);
    if (w >= kTcPanel && w % kTcPanel == 0) d.tc_sp = w;
  }
  if (cfg_sp >= kTcPanel && cfg_sp % kTcPanel == 0) d.tc_sp = cfg_sp;
  const int sp = d.tc_sp;
  for (auto& L : d.levels) {
    std::vector<std::pair<int, int32_t>> ends;  // (p0, node)
    for (int32_t i : L.nodes_by_k) {
      const MFNode& nd = s.nodes[i];
      for (int64_t p0 = 0; p0 < nd.k; p0 += kTcPanel) {
        const int64_t lo = p0 + std::min<int64_t>(kTcPanel, nd.k - p0);
        const int64_t bnd = std::min<int64_t>(nd.k, (p0 / sp) * (int64_t)sp + sp);
        if (lo == bnd && bnd < nd.f) ends.push_back({(int)p0, i});
      }
    }
    std::stable_sort(ends.begin(), ends.end(),
                     [](const std::pair<int, int32_t>& a, const std::pair<int, int32_t>& b) {
                       return a.first < b.first;
                     });
    for (size_t a = 0; a < ends.size();) {
      size_t b = a;
      TcLaunch t;
      t.p0 = ends[a].first;
      TcPlan pl;  // the tiles of every front, front by front
      for (; b < ends.size() && ends[b].first == t.p0; ++b) {
        const MFNode& nd = s.nodes[ends[b].second];
        const int64_t sp0 = (t.p0 / sp) * (int64_t)sp;
        const int64_t bnd = std::min<int64_t>(nd.k, sp0 + sp);
        add_tiles(pl, ends[b].second, bnd, nd.f, bnd, nd.f, sp0, bnd - sp0);
        t.flops += mac_flops * (double)(nd.f - bnd) * (double)(nd.f - bnd) * (double)(bnd - sp0);
      }
      cudaError_t e = upload_plan(pl, t);
      L.tcl.push_back(t);  // registered before a failure so that free_dev releases it
      if (e != cudaSuccess) return e;
      max_chunks = std::max(max_chunks, t.nchunks);
      a = b;
    }
    // panel updates on the tensor cores
    if (L.max_k < d.tc_panel_k || L.nodes_by_k.size() < 2) continue;
    for (int p0 = 0; p0 < L.max_k; p0 += kTcPanel) {
      TcLaunch t;
      t.p0 = p0;
      TcPlan pl;
      for (int32_t i : L.nodes_by_k) {
        const MFNode& nd = s.nodes[i];
        if (nd.k <= p0) break;  // k-descending
        const int64_t nb = std::min<int64_t>(kTcPanel, nd.k - p0), lo = p0 + nb;
        const int64_t bnd = std::min<int64_t>(nd.k, (p0 / sp) * (int64_t)sp + sp);
        if (bnd <= lo) continue;
        add_tiles(pl, i, lo, nd.f, lo, bnd, p0, nb);   // rows [lo, f) x cols [lo, bnd)
        add_tiles(pl, i, lo, bnd, bnd, nd.f, p0, nb);  // rows [lo, bnd) x cols [bnd, f)
        t.flops += mac_flops * (double)nb *
                   ((double)(nd.f - lo) * (bnd - lo) + (double)(bnd - lo) * (nd.f - bnd));
      }
      cudaError_t e = upload_plan(pl, t);
      L.tcp.push_back(t);
      if (e != cudaSuccess) return e;
      max_chunks = std::max(max_chunks, t.nchunks);
    }
  }
  // one image buffer serves every launch (launches are stream-ordered)
  if (max_chunks > 0) return cudaMalloc((void**)&d.d_img, (size_t)max_chunks * chunk_bytes);
  return cudaSuccess;
}

cudaError_t setup_device(MFHandle& h, int dtype) {
  MFDevice& d = h.dev;
  int dev = 0;
  cudaGetDevice(&dev);
  if (d.device == dev && d.dtype == dtype) return cudaSuccess;
  free_dev(d);
  d.device = dev;
  d.dtype = dtype;
  d.elem = elem_size(dtype);
  const MFSymbolic& s = h.sym;
  std::vector<DNode> dn(s.nodes.size());
  std::vector<int32_t> U;
  for (size_t i = 0; i < s.nodes.size(); ++i) {
    const MFNode& nd = s.nodes[i];
    dn[i].off = nd.front_off;
    dn[i].start = nd.start;
    dn[i].f = (int32_t)nd.f;
    dn[i].k = (int32_t)nd.k;
    dn[i].u_off = (int64_t)U.size();
    for (int64_t u : nd.U) U.push_back((int32_t)u);
    dn[i].ea_off = nd.ea_off;
    dn[i].parent = nd.parent;
    dn[i].child_slot = 0;
  }
  for (size_t i = 0; i < s.nodes.size(); ++i)
    for (size_t c = 0; c < s.nodes[i].children.size(); ++c) dn[s.nodes[i].children[c]].child_slot = (int)c;
  d.levels.assign(s.max_level + 1, MFLevel());
  for (size_t i = 0; i < s.nodes.size(); ++i) {
    const MFNode& nd = s.nodes[i];
    MFLevel& L = d.levels[nd.level];
    L.nodes_by_k.push_back((int32_t)i);
    for (size_t c = 0; c < nd.children.size() && c < 2; ++c) L.kids[c].push_back(nd.children[c]);
  }
  cudaError_t e = cudaSuccess;
  for (auto& L : d.levels) {
    std::sort(L.nodes_by_k.begin(), L.nodes_by_k.end(),
              [&](int32_t a, int32_t b) { return s.nodes[a].k > s.nodes[b].k; });
    for (int32_t i : L.nodes_by_k) {
      L.k_sorted.push_back((int)s.nodes[i].k);
      L.f_sorted.push_back((int)s.nodes[i].f);
      L.max_k = std::max<int>(L.max_k, (int)s.nodes[i].k);
      L.max_rest = std::max<int>(L.max_rest, (int)s.nodes[i].f);
      L.max_u = std::max<int>(L.max_u, (int)(s.nodes[i].f - s.nodes[i].k));
    }
    if (e == cudaSuccess) e = upv(&L.d_nodes, L.nodes_by_k);
    for (int c = 0; c < 2; ++c)
      if (e == cudaSuccess) e = upv(&L.d_kids[c], L.kids[c]);
  }
  if (e == cudaSuccess) e = upv(&d.d_nodes, dn);
  if (e == cudaSuccess) e = upv(&d.d_U, U);
  if (e == cudaSuccess) e = upv(&d.d_ea, s.ea_map);
  if (e == cudaSuccess) e = upv(&d.d_src, s.scat_src);
  if (e == cudaSuccess) e = upv(&d.d_dst, s.scat_dst);
  if (e == cudaSuccess) e = upv(&d.d_perm, s.perm);
  if (e == cudaSuccess) e = cudaMalloc(&d.arena, (size_t)std::max<int64_t>(s.arena, 1) * d.elem);
  if (e == cudaSuccess) e = cudaMalloc(&d.d_x, (size_t)std::max<int64_t>(s.n, 1) * d.elem);
  if (e == cudaSuccess) e = cudaMalloc((void**)&d.d_flag, 16);
  if (e == cudaSuccess && dtype == SUCEM_C64)
    e = plan_tc(d, s, kMacFlops<float2>, tc::chunk_bytes<float2>(), h.cfg_superpanel, h.cfg_panel_k);
  if (e == cudaSuccess && dtype == SUCEM_F32)
    e = plan_tc(d, s, kMacFlops<float>, tc::chunk_bytes<float>(), h.cfg_superpanel, h.cfg_panel_k);
  if (e != cudaSuccess) free_dev(d);
  return e;
}

// a kernel launched with programmatic dependent launch on its stream (see
// pdl_wait / pdl_trigger): the solve kernels and the factorisation's level
// kernels
template <typename... KArgs, typename... Args>
void launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                Args... args) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, ((KArgs)args)...);
}

// events around the i-th tensor-core launch of a factorisation
cudaError_t tc_event(MFDevice& d, int i, int which, cudaStream_t st) {
  while ((int)d.tc_ev.size() < 2 * (i + 1)) {
    cudaEvent_t ev;
    cudaError_t e = cudaEventCreate(&ev);
    if (e != cudaSuccess) return e;
    d.tc_ev.push_back(ev);
  }
  return cudaEventRecord(d.tc_ev[2 * i + which], st);
}

// one tensor-core update launch (persistent: one CTA per SM, at most one per
// tile), with events around it for sucem_lu_kernel_stats
template <typename S>
cudaError_t tc_launch(MFDevice& d, const TcLaunch& t, S* arena, cudaStream_t st) {
  if constexpr (!kTensorCore<S>) {
    return cudaErrorInvalidValue;  // double precision has no tensor-core plan
  } else {
    if (t.ntiles == 0) return cudaSuccess;
    const int grid = std::max(1, std::min(t.ntiles, d.sm_count));
    cudaError_t e = tc_event(d, d.tc_n, 0, st);
    if (e != cudaSuccess) return e;
    launch_pdl(tc_presplit_kernel<S>, t.nchunks, 256, 0, st, t.d_strips, t.d_chunk_strip, d.d_nodes, arena,
                                                      d.d_img);
    launch_pdl(tc_update_kernel<S>, grid, tc::THREADS, tc::smem_bytes<S>(), st, 
        t.d_tiles, t.ntiles, d.d_nodes, arena, d.d_img, d.d_flag + 1);
    e = tc_event(d, d.tc_n, 1, st);
    if (e != cudaSuccess) return e;
    d.tc_n++;
    d.tc_flops += t.flops;
    count_launch(2);
    return cudaSuccess;
  }
}

template <typename S>
cudaError_t factor_t(MFHandle& h, const void* vals, double tau, cudaStream_t st) {
  // panel width 64 (32 for complex double, whose tiles would not fit)
  constexpr int NBT = sizeof(S) <= 8 ? 64 : 32;
  static_assert(!kTensorCore<S> || NBT == kTcPanel, "tensor-core plan assumes this panel width");
  const size_t trsm_smem = sizeof(S) * ((size_t)(NBT + 64) * (NBT + 1) + NBT);
  // grids of at most one block per SM request this much shared memory so
  // that no two of their (latency-bound) blocks share an SM
  constexpr size_t kSoloSmem = 116 * 1024;
  const size_t gemm_smem = sizeof(S) * (size_t)NBT * (65 + 64);
  constexpr int kSchurKC = 32;
  const size_t schur_smem = sizeof(S) * (size_t)kSchurKC * (65 + 64);
  {
    cudaError_t ea = cudaFuncSetAttribute(panel_trsm_kernel<S, NBT>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)std::max(trsm_smem, kSoloSmem));
    if (ea == cudaSuccess)
      ea = cudaFuncSetAttribute(diag_lu_kernel<S, NBT>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSoloSmem);
    if (ea == cudaSuccess)
      ea = cudaFuncSetAttribute(gemm_update_kernel<S, NBT>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem);
    if constexpr (kTensorCore<S>)
      if (ea == cudaSuccess)
        ea = cudaFuncSetAttribute(tc_update_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  tc::smem_bytes<S>());
    if (ea == cudaSuccess)
      ea = cudaFuncSetAttribute(schur_update_kernel<S, kSchurKC>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)schur_smem);
    if (ea != cudaSuccess) return ea;
  }
  MFDevice& d = h.dev;
  const MFSymbolic& s = h.sym;
  S* arena = (S*)d.arena;
  d.tc_n = 0;
  d.tc_flops = 0;
  cudaError_t e = cudaMemsetAsync(arena, 0, (size_t)s.arena * sizeof(S), st);
  // d_flag[0]: perturbed-pivot count; d_flag[1]: tensor-core update timed
  // out; d_flag[2..3]: max |a_ij| (as bits)
  if (e == cudaSuccess) e = cudaMemsetAsync(d.d_flag, 0, 16, st);
  if (e != cudaSuccess) return e;
  unsigned long long* amax = reinterpret_cast<unsigned long long*>(d.d_flag + 2);
  max_abs_kernel<S><<<256, 256, 0, st>>>(s.nnz, (const S*)vals, amax);
  count_launch(1);
  const int64_t m = (int64_t)s.scat_src.size();
  if (m > 0) {
    scatter_kernel<S><<<(unsigned)((m + 255) / 256), 256, 0, st>>>(m, d.d_src, d.d_dst,
                                                                   (const S*)vals, arena);
    count_launch(1);
  }
  // SUCEM_LU_PROFILE=1 prints the device time of every tree level (stderr);
  // =2 also splits it by kernel kind (every launch then synchronises, so the
  // split includes each launch's latency)
  const char* prof_env = getenv("SUCEM_LU_PROFILE");
  const bool prof = prof_env != nullptr;
  const bool prof2 = prof && atoi(prof_env) >= 2;
  cudaEvent_t ev[2], kev[2];
  double kind_ms[6] = {0, 0, 0, 0, 0, 0};  // extend-add, diag, trsm, gemm, tensor core, schur
  if (prof) {
    cudaEventCreate(&ev[0]);
    cudaEventCreate(&ev[1]);
    cudaEventCreate(&kev[0]);
    cudaEventCreate(&kev[1]);
    cudaEventRecord(ev[0], st);
    cudaEventRecord(kev[0], st);
  }
  auto mark = [&](int kind) {
    if (!prof2) return;
    cudaEventRecord(kev[1], st);
    cudaEventSynchronize(kev[1]);
    float ms = 0;
    cudaEventElapsedTime(&ms, kev[0], kev[1]);
    kind_ms[kind] += ms;
    cudaEventRecord(kev[0], st);
  };
  for (size_t lv = 0; lv < d.levels.size(); ++lv) {
    const MFLevel& L = d.levels[lv];
    for (int c = 0; c < 2; ++c) {
      const int nk = (int)L.kids[c].size();
      if (nk == 0) continue;
      dim3 grid(std::max(16, std::min(1024, 8192 / nk)), nk);
      launch_pdl(extend_add_kernel<S>, grid, 256, 0, st, L.d_kids[c], nk, d.d_nodes, d.d_ea, arena);
      count_launch(1);
      mark(0);
    }
    // single precision: every level in super-panels of d.tc_sp columns,
    // the trailing blocks on the tensor cores (precomputed launch lists);
    // double precision: one Schur update per level
    const int nall = (int)L.nodes_by_k.size();
    const bool tc_level = kTensorCore<S> && d.tc_sp > 0;
    const int spw = tc_level ? d.tc_sp : 0;
    size_t next_tc = 0;
    for (int p0 = 0; p0 < L.max_k; p0 += NBT) {
      // active fronts: prefix of the k-descending list with k > p0
      int cnt = 0;
      while (cnt < (int)L.k_sorted.size() && L.k_sorted[cnt] > p0) ++cnt;
      if (cnt == 0) break;
      launch_pdl(diag_lu_kernel<S, NBT>, cnt, 256, cnt <= d.sm_count ? kSoloSmem : 0, st, 
          L.d_nodes, cnt, d.d_nodes, arena, p0, amax, tau, d.d_flag);
      count_launch(1);
      mark(1);
      const int rest = std::max(0, L.max_rest - p0 - 1);
      const int tiles = (rest + 63) / 64;
      if (tiles > 0) {
        dim3 g1(2 * tiles, cnt);
        const size_t tsm = (int64_t)g1.x * g1.y <= d.sm_count ? std::max(trsm_smem, kSoloSmem)
                                                               : trsm_smem;
        launch_pdl(panel_trsm_kernel<S, NBT>, g1, 256, tsm, st, L.d_nodes, cnt, d.d_nodes, arena, p0);
        count_launch(1);
        mark(2);
        // K = nb panel update outside the deferred block
        const size_t pi = (size_t)(p0 / NBT);
        if (tc_level && pi < L.tcp.size()) {
          const TcLaunch& t = L.tcp[pi];
          if (t.ntiles > 0) {
            e = tc_launch<S>(d, t, arena, st);
            if (e != cudaSuccess) return e;
          }
          mark(4);
        } else {
          const int tpd = (rest + 63) / 64;
          dim3 g2(tpd * tpd, cnt);
          launch_pdl(gemm_update_kernel<S, NBT>, g2, 256, gemm_smem, st, L.d_nodes, cnt, d.d_nodes,
                                                                  arena, p0, spw);
          count_launch(1);
          mark(3);
        }
      }
      if (tc_level) {
        // fronts whose super-panel ends with this panel: trailing block on
        // the tensor cores, one launch over exactly those fronts
        while (next_tc < L.tcl.size() && L.tcl[next_tc].p0 == p0) {
          e = tc_launch<S>(d, L.tcl[next_tc++], arena, st);
          if (e != cudaSuccess) return e;
          mark(4);
        }
      }
    }
    // Schur blocks F[k:f, k:f] -= L21 U12 with the full K = k, before the
    // parent level's extend-add reads them
    if (!tc_level && L.max_u > 0 && nall > 0) {
      // one batched launch for all fronts of the level
      const int tpd = (L.max_u + 63) / 64;
      dim3 g3(tpd * tpd, nall);
      launch_pdl(schur_update_kernel<S, kSchurKC>, g3, 256, schur_smem, st, L.d_nodes, nall, d.d_nodes,
                                                                     arena);
      count_launch(1);
      mark(5);
    }
    if (prof) {
      cudaEventRecord(ev[1], st);
      cudaEventSynchronize(ev[1]);
      float ms = 0;
      cudaEventElapsedTime(&ms, ev[0], ev[1]);
      fprintf(stderr, "[sucem lu] level %zu fronts %zu max_k %d max_f %d  %.3f ms", lv,
              L.nodes_by_k.size(), L.max_k, L.max_rest, ms);
      if (prof2)
        fprintf(stderr, "  (extend %.3f diag %.3f trsm %.3f gemm %.3f tc %.3f schur %.3f)", kind_ms[0],
                kind_ms[1], kind_ms[2], kind_ms[3], kind_ms[4], kind_ms[5]);
      fprintf(stderr, "\n");
      for (double& k : kind_ms) k = 0;
      cudaEventRecord(ev[0], st);
    }
  }
  if (prof) {
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    cudaEventDestroy(kev[0]);
    cudaEventDestroy(kev[1]);
  }
  return cudaGetLastError();
}

template <typename S>
cudaError_t solve_prepare() {
  constexpr int P = solve_panel<S>();
  const size_t smem = sizeof(S) * (size_t)P * (P + 2);
  cudaError_t e = cudaFuncSetAttribute(fwd_trsv_kernel<S>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(bwd_trsv_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
  // the 64-row tiles (solve_launches)
  const int smem_s = (int)(sizeof(S) * 64 * 66);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(fwd_trsv_kernel<S, 64, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem_s);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(bwd_trsv_kernel<S, 64, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem_s);
  return e;
}

// The launches of one solve on the work vector d_x (captured into a graph);
// returns their count, or -1 when an event or stream call failed.
//
// Levels of three or more sub-steps and at most kLookaheadFronts fronts
// (the few large fronts at the top of the tree, whose sub-steps form the
// solve's critical path) take a look-ahead
// schedule over two streams: each sub-step's products are split into the
// part the next sub-step's triangular solve needs (the next 128 rows
// forward, the just-solved 128 columns backward), kept on the main stream
// between the triangular solves, and the rest, issued on a side stream
// that runs beside the next sub-step (forward: rows beyond the next
// sub-panel; backward: columns solved two sub-steps earlier).  The two
// launches that add to the same rows concurrently do so atomically.
// SUCEM_LU_SOLVE_SEQUENTIAL keeps one stream throughout.
template <typename S>
int solve_launches(MFDevice& d, cudaStream_t st) {
  constexpr int P = solve_panel<S>();
  const size_t smem = sizeof(S) * (size_t)P * (P + 2);
  S* x = (S*)d.d_x;
  const S* arena = (const S*)d.arena;
  const bool look = !getenv("SUCEM_LU_SOLVE_SEQUENTIAL");
  cudaStream_t side = d.cap_side;
  int n = 0;
  // events of one level, reused level after level (a wait captures the
  // event's node at the time of the call)
  int evi = 0;
  bool ok = true;
  auto ev = [&]() -> cudaEvent_t {
    while ((int)d.solve_ev.size() <= evi) {
      cudaEvent_t e;
      if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
        ok = false;
        return nullptr;
      }
      d.solve_ev.push_back(e);
    }
    return d.solve_ev[evi++];
  };
  auto record = [&](cudaEvent_t e, cudaStream_t s) { ok = ok && e && cudaEventRecord(e, s) == cudaSuccess; };
  auto wait = [&](cudaStream_t s, cudaEvent_t e) { ok = ok && e && cudaStreamWaitEvent(s, e, 0) == cudaSuccess; };
  const int kAll = 1 << 30;
  // the look-ahead pays on the few large fronts at the top of a tree, whose
  // sub-steps are a latency chain; levels of many fronts are bound by their
  // bytes and take the one-stream sequence
  constexpr int kLookaheadFronts = 64;
  // the fronts a sub-step touches (the k-descending prefix with k > j P)
  // and the grid width of its products: the mean work per active front in
  // warps of 8 per block (grid-stride loops take the larger fronts), so a
  // level of many small fronts and a few large ones launches no empty blocks
  auto active = [&](const MFLevel& L, int j) {
    int c = 0;
    while (c < (int)L.k_sorted.size() && L.k_sorted[c] > j * P) ++c;
    return c;
  };
  // the triangular solves of a sub-step: fronts whose sub-panel holds more
  // than 64 rows (a prefix of the k-descending list) take the 128-row tile
  // with 1024 threads, the rest the 64-row tile with 256 threads
  constexpr int PS = 64, TS = 256;
  const size_t smem_s = sizeof(S) * (size_t)PS * (PS + 2);
  auto trsv = [&](const MFLevel& L, int j, int na, bool fwd, cudaStream_t s) {
    int nb = 0;
    while (nb < na && L.k_sorted[nb] > j * P + PS) ++nb;
    if (nb > 0) {
      if (fwd)
        launch_pdl(fwd_trsv_kernel<S>, nb, kTrsvThreads, smem, s, L.d_nodes, nb, d.d_nodes, arena, x, j);
      else
        launch_pdl(bwd_trsv_kernel<S>, nb, kTrsvThreads, smem, s, L.d_nodes, nb, d.d_nodes, arena, x, j);
      ++n;
    }
    if (na > nb) {
      const int32_t* rest = L.d_nodes + nb;
      if (fwd)
        launch_pdl(fwd_trsv_kernel<S, PS, TS>, na - nb, TS, smem_s, s, rest, na - nb, d.d_nodes, arena, x, j);
      else
        launch_pdl(bwd_trsv_kernel<S, PS, TS>, na - nb, TS, smem_s, s, rest, na - nb, d.d_nodes, arena, x, j);
      ++n;
    }
  };
  auto fwd_width = [&](const MFLevel& L, int j, int na, int lo, int hi) {
    int64_t rows = 0;
    for (int a = 0; a < na; ++a) {
      const int c1 = std::min(L.k_sorted[a], (j + 1) * P);
      rows += std::max(0, std::min(L.f_sorted[a] - c1, hi) - lo);
    }
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(512, (rows / std::max(na, 1) + 7) / 8));
  };
  auto bwd_width = [&](const MFLevel& L, int j, int na, int lo, int hi) {
    int64_t items = 0;
    for (int a = 0; a < na; ++a) {
      const int c0 = j * P, c1 = std::min(L.k_sorted[a], c0 + P);
      const int cols = std::max(0, std::min(L.f_sorted[a] - c1, hi) - lo);
      items += (int64_t)(c1 - c0) * ((cols + kBwdChunk - 1) / kBwdChunk);
    }
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(512, (items / std::max(na, 1) + 7) / 8));
  };
  for (size_t lv = 0; lv < d.levels.size() && ok; ++lv) {
    const MFLevel& L = d.levels[lv];
    const int cnt = (int)L.nodes_by_k.size();
    const int nsub = (L.max_k + P - 1) / P;
    if (!look || nsub < 3 || cnt > kLookaheadFronts || !side) {
      for (int j = 0; j < nsub; ++j) {
        const int na = active(L, j);
        trsv(L, j, na, true, st);
        dim3 g(fwd_width(L, j, na, 0, kAll), na);
        launch_pdl(fwd_gemv_kernel<S, false>, g, 256, 0, st, L.d_nodes, na, d.d_nodes, d.d_U, arena, x,
                                                      j, 0, kAll);
        n += 1;
      }
      continue;
    }
    evi = 0;
    std::vector<cudaEvent_t> done_rest(nsub, nullptr);
    for (int j = 0; j < nsub && ok; ++j) {
      if (j >= 2) wait(st, done_rest[j - 2]);
      const int na = active(L, j);
      trsv(L, j, na, true, st);
      cudaEvent_t solved = ev();
      record(solved, st);
      // the next sub-panel's rows, then the rest beside the next sub-step
      launch_pdl(fwd_gemv_kernel<S, true>, dim3(fwd_width(L, j, na, 0, P), na), 256, 0, st,
                 L.d_nodes, na, d.d_nodes, d.d_U, arena, x, j, 0, P);
      wait(side, solved);
      {
        dim3 g(fwd_width(L, j, na, P, kAll), na);
        launch_pdl(fwd_gemv_kernel<S, true>, g, 256, 0, side, L.d_nodes, na, d.d_nodes, d.d_U, arena, x,
                                                      j, P, kAll);
      }
      done_rest[j] = ev();
      record(done_rest[j], side);
      n += 2;
    }
    wait(st, done_rest[nsub - 1]);  // the side stream's launches are ordered
  }
  for (int lv = (int)d.levels.size() - 1; lv >= 0 && ok; --lv) {
    const MFLevel& L = d.levels[lv];
    const int cnt = (int)L.nodes_by_k.size();
    const int nsub = (L.max_k + P - 1) / P;
    if (!look || nsub < 3 || cnt > kLookaheadFronts || !side) {
      for (int j = nsub - 1; j >= 0; --j) {
        const int na = active(L, j);
        dim3 g(bwd_width(L, j, na, 0, kAll), na);
        launch_pdl(bwd_gemv_kernel<S, false>, g, 256, 0, st, L.d_nodes, na, d.d_nodes, d.d_U, arena, x,
                                                      j, 0, kAll);
        trsv(L, j, na, false, st);
        n += 1;
      }
      continue;
    }
    evi = 0;
    std::vector<cudaEvent_t> solved(nsub, nullptr);
    cudaEvent_t start = ev();
    record(start, st);
    wait(side, start);
    for (int j = nsub - 1; j >= 0 && ok; --j) {
      // side: the columns solved two or more sub-steps ago (and the
      // ancestors'), beside the triangular solve of sub-step j + 1
      if (j + 2 < nsub) wait(side, solved[j + 2]);
      const int na = active(L, j);
      {
        dim3 g(bwd_width(L, j, na, P, kAll), na);
        launch_pdl(bwd_gemv_kernel<S, true>, g, 256, 0, side, L.d_nodes, na, d.d_nodes, d.d_U, arena, x,
                                                      j, P, kAll);
      }
      cudaEvent_t rest_done = ev();
      record(rest_done, side);
      // main: the columns of sub-step j + 1, just solved
      launch_pdl(bwd_gemv_kernel<S, true>, dim3(bwd_width(L, j, na, 0, P), na), 256, 0, st,
                 L.d_nodes, na, d.d_nodes, d.d_U, arena, x, j, 0, P);
      wait(st, rest_done);
      trsv(L, j, na, false, st);
      solved[j] = ev();
      record(solved[j], st);
      n += 2;
    }
  }
  return ok ? n : -1;
}

// one solve on d_x: the launch sequence is fixed by the symbolic structure
// and the device buffers, so it is captured once into a CUDA graph (on a
// private stream) and replayed into the caller's stream afterwards
template <typename S>
cudaError_t solve_t(MFHandle& h, cudaStream_t st) {
  MFDevice& d = h.dev;
  cudaError_t e = cudaSuccess;
  if (!d.solve_exec) {
    e = solve_prepare<S>();
    if (e != cudaSuccess) return e;
    if (!d.cap_stream) e = cudaStreamCreateWithFlags(&d.cap_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess && !d.cap_side) e = cudaStreamCreateWithFlags(&d.cap_side, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(d.cap_stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    const int n = solve_launches<S>(d, d.cap_stream);
    e = cudaStreamEndCapture(d.cap_stream, &g);
    if (e == cudaSuccess && n < 0) e = cudaErrorInvalidResourceHandle;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&d.solve_exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      d.solve_exec = nullptr;
      return e;
    }
    d.solve_n = n;
  }
  e = cudaGraphLaunch(d.solve_exec, st);
  count_launch(d.solve_n);
  return e;
}

template <typename S, typename T>
cudaError_t solve_io(MFHandle& h, const void* b, void* xout, cudaStream_t st) {
  const int64_t n = h.sym.n;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  permute_in_kernel<S, T><<<blocks, 256, 0, st>>>(n, h.dev.d_perm, (const T*)b, (S*)h.dev.d_x);
  cudaError_t e = solve_t<S>(h, st);
  if (e != cudaSuccess) return e;
  permute_out_kernel<S, T><<<blocks, 256, 0, st>>>(n, h.dev.d_perm, (const S*)h.dev.d_x, (T*)xout);
  count_launch(2);
  return cudaGetLastError();
}

}  // namespace

cudaError_t mf_factor(MFHandle& h, int dtype, const void* vals, double tau, cudaStream_t st) {
  cudaError_t e = setup_device(h, dtype);
  if (e != cudaSuccess) return e;
  switch (dtype) {
    case SUCEM_F32: e = factor_t<float>(h, vals, tau, st); break;
    case SUCEM_F64: e = factor_t<double>(h, vals, tau, st); break;
    case SUCEM_C64: e = factor_t<float2>(h, vals, tau, st); break;
    case SUCEM_C128: e = factor_t<double2>(h, vals, tau, st); break;
    default: return cudaErrorInvalidValue;
  }
  MFDevice& d = h.dev;
  if (e == cudaSuccess && !d.factor_ev) e = cudaEventCreateWithFlags(&d.factor_ev, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(d.factor_ev, st);
  d.factored = e == cudaSuccess;
  d.checked = false;
  d.valid = true;
  return e;
}

// waits for the last factorisation (once per factorisation) and reads its
// flags: 0 = usable, -1 = a bounded wait of its tensor-core update gave up
// (the factor is invalid), -2 = not factored / CUDA error
int mf_factor_status(MFHandle& h) {
  MFDevice& d = h.dev;
  if (!d.factored || !d.d_flag) return -2;
  if (!d.checked) {
    int v[2] = {0, 0};
    if (cudaEventSynchronize(d.factor_ev) != cudaSuccess ||
        cudaMemcpy(v, d.d_flag, sizeof(v), cudaMemcpyDeviceToHost) != cudaSuccess)
      return -2;
    d.perturbed = v[0];
    d.valid = v[1] == 0;
    d.checked = true;
  }
  return d.valid ? 0 : -1;
}

cudaError_t mf_mark_timed_out(MFHandle& h) {
  MFDevice& d = h.dev;
  if (!d.factored || !d.d_flag) return cudaErrorNotReady;
  const int one = 1;
  cudaError_t e = cudaEventSynchronize(d.factor_ev);
  if (e == cudaSuccess) e = cudaMemcpy(d.d_flag + 1, &one, sizeof(int), cudaMemcpyHostToDevice);
  d.checked = false;
  return e;
}

// b and x may have the factor's precision or the matching double precision
cudaError_t mf_solve(MFHandle& h, int io_dtype, const void* b, void* x, cudaStream_t st) {
  if (!h.dev.factored) return cudaErrorNotReady;
  const int f = h.dev.dtype;
  if (f == SUCEM_F32 && io_dtype == SUCEM_F32) return solve_io<float, float>(h, b, x, st);
  if (f == SUCEM_F32 && io_dtype == SUCEM_F64) return solve_io<float, double>(h, b, x, st);
  if (f == SUCEM_F64 && io_dtype == SUCEM_F64) return solve_io<double, double>(h, b, x, st);
  if (f == SUCEM_C64 && io_dtype == SUCEM_C64) return solve_io<float2, float2>(h, b, x, st);
  if (f == SUCEM_C64 && io_dtype == SUCEM_C128) return solve_io<float2, double2>(h, b, x, st);
  if (f == SUCEM_C128 && io_dtype == SUCEM_C128) return solve_io<double2, double2>(h, b, x, st);
  return cudaErrorInvalidValue;
}

int mf_perturbed(MFHandle& h) {
  const int st = mf_factor_status(h);
  if (st == -2) return 0;
  // d_flag[1]: a bounded wait of the tensor-core update gave up
  return st < 0 ? -1 : h.dev.perturbed;
}

// new plan parameters: the device state (arena, plan) is rebuilt at the
// next factorisation
cudaError_t mf_configure(MFHandle& h, int superpanel, int panel_k) {
  if (superpanel != 0 && (superpanel < kTcPanel || superpanel % kTcPanel != 0))
    return cudaErrorInvalidValue;
  if (panel_k < 0) return cudaErrorInvalidValue;
  if (superpanel == h.cfg_superpanel && panel_k == h.cfg_panel_k) return cudaSuccess;
  h.cfg_superpanel = superpanel;
  h.cfg_panel_k = panel_k;
  free_dev(h.dev);
  return cudaSuccess;
}

void mf_tc_stats(MFHandle& h, double* out) {
  MFDevice& d = h.dev;
  double ms = 0;
  for (int i = 0; i < d.tc_n; ++i) {
    float t = 0;
    if (cudaEventSynchronize(d.tc_ev[2 * i + 1]) == cudaSuccess &&
        cudaEventElapsedTime(&t, d.tc_ev[2 * i], d.tc_ev[2 * i + 1]) == cudaSuccess)
      ms += t;
  }
  out[0] = d.tc_n;
  out[1] = ms;
  out[2] = d.tc_flops;
}

void mf_free(MFHandle& h) { free_dev(h.dev); }

MFHandle* mf_new() { return new MFHandle(); }
void mf_delete(MFHandle* h) {
  if (!h) return;
  free_dev(h->dev);
  delete h;
}
MFSymbolic& mf_sym(MFHandle* h) { return h->sym; }

// the bounded-wait self-test (wait_selftest_kernel): *gave_up = 1 when the
// wait ran out as it must
cudaError_t mf_wait_selftest(int polls, int* gave_up) {
  int* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(int));
  if (e != cudaSuccess) return e;
  int h = -1;
  e = cudaMemcpy(d, &h, sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    wait_selftest_kernel<<<1, 32>>>(polls, d);
    count_launch(1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  *gave_up = h;
  return e;
}

}  // namespace sucem
