// Sparse linear-algebra kernels on the space's CSR pattern: essential-row
// treatment, SpMV (real / complex, single / double), linear combinations of
// value arrays and exact-zero compaction.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/sucem_gb300.h"
#include "device.h"
#include "linalg.h"
#include "handle.h"

namespace sucem {

int fail(const std::string& msg, int code);
int cuda_fail(cudaError_t e, const char* where);
void count_launch(int k);

namespace {

// ---- essential rows: zero the row, unit diagonal (DirichletBC.apply) ----
template <typename V>
__global__ void ident_rows_kernel(const int32_t* __restrict__ indptr,
                                  const int32_t* __restrict__ indices,
                                  const int32_t* __restrict__ rows, int64_t nrows, V* vals) {
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= nrows) return;
  const int r = rows[w];
  const int a = indptr[r], b = indptr[r + 1];
  for (int k = a + lane; k < b; k += 32) vals[k] = indices[k] == r ? V(1) : V(0);
}

template <typename R>
struct C2;
template <>
struct C2<float> {
  using T = float2;
};
template <>
struct C2<double> {
  using T = double2;
};

template <typename R>
__device__ __forceinline__ typename C2<R>::T cmul(typename C2<R>::T a, typename C2<R>::T b) {
  typename C2<R>::T z;
  z.x = a.x * b.x - a.y * b.y;
  z.y = a.x * b.y + a.y * b.x;
  return z;
}

// ---- SpMV: y = A x, TPR lanes per row, shuffle reduction ----
template <typename R, bool CPLX, int TPR>
__global__ void spmv_kernel(int64_t n, const int32_t* __restrict__ indptr,
                            const int32_t* __restrict__ indices, const void* __restrict__ vals_,
                            const void* __restrict__ x_, void* __restrict__ y_) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t row = tid / TPR;
  const int sub = threadIdx.x % TPR;
  // no early return: every lane of the warp takes part in the shuffles
  const bool valid = row < n;
  const int a = valid ? __ldg(&indptr[row]) : 0, b = valid ? __ldg(&indptr[row + 1]) : 0;
  if (!CPLX) {
    const R* vals = (const R*)vals_;
    const R* x = (const R*)x_;
    R acc = 0;
    for (int k = a + sub; k < b; k += TPR) acc += __ldg(&vals[k]) * __ldg(&x[__ldg(&indices[k])]);
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, TPR);
    if (valid && sub == 0) ((R*)y_)[row] = acc;
  } else {
    using CT = typename C2<R>::T;
    const CT* vals = (const CT*)vals_;
    const CT* x = (const CT*)x_;
    R ar = 0, ai = 0;
    for (int k = a + sub; k < b; k += TPR) {
      // the matrix streams through once (evict-first), x is gathered
      // through the read-only path
      const CT v = __ldcs(&vals[k]);
      const CT xv = __ldg(&x[__ldcs(&indices[k])]);
      ar += v.x * xv.x - v.y * xv.y;
      ai += v.x * xv.y + v.y * xv.x;
    }
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) {
      ar += __shfl_down_sync(0xffffffffu, ar, o, TPR);
      ai += __shfl_down_sync(0xffffffffu, ai, o, TPR);
    }
    if (valid && sub == 0) {
      CT z;
      z.x = ar;
      z.y = ai;
      ((CT*)y_)[row] = z;
    }
  }
}

template <typename R, bool CPLX>
cudaError_t spmv_dispatch(int64_t n, int64_t nnz, const int32_t* indptr, const int32_t* indices,
                          const void* vals, const void* x, void* y, cudaStream_t s) {
  const double mean = n ? (double)nnz / (double)n : 0.0;
  const int threads = 256;
#define LAUNCH(TPR)                                                                     \
  {                                                                                     \
    int64_t blocks = (n * TPR + threads - 1) / threads;                                 \
    spmv_kernel<R, CPLX, TPR><<<(unsigned)blocks, threads, 0, s>>>(n, indptr, indices, \
                                                                    vals, x, y);        \
    return cudaGetLastError();                                                          \
  }
  if (mean <= 12) LAUNCH(4);
  // complex double: 8 lanes per row measured faster than 16 on the 20^3
  // order-2 matrix (42.5 entries per row: 0.213 against 0.266 ms)
  if (mean <= 24 || (CPLX && sizeof(R) == 8 && mean <= 56)) LAUNCH(8);
  if (mean <= 56) LAUNCH(16);
  LAUNCH(32);
#undef LAUNCH
}

// ---- linear combination of value arrays ----
// real out:    out = a*X + b*Y
// complex out: out = (a*X + b*Y) + j*(c*Z)
template <typename R>
__global__ void combine_kernel(int64_t m, R a, const R* __restrict__ X, R b,
                               const R* __restrict__ Y, R c, const R* __restrict__ Z, R* out,
                               int cplx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  R re = (X ? a * X[i] : R(0)) + (Y ? b * Y[i] : R(0));
  if (cplx) {
    out[2 * i] = re;
    out[2 * i + 1] = Z ? c * Z[i] : R(0);
  } else {
    out[i] = re;
  }
}

// ---- exact-zero compaction of a complex CSR (scipy binop semantics) ----
template <typename R>
__global__ void count_nonzero_kernel(int64_t n, const int32_t* __restrict__ indptr,
                                     const R* __restrict__ vals, int32_t* __restrict__ counts) {
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= n) return;
  const int a = indptr[w], b = indptr[w + 1];
  int c = 0;
  for (int k = a + lane; k < b; k += 32) c += (vals[2 * k] != R(0) || vals[2 * k + 1] != R(0));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if (lane == 0) counts[w] = c;
}

// single-block exclusive scan over n counts -> out_indptr[0..n]
__global__ void scan_kernel(int64_t n, const int32_t* __restrict__ counts,
                            int32_t* __restrict__ out_indptr) {
  __shared__ int32_t part[1024];
  const int t = threadIdx.x;
  const int64_t chunk = (n + blockDim.x - 1) / blockDim.x;
  const int64_t lo = t * chunk, hi = lo + chunk < n ? lo + chunk : n;
  int32_t s = 0;
  for (int64_t i = lo; i < hi; ++i) s += counts[i];
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    int32_t run = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      int32_t v = part[i];
      part[i] = run;
      run += v;
    }
    out_indptr[n] = run;
  }
  __syncthreads();
  int32_t run = part[t];
  for (int64_t i = lo; i < hi; ++i) {
    out_indptr[i] = run;
    run += counts[i];
  }
}

template <typename R>
__global__ void compact_kernel(int64_t n, const int32_t* __restrict__ indptr,
                               const int32_t* __restrict__ indices, const R* __restrict__ vals,
                               const int32_t* __restrict__ out_indptr, int32_t* out_indices,
                               R* out_vals) {
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= n) return;
  const int a = indptr[w], b = indptr[w + 1];
  int base = out_indptr[w];
  for (int k0 = a; k0 < b; k0 += 32) {
    const int k = k0 + lane;
    const bool keep = k < b && (vals[2 * k] != R(0) || vals[2 * k + 1] != R(0));
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) {
      const int pos = base + __popc(m & ((1u << lane) - 1u));
      out_indices[pos] = indices[k];
      out_vals[2 * pos] = vals[2 * k];
      out_vals[2 * pos + 1] = vals[2 * k + 1];
    }
    base += __popc(m);
  }
}

// ---- vector kernels ----
template <typename R, bool CPLX>
__global__ void axpby_kernel(int64_t n, double ar, double ai, const R* __restrict__ x, double br,
                             double bi, R* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!CPLX) {
    const double xv = x ? (double)x[i] : 0.0;
    const double yv = br != 0.0 ? (double)y[i] : 0.0;
    y[i] = (R)(ar * xv + br * yv);
  } else {
    const double xr = x ? (double)x[2 * i] : 0.0, xi = x ? (double)x[2 * i + 1] : 0.0;
    double yr = 0, yi = 0;
    if (br != 0.0 || bi != 0.0) {
      yr = (double)y[2 * i];
      yi = (double)y[2 * i + 1];
    }
    y[2 * i] = (R)(ar * xr - ai * xi + br * yr - bi * yi);
    y[2 * i + 1] = (R)(ar * xi + ai * xr + br * yi + bi * yr);
  }
}

// partial sums of conj(x).y (or x.y) per block, in double precision
template <typename R, bool CPLX>
__global__ void dot_partial_kernel(int64_t n, const R* __restrict__ x, const R* __restrict__ y,
                                   int conj, double2* __restrict__ partial) {
  __shared__ double sr[32], si[32];
  double ar = 0, ai = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (!CPLX) {
      ar += (double)x[i] * (double)y[i];
    } else {
      const double xr = x[2 * i], xi = conj ? -(double)x[2 * i + 1] : (double)x[2 * i + 1];
      const double yr = y[2 * i], yi = y[2 * i + 1];
      ar += xr * yr - xi * yi;
      ai += xr * yi + xi * yr;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    ar += __shfl_down_sync(~0u, ar, o);
    ai += __shfl_down_sync(~0u, ai, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sr[w] = ar;
    si[w] = ai;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    ar = l < nw ? sr[l] : 0.0;
    ai = l < nw ? si[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      ar += __shfl_down_sync(~0u, ar, o);
      ai += __shfl_down_sync(~0u, ai, o);
    }
    if (l == 0) partial[blockIdx.x] = make_double2(ar, ai);
  }
}

// fixed-order sum of the block partials (deterministic)
__global__ void dot_final_kernel(int nparts, const double2* __restrict__ partial,
                                 double2* __restrict__ out) {
  __shared__ double sr[32], si[32];
  double ar = 0, ai = 0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    ar += partial[i].x;
    ai += partial[i].y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    ar += __shfl_down_sync(~0u, ar, o);
    ai += __shfl_down_sync(~0u, ai, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sr[w] = ar;
    si[w] = ai;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    ar = l < nw ? sr[l] : 0.0;
    ai = l < nw ? si[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      ar += __shfl_down_sync(~0u, ar, o);
      ai += __shfl_down_sync(~0u, ai, o);
    }
    if (l == 0) *out = make_double2(ar, ai);
  }
}

// ---- block Gram-Schmidt of FGMRES (vec_gs) ----
// partial[b * k + i] = sum over block b's grid-stride slice of conj(V_i) w
// (V_i = V + i * ldv), one basis vector after the other (w is re-read from
// L2), each block reduced in a fixed order
template <typename R, bool CPLX>
__global__ void multidot_partial_kernel(int64_t n, const R* __restrict__ V, int64_t ldv, int k,
                                        const R* __restrict__ w, double2* __restrict__ partial) {
  __shared__ double sr[32], si[32];
  const int wi = threadIdx.x >> 5, l = threadIdx.x & 31;
  for (int i = 0; i < k; ++i) {
    const R* v = V + (CPLX ? 2 : 1) * (int64_t)i * ldv;
    double ar = 0, ai = 0;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
      if (!CPLX) {
        ar += (double)v[e] * (double)w[e];
      } else {
        const double vr = v[2 * e], vi = -(double)v[2 * e + 1];
        const double wr = w[2 * e], wim = w[2 * e + 1];
        ar += vr * wr - vi * wim;
        ai += vr * wim + vi * wr;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      ar += __shfl_down_sync(~0u, ar, o);
      ai += __shfl_down_sync(~0u, ai, o);
    }
    if (l == 0) {
      sr[wi] = ar;
      si[wi] = ai;
    }
    __syncthreads();
    if (wi == 0) {
      const int nw = blockDim.x >> 5;
      ar = l < nw ? sr[l] : 0.0;
      ai = l < nw ? si[l] : 0.0;
      for (int o = 16; o > 0; o >>= 1) {
        ar += __shfl_down_sync(~0u, ar, o);
        ai += __shfl_down_sync(~0u, ai, o);
      }
      if (l == 0) partial[(int64_t)blockIdx.x * k + i] = make_double2(ar, ai);
    }
    __syncthreads();
  }
}

// h[i] (+)= sum_b partial[b * k + i]: block i, a fixed-order tree over the
// blocks' partials (deterministic)
__global__ void multidot_final_kernel(int nparts, int k, const double2* __restrict__ partial,
                                      double2* __restrict__ h, int accumulate) {
  __shared__ double sr[32], si[32];
  const int i = blockIdx.x;
  if (i >= k) return;
  double ar = 0, ai = 0;
  for (int b = threadIdx.x; b < nparts; b += blockDim.x) {
    ar += partial[(int64_t)b * k + i].x;
    ai += partial[(int64_t)b * k + i].y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    ar += __shfl_down_sync(~0u, ar, o);
    ai += __shfl_down_sync(~0u, ai, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sr[w] = ar;
    si[w] = ai;
  }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    ar = l < nw ? sr[l] : 0.0;
    ai = l < nw ? si[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      ar += __shfl_down_sync(~0u, ar, o);
      ai += __shfl_down_sync(~0u, ai, o);
    }
    if (l == 0) {
      if (accumulate) {
        h[i].x += ar;
        h[i].y += ai;
      } else {
        h[i] = make_double2(ar, ai);
      }
    }
  }
}

// w -= sum_i c[i] V_i with the coefficients c = h (device memory)
template <typename R, bool CPLX>
__global__ void multiaxpy_kernel(int64_t n, const R* __restrict__ V, int64_t ldv, int k,
                                 const double2* __restrict__ c, R* __restrict__ w) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (!CPLX) {
      double acc = w[e];
      for (int i = 0; i < k; ++i) acc -= c[i].x * (double)V[(int64_t)i * ldv + e];
      w[e] = (R)acc;
    } else {
      double ar = w[2 * e], ai = w[2 * e + 1];
      for (int i = 0; i < k; ++i) {
        const R* v = V + 2 * (int64_t)i * ldv;
        const double vr = v[2 * e], vi = v[2 * e + 1];
        ar -= c[i].x * vr - c[i].y * vi;
        ai -= c[i].x * vi + c[i].y * vr;
      }
      w[2 * e] = (R)ar;
      w[2 * e + 1] = (R)ai;
    }
  }
}

constexpr int kGsBlocks = 256;

// classical Gram-Schmidt with one reorthogonalisation of w against the k
// basis vectors V_i (rows of V, leading dimension ldv elements), all on
// the device: h[0:k] = the two passes' coefficients summed, h[k].x = |w|^2
// after both.  work: kGsBlocks * (k + 1) double2 partials.
template <typename R, bool CPLX>
cudaError_t gs_t(int64_t n, const R* V, int64_t ldv, int k, R* w, double2* work, double2* h,
                 cudaStream_t s) {
  const int threads = 256;
  const unsigned blocks = (unsigned)std::min<int64_t>(kGsBlocks * 4, (n + threads - 1) / threads);
  for (int pass = 0; pass < 2 && k > 0; ++pass) {
    multidot_partial_kernel<R, CPLX><<<kGsBlocks, threads, 0, s>>>(n, V, ldv, k, w, work);
    multidot_final_kernel<<<k, 256, 0, s>>>(kGsBlocks, k, work, h, pass);
    // the second pass subtracts only its own coefficients: they follow
    // h's first-pass values in work's tail, so reduce them there first
    if (pass == 0) {
      multiaxpy_kernel<R, CPLX><<<blocks, threads, 0, s>>>(n, V, ldv, k, h, w);
    } else {
      multidot_final_kernel<<<k, 256, 0, s>>>(kGsBlocks, k, work, work + (int64_t)kGsBlocks * k, 0);
      multiaxpy_kernel<R, CPLX><<<blocks, threads, 0, s>>>(n, V, ldv, k, work + (int64_t)kGsBlocks * k, w);
    }
  }
  multidot_partial_kernel<R, CPLX><<<kGsBlocks, threads, 0, s>>>(n, w, 0, 1, w, work);
  multidot_final_kernel<<<1, 256, 0, s>>>(kGsBlocks, 1, work, h + k, 0);
  return cudaGetLastError();
}

// segmented dot products of real double vectors: out[s] = sum_{i in seg s} x_i y_i
// one block per segment, fixed-order reduction
__global__ void seg_dot_kernel(int nseg, const int64_t* __restrict__ seg, const double* __restrict__ x,
                               const double* __restrict__ y, int64_t ldx, int nvec,
                               double* __restrict__ out) {
  // blockIdx.x = segment, blockIdx.y = vector index j: out[j*nseg + s] = x_j . y
  __shared__ double sh[32];
  const int s = blockIdx.x, j = blockIdx.y;
  if (s >= nseg || j >= nvec) return;
  const double* xj = x + (int64_t)j * ldx;
  double a = 0;
  for (int64_t i = seg[s] + threadIdx.x; i < seg[s + 1]; i += blockDim.x) a += xj[i] * y[i];
  for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(~0u, a, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = a;
  __syncthreads();
  if (w == 0) {
    a = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(~0u, a, o);
    if (l == 0) out[(int64_t)j * nseg + s] = a;
  }
}

// y_i = b[s] * y_i + sum_j a[j*nseg + s] * x_j,i for i in segment s
__global__ void seg_axpy_kernel(int nseg, const int64_t* __restrict__ seg, int64_t n,
                                const int32_t* __restrict__ seg_of, const double* __restrict__ x,
                                int64_t ldx, int nvec, const double* __restrict__ a,
                                const double* __restrict__ b, double* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = seg_of[i];
  double v = b ? b[s] * y[i] : y[i];
  for (int j = 0; j < nvec; ++j) v += a[(int64_t)j * nseg + s] * x[(int64_t)j * ldx + i];
  y[i] = v;
}

// dst[i] = src[idx[i]] for 8-byte or 16-byte elements
template <typename T>
__global__ void gather_kernel(int64_t m, const int64_t* __restrict__ idx, const T* __restrict__ src,
                              T* __restrict__ dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) dst[i] = src[idx[i]];
}

template <typename D, typename S>
__global__ void convert_kernel(int64_t m, const S* __restrict__ src, D* __restrict__ dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) dst[i] = (D)src[i];
}

}  // namespace

constexpr int kDotBlocks = 512;

cudaError_t vec_dot(int64_t n, int dtype, const void* x, const void* y, int conj,
                    double2* partial, double2* out, cudaStream_t s) {
  const int threads = 256;
  switch (dtype) {
    case SUCEM_F32:
      dot_partial_kernel<float, false><<<kDotBlocks, threads, 0, s>>>(n, (const float*)x, (const float*)y, conj, partial);
      break;
    case SUCEM_F64:
      dot_partial_kernel<double, false><<<kDotBlocks, threads, 0, s>>>(n, (const double*)x, (const double*)y, conj, partial);
      break;
    case SUCEM_C64:
      dot_partial_kernel<float, true><<<kDotBlocks, threads, 0, s>>>(n, (const float*)x, (const float*)y, conj, partial);
      break;
    case SUCEM_C128:
      dot_partial_kernel<double, true><<<kDotBlocks, threads, 0, s>>>(n, (const double*)x, (const double*)y, conj, partial);
      break;
    default: return cudaErrorInvalidValue;
  }
  dot_final_kernel<<<1, 256, 0, s>>>(kDotBlocks, partial, out);
  return cudaGetLastError();
}

cudaError_t spmv(const DeviceSpace& d, int dtype, const void* vals, const void* x, void* y,
                 cudaStream_t s) {
  return spmv_raw(d.n, d.nnz, d.indptr, d.indices, dtype, vals, x, y, s);
}

cudaError_t spmv_raw(int64_t n, int64_t nnz, const int32_t* indptr, const int32_t* indices,
                     int dtype, const void* vals, const void* x, void* y, cudaStream_t s) {
  switch (dtype) {
    case SUCEM_F32: return spmv_dispatch<float, false>(n, nnz, indptr, indices, vals, x, y, s);
    case SUCEM_F64: return spmv_dispatch<double, false>(n, nnz, indptr, indices, vals, x, y, s);
    case SUCEM_C64: return spmv_dispatch<float, true>(n, nnz, indptr, indices, vals, x, y, s);
    case SUCEM_C128: return spmv_dispatch<double, true>(n, nnz, indptr, indices, vals, x, y, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace sucem

using sucem::fail;
using sucem::cuda_fail;

static const sucem::DeviceSpace* dev_of(const sucem_space* sp) {
  return sp ? sp->s.dev : nullptr;
}

extern "C" {

int sucem_apply_essential(const sucem_space* sp, int dtype, void* vals, const int32_t* rows,
                          int64_t nrows, void* stream) {
  const sucem::DeviceSpace* d = dev_of(sp);
  if (!d) return fail("space is not on a device", SUCEM_ERR_STATE);
  if (nrows == 0) return SUCEM_OK;
  if (!vals || !rows) return fail("null argument", SUCEM_ERR_ARG);
  const int threads = 256;
  const unsigned blocks = (unsigned)((nrows * 32 + threads - 1) / threads);
  cudaStream_t s = (cudaStream_t)stream;
  switch (dtype) {
    case SUCEM_F32:
      sucem::ident_rows_kernel<float><<<blocks, threads, 0, s>>>(d->indptr, d->indices, rows, nrows,
                                                                 (float*)vals);
      break;
    case SUCEM_F64:
      sucem::ident_rows_kernel<double><<<blocks, threads, 0, s>>>(d->indptr, d->indices, rows,
                                                                  nrows, (double*)vals);
      break;
    default: return fail("essential rows: dtype must be F32 or F64", SUCEM_ERR_ARG);
  }
  cudaError_t e = cudaGetLastError();
  sucem::count_launch(1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_apply_essential");
}

int sucem_spmv(const sucem_space* sp, int dtype, const void* vals, const void* x, void* y,
               void* stream) {
  const sucem::DeviceSpace* d = dev_of(sp);
  if (!d) return fail("space is not on a device", SUCEM_ERR_STATE);
  if (!vals || !x || !y) return fail("null argument", SUCEM_ERR_ARG);
  cudaError_t e = sucem::spmv(*d, dtype, vals, x, y, (cudaStream_t)stream);
  sucem::count_launch(1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_spmv");
}

int sucem_spmv_csr(int64_t n, int64_t nnz, const int32_t* indptr, const int32_t* indices,
                   int dtype, const void* vals, const void* x, void* y, void* stream) {
  if (!indptr || !indices || !vals || !x || !y) return fail("null argument", SUCEM_ERR_ARG);
  cudaError_t e = sucem::spmv_raw(n, nnz, indptr, indices, dtype, vals, x, y, (cudaStream_t)stream);
  sucem::count_launch(1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_spmv_csr");
}

int sucem_vec_axpby(int64_t n, int dtype, double ar, double ai, const void* x, double br,
                    double bi, void* y, void* stream) {
  if (!y) return fail("null output", SUCEM_ERR_ARG);
  if (n == 0) return SUCEM_OK;
  const int threads = 256;
  const unsigned blocks = (unsigned)((n + threads - 1) / threads);
  cudaStream_t s = (cudaStream_t)stream;
  switch (dtype) {
    case SUCEM_F32:
      sucem::axpby_kernel<float, false><<<blocks, threads, 0, s>>>(n, ar, ai, (const float*)x, br, bi, (float*)y);
      break;
    case SUCEM_F64:
      sucem::axpby_kernel<double, false><<<blocks, threads, 0, s>>>(n, ar, ai, (const double*)x, br, bi, (double*)y);
      break;
    case SUCEM_C64:
      sucem::axpby_kernel<float, true><<<blocks, threads, 0, s>>>(n, ar, ai, (const float*)x, br, bi, (float*)y);
      break;
    case SUCEM_C128:
      sucem::axpby_kernel<double, true><<<blocks, threads, 0, s>>>(n, ar, ai, (const double*)x, br, bi, (double*)y);
      break;
    default: return fail("bad dtype", SUCEM_ERR_ARG);
  }
  cudaError_t e = cudaGetLastError();
  sucem::count_launch(1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_vec_axpby");
}

int64_t sucem_vec_dot_work_bytes(void) { return (int64_t)sucem::kDotBlocks * 16; }

int64_t sucem_vec_gs_work_bytes(int k) {
  return (int64_t)sucem::kGsBlocks * (k + 1) * 16 + (int64_t)(k + 1) * 16;
}

int sucem_vec_gs(int64_t n, int dtype, const void* V, int64_t ldv, int k, void* w, void* work,
                 double* h, void* stream) {
  if (!w || !work || !h || (k > 0 && !V)) return fail("null argument", SUCEM_ERR_ARG);
  if (k < 0 || k > 63 || ldv < n) return fail("0 <= k <= 63 and ldv >= n required", SUCEM_ERR_ARG);
  cudaStream_t s = (cudaStream_t)stream;
  double2* wk = (double2*)work;
  double2* hh = (double2*)h;
  cudaError_t e;
  switch (dtype) {
    case SUCEM_F64: e = sucem::gs_t<double, false>(n, (const double*)V, ldv, k, (double*)w, wk, hh, s); break;
    case SUCEM_C128: e = sucem::gs_t<double, true>(n, (const double*)V, ldv, k, (double*)w, wk, hh, s); break;
    default: return fail("block Gram-Schmidt: dtype must be F64 or C128", SUCEM_ERR_ARG);
  }
  sucem::count_launch(k > 0 ? 9 : 2);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_vec_gs");
}

int sucem_vec_dot(int64_t n, int dtype, const void* x, const void* y, int conj, void* work,
                  double* out, void* stream) {
  if (!x || !y || !work || !out) return fail("null argument", SUCEM_ERR_ARG);
  cudaError_t e = sucem::vec_dot(n, dtype, x, y, conj, (double2*)work, (double2*)out,
                                 (cudaStream_t)stream);
  sucem::count_launch(2);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_vec_dot");
}

int sucem_gather(int64_t m, int elem_bytes, const int64_t* idx, const void* src, void* dst,
                 void* stream) {
  if (!idx || !src || !dst) return fail("null argument", SUCEM_ERR_ARG);
  if (m == 0) return SUCEM_OK;
  const unsigned blocks = (unsigned)((m + 255) / 256);
  cudaStream_t s = (cudaStream_t)stream;
  if (elem_bytes == 4)
    sucem::gather_kernel<float><<<blocks, 256, 0, s>>>(m, idx, (const float*)src, (float*)dst);
  else if (elem_bytes == 8)
    sucem::gather_kernel<double><<<blocks, 256, 0, s>>>(m, idx, (const double*)src, (double*)dst);
  else if (elem_bytes == 16)
    sucem::gather_kernel<double2><<<blocks, 256, 0, s>>>(m, idx, (const double2*)src, (double2*)dst);
  else
    return fail("element size must be 4, 8 or 16 bytes", SUCEM_ERR_ARG);
  cudaError_t e = cudaGetLastError();
  sucem::count_launch(1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_gather");
}

int sucem_seg_dot(int nseg, const int64_t* seg_ptr, const double* X, int64_t ldx, int nvec,
                  const double* y, double* out, void* stream) {
  if (!seg_ptr || !X || !y || !out) return fail("null argument", SUCEM_ERR_ARG);
  if (nseg <= 0 || nvec <= 0) return SUCEM_OK;
  if (nvec > 65535) return fail("too many vectors", SUCEM_ERR_ARG);
  dim3 grid((unsigned)nseg, (unsigned)nvec);
  sucem::seg_dot_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(nseg, seg_ptr, X, y, ldx, nvec, out);
  cudaError_t e = cudaGetLastError();
  sucem::count_launch(1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_seg_dot");
}

int sucem_seg_axpy(int nseg, const int64_t* seg_ptr, int64_t n, const int32_t* seg_of,
                   const double* X, int64_t ldx, int nvec, const double* a, const double* b,
                   double* y, void* stream) {
  if (!seg_ptr || !seg_of || !y || (nvec > 0 && (!X || !a))) return fail("null argument", SUCEM_ERR_ARG);
  if (n == 0) return SUCEM_OK;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  sucem::seg_axpy_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(nseg, seg_ptr, n, seg_of, X, ldx,
                                                                   nvec, a, b, y);
  cudaError_t e = cudaGetLastError();
  sucem::count_launch(1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_seg_axpy");
}

int sucem_vec_convert(int64_t count, int dst_real_bytes, void* dst, int src_real_bytes,
                      const void* src, void* stream) {
  if (!dst || !src) return fail("null argument", SUCEM_ERR_ARG);
  if (count == 0) return SUCEM_OK;
  const int threads = 256;
  const unsigned blocks = (unsigned)((count + threads - 1) / threads);
  cudaStream_t s = (cudaStream_t)stream;
  if (dst_real_bytes == 4 && src_real_bytes == 8)
    sucem::convert_kernel<float, double><<<blocks, threads, 0, s>>>(count, (const double*)src, (float*)dst);
  else if (dst_real_bytes == 8 && src_real_bytes == 4)
    sucem::convert_kernel<double, float><<<blocks, threads, 0, s>>>(count, (const float*)src, (double*)dst);
  else if (dst_real_bytes == src_real_bytes)
    return cudaMemcpyAsync(dst, src, count * dst_real_bytes, cudaMemcpyDeviceToDevice, s) == cudaSuccess
               ? SUCEM_OK
               : fail("copy failed", SUCEM_ERR_CUDA);
  else
    return fail("real sizes must be 4 or 8", SUCEM_ERR_ARG);
  cudaError_t e = cudaGetLastError();
  sucem::count_launch(1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_vec_convert");
}

int sucem_combine(int64_t m, int real_bytes, double a, const void* X, double b, const void* Y,
                  double c, const void* Z, void* out, int complex_out, void* stream) {
  if (!out) return fail("null output", SUCEM_ERR_ARG);
  if (m == 0) return SUCEM_OK;
  const int threads = 256;
  const unsigned blocks = (unsigned)((m + threads - 1) / threads);
  cudaStream_t s = (cudaStream_t)stream;
  if (real_bytes == 4)
    sucem::combine_kernel<float><<<blocks, threads, 0, s>>>(m, (float)a, (const float*)X, (float)b,
                                                            (const float*)Y, (float)c,
                                                            (const float*)Z, (float*)out,
                                                            complex_out);
  else if (real_bytes == 8)
    sucem::combine_kernel<double><<<blocks, threads, 0, s>>>(m, a, (const double*)X, b,
                                                             (const double*)Y, c,
                                                             (const double*)Z, (double*)out,
                                                             complex_out);
  else
    return fail("real_bytes must be 4 or 8", SUCEM_ERR_ARG);
  cudaError_t e = cudaGetLastError();
  sucem::count_launch(1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_combine");
}

int sucem_compact_count(const sucem_space* sp, int dtype, const void* vals, int32_t* out_indptr,
                        int32_t* work, void* stream) {
  const sucem::DeviceSpace* d = dev_of(sp);
  if (!d) return fail("space is not on a device", SUCEM_ERR_STATE);
  if (!vals || !out_indptr || !work) return fail("null argument", SUCEM_ERR_ARG);
  if (dtype != SUCEM_C64 && dtype != SUCEM_C128)
    return fail("compaction needs a complex dtype", SUCEM_ERR_ARG);
  cudaStream_t s = (cudaStream_t)stream;
  const int threads = 256;
  const unsigned blocks = (unsigned)((d->n * 32 + threads - 1) / threads);
  // no rows: no count launch (a zero-block grid is a launch error); the
  // scan still writes out_indptr[0] = 0
  if (d->n > 0 && dtype == SUCEM_C64)
    sucem::count_nonzero_kernel<float><<<blocks, threads, 0, s>>>(d->n, d->indptr,
                                                                  (const float*)vals, work);
  else if (d->n > 0)
    sucem::count_nonzero_kernel<double><<<blocks, threads, 0, s>>>(d->n, d->indptr,
                                                                   (const double*)vals, work);
  sucem::scan_kernel<<<1, 1024, 0, s>>>(d->n, work, out_indptr);
  cudaError_t e = cudaGetLastError();
  sucem::count_launch(d->n > 0 ? 2 : 1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_compact_count");
}

int sucem_compact_fill(const sucem_space* sp, int dtype, const void* vals,
                       const int32_t* out_indptr, int32_t* out_indices, void* out_vals,
                       void* stream) {
  const sucem::DeviceSpace* d = dev_of(sp);
  if (!d) return fail("space is not on a device", SUCEM_ERR_STATE);
  if (d->n == 0) return SUCEM_OK;  // nothing to fill
  cudaStream_t s = (cudaStream_t)stream;
  const int threads = 256;
  const unsigned blocks = (unsigned)((d->n * 32 + threads - 1) / threads);
  if (dtype == SUCEM_C64)
    sucem::compact_kernel<float><<<blocks, threads, 0, s>>>(d->n, d->indptr, d->indices,
                                                            (const float*)vals, out_indptr,
                                                            out_indices, (float*)out_vals);
  else if (dtype == SUCEM_C128)
    sucem::compact_kernel<double><<<blocks, threads, 0, s>>>(d->n, d->indptr, d->indices,
                                                             (const double*)vals, out_indptr,
                                                             out_indices, (double*)out_vals);
  else
    return fail("compaction needs a complex dtype", SUCEM_ERR_ARG);
  cudaError_t e = cudaGetLastError();
  sucem::count_launch(1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_compact_fill");
}

}  // extern "C"

// ---- allocation-free variant of the compaction count --------------------
// Some callers of this library cannot allocate device memory at the moment
// they need a compaction: a serving loop that reserved its whole HBM budget
// up front for resident problems, or a host that lets another allocator own
// the device memory.  For them the per-row count scratch of
// sucem_compact_count lives in this fixed device array instead of a
// caller-provided buffer.  Every GPU that loads the library holds it until
// the process exits.
namespace sucem {
namespace {

constexpr int64_t kNoAllocMaxRows = int64_t(1) << 20;  // 4 MiB of int32 counts
static __device__ __align__(256) int32_t g_noalloc_counts[kNoAllocMaxRows];

constexpr int kMaxDevices = 64;
int32_t* g_noalloc_ptr[kMaxDevices] = {nullptr};
std::mutex g_noalloc_mutex;

// Device address of the array for the current device.  In host code the
// array's name is only a host-side stand-in, so the address must come from
// cudaGetSymbolAddress, looked up once per device with that device current.
// The cached address is not refreshed after cudaDeviceReset: a process that
// resets a device must not call the allocation-free entry point on it again.
int noalloc_scratch(int32_t** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "sucem_compact_count_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail("device index out of range", SUCEM_ERR_ARG);
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_counts);
    if (e != cudaSuccess) return cuda_fail(e, "sucem_compact_count_noalloc: cudaGetSymbolAddress");
    g_noalloc_ptr[dev] = static_cast<int32_t*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return SUCEM_OK;
}

}  // namespace
}  // namespace sucem

extern "C" int sucem_compact_count_noalloc(const sucem_space* sp, int dtype, const void* vals,
                                           int32_t* out_indptr, void* stream) {
  const sucem::DeviceSpace* d = dev_of(sp);
  if (!d) return fail("space is not on a device", SUCEM_ERR_STATE);
  if (!vals || !out_indptr) return fail("null argument", SUCEM_ERR_ARG);
  if (dtype != SUCEM_C64 && dtype != SUCEM_C128)
    return fail("compaction needs a complex dtype", SUCEM_ERR_ARG);
  if (d->n > sucem::kNoAllocMaxRows)
    return fail("sucem_compact_count_noalloc: the matrix has " + std::to_string(d->n) +
                    " rows; the allocation-free scratch holds at most " +
                    std::to_string(sucem::kNoAllocMaxRows) +
                    " (use sucem_compact_count with a caller buffer)",
                SUCEM_ERR_ARG);
  int32_t* counts = nullptr;
  int rc = sucem::noalloc_scratch(&counts);
  if (rc != SUCEM_OK) return rc;
  // the count kernel writes counts[0, n) before the scan reads them, so the
  // contents left by an earlier call need no clearing
  cudaStream_t s = (cudaStream_t)stream;
  const int threads = 256;
  const unsigned blocks = (unsigned)((d->n * 32 + threads - 1) / threads);
  // no rows: skip the count launch (a zero-block grid is a launch error);
  // the scan still writes out_indptr[0] = 0
  if (d->n > 0 && dtype == SUCEM_C64)
    sucem::count_nonzero_kernel<float><<<blocks, threads, 0, s>>>(d->n, d->indptr,
                                                                  (const float*)vals, counts);
  else if (d->n > 0)
    sucem::count_nonzero_kernel<double><<<blocks, threads, 0, s>>>(d->n, d->indptr,
                                                                   (const double*)vals, counts);
  sucem::scan_kernel<<<1, 1024, 0, s>>>(d->n, counts, out_indptr);
  cudaError_t e = cudaGetLastError();
  sucem::count_launch(d->n > 0 ? 2 : 1);
  return e == cudaSuccess ? SUCEM_OK : cuda_fail(e, "sucem_compact_count_noalloc");
}
