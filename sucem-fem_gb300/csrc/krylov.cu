// Preconditioned BiCGStab with every scalar on the device: the GPU
// replacement of the reference's BiCGStabSolver
// (sucemfem/Utilities/LinalgSolvers.py:239-248, scipy.sparse.linalg.bicgstab
// with a spilu or diagonal preconditioner set at :107-127).
//
// One iteration (right preconditioning, M^-1 = none, the inverse diagonal,
// or an LU solve):
//   I1  beta = (rho_new / rho)(alpha / omega); p = r + beta (p - omega v);
//       phat = M^-1 p                       (rho_new from the partials of I5)
//   I2  v = A phat; partials of (rhat, v)
//   I3  alpha = rho_new / (rhat, v); s = r - alpha v (in r); shat = M^-1 s
//   I4  t = A shat; partials of (t, s), (t, t)
//   I5  omega = (t, s) / (t, t); x += alpha phat + omega shat; r = s - omega t;
//       partials of (rhat, r), (r, r)
//   I6  one block: the status word (converged, breakdown, iteration limit)
// Dot products: every block of a fixed grid writes a partial sum (double
// precision, complex) in a fixed order; the kernel that needs the value
// adds the partials itself, so no scalar ever goes to the host and the
// results are bit-reproducible.  Scalars are written only by kernels that
// run after every reader of the old value.  Every kernel returns at once
// when the status word is set, so a CUDA graph of `batch` iterations
// early-exits after convergence; without an LU preconditioner the batch is
// captured once and replayed, and the host reads the status word once per
// batch.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/sucem_gb300.h"

namespace sucem {
int fail(const std::string& msg, int code);
int cuda_fail(cudaError_t e, const char* where);
void count_launch(int k);

namespace {

constexpr int kThreads = 256;
constexpr int kNP = 6;  // partial sums: (rhat,r) (r,r) (rhat,v) (t,s) (t,t) (b,b)
enum { P_RHR = 0, P_RR = 1, P_RHV = 2, P_TS = 3, P_TT = 4, P_BB = 5 };
// device scalars (double2 each): rho, alpha, omega, then counters
enum { SC_RHO = 0, SC_ALPHA = 1, SC_OMEGA = 2, SC_N = 4 };
// status word: [0] state (0 running, 1 converged, 2 iteration limit, -1
// breakdown rho = 0, -2 breakdown omega = 0), [1] iterations done
struct KState {
  double2* sc;
  double2* part;  // [kNP][nb]
  int* status;
  int nb;
};

template <typename T>
struct CT;
template <>
struct CT<float> {
  using V = float2;
};
template <>
struct CT<double> {
  using V = double2;
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
// conj(a) * b
__device__ __forceinline__ double2 cdotc(double2 a, double2 b) {
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
template <typename V>
__device__ __forceinline__ double2 ld(const V* p, int64_t i) {
  const V v = p[i];
  return make_double2((double)v.x, (double)v.y);
}
template <typename V>
__device__ __forceinline__ void st(V* p, int64_t i, double2 z) {
  V v;
  v.x = z.x;
  v.y = z.y;
  p[i] = v;
}

// block-wide sum of a double2 (all threads call; result valid in thread 0)
__device__ __forceinline__ double2 block_sum(double2 v, double2* sh) {
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, o);
    v.y += __shfl_down_sync(0xffffffffu, v.y, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double2 s = make_double2(0.0, 0.0);
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      s.x += sh[i].x;
      s.y += sh[i].y;
    }
  return s;
}

// the sum of partial set q, in a fixed order (every thread gets it)
__device__ __forceinline__ double2 reduce_part(const KState& k, int q, double2* sh) {
  double2 v = make_double2(0.0, 0.0);
  for (int i = threadIdx.x; i < k.nb; i += blockDim.x) {
    v.x += k.part[q * k.nb + i].x;
    v.y += k.part[q * k.nb + i].y;
  }
  const double2 s = block_sum(v, sh);
  __syncthreads();
  if (threadIdx.x == 0) sh[32] = s;
  __syncthreads();
  return sh[32];
}

__device__ __forceinline__ void write_part(const KState& k, int q, double2 v, double2* sh) {
  const double2 s = block_sum(v, sh);
  if (threadIdx.x == 0) k.part[q * k.nb + blockIdx.x] = s;
}

// y_i = (A x)_i for rows of this thread's warp share (one warp per row)
template <typename V>
__device__ __forceinline__ double2 row_dot(const int32_t* __restrict__ indptr,
                                           const int32_t* __restrict__ indices,
                                           const V* __restrict__ vals, const V* __restrict__ x,
                                           int64_t row, int lane) {
  const int a = __ldg(&indptr[row]), b = __ldg(&indptr[row + 1]);
  double2 acc = make_double2(0.0, 0.0);
  for (int q = a + lane; q < b; q += 32) {
    const double2 av = ld(vals, q), xv = ld(x, __ldg(&indices[q]));
    acc.x += av.x * xv.x - av.y * xv.y;
    acc.y += av.x * xv.y + av.y * xv.x;
  }
  for (int o = 16; o > 0; o >>= 1) {
    acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
    acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
  }
  return acc;
}

// setup: r = b - A x, rhat = r, p = v = 0; partials (rhat, r), (r, r), (b, b);
// dinv = 1 / diag(A) when requested
template <typename V>
__global__ void __launch_bounds__(kThreads)
    k_init(int64_t n, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
           const V* __restrict__ vals, const V* __restrict__ b, const V* __restrict__ x, V* r,
           V* rhat, V* p, V* v, V* dinv, KState k) {
  __shared__ double2 sh[33];
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * kThreads + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * kThreads) >> 5;
  double2 prr = make_double2(0.0, 0.0), pbb = prr;
  for (int64_t i = gw; i < n; i += nw) {
    const double2 ax = row_dot(indptr, indices, vals, x, i, lane);
    if (lane == 0) {
      const double2 bi = ld(b, i);
      const double2 ri = make_double2(bi.x - ax.x, bi.y - ax.y);
      st(r, i, ri);
      st(rhat, i, ri);
      st(p, i, make_double2(0.0, 0.0));
      st(v, i, make_double2(0.0, 0.0));
      prr.x += ri.x * ri.x + ri.y * ri.y;
      pbb.x += bi.x * bi.x + bi.y * bi.y;
    }
    if (dinv) {
      // diagonal entry of row i (zero diagonal: no scaling)
      const int a = __ldg(&indptr[i]), e = __ldg(&indptr[i + 1]);
      double2 dv = make_double2(0.0, 0.0);
      for (int q = a + lane; q < e; q += 32)
        if (__ldg(&indices[q]) == i) dv = ld(vals, q);
      for (int o = 16; o > 0; o >>= 1) {
        dv.x += __shfl_xor_sync(0xffffffffu, dv.x, o);
        dv.y += __shfl_xor_sync(0xffffffffu, dv.y, o);
      }
      if (lane == 0) {
        const bool z = dv.x == 0.0 && dv.y == 0.0;
        st(dinv, i, z ? make_double2(1.0, 0.0) : cdiv(make_double2(1.0, 0.0), dv));
      }
    }
  }
  write_part(k, P_RHR, prr, sh);  // rhat = r: (rhat, r) = (r, r), real
  __syncthreads();
  write_part(k, P_RR, prr, sh);
  __syncthreads();
  write_part(k, P_BB, pbb, sh);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    for (int s = 0; s < SC_N; ++s) k.sc[s] = make_double2(1.0, 0.0);
    k.status[0] = 0;
    k.status[1] = 0;
  }
}

// I1: direction p and phat = M^-1 p (M^-1 diagonal or none; with an LU
// preconditioner phat is the LU solve that follows)
template <typename V>
__global__ void __launch_bounds__(kThreads)
    k_dir(int64_t n, const V* __restrict__ r, V* p, const V* __restrict__ v, V* phat,
          const V* __restrict__ dinv, KState k) {
  __shared__ double2 sh[33];
  if (k.status[0] != 0) return;
  const double2 rho_new = reduce_part(k, P_RHR, sh);
  const bool first = k.status[1] == 0;
  const double2 beta = first ? make_double2(0.0, 0.0)
                             : cmul(cdiv(rho_new, k.sc[SC_RHO]), cdiv(k.sc[SC_ALPHA], k.sc[SC_OMEGA]));
  const double2 om = k.sc[SC_OMEGA];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 ri = ld(r, i);
    double2 pi = ri;
    if (!first) {
      const double2 pv = ld(p, i), vv = ld(v, i);
      const double2 t = make_double2(pv.x - (om.x * vv.x - om.y * vv.y),
                                     pv.y - (om.x * vv.y + om.y * vv.x));
      const double2 bt = cmul(beta, t);
      pi = make_double2(ri.x + bt.x, ri.y + bt.y);
    }
    st(p, i, pi);
    if (phat) st(phat, i, dinv ? cmul(ld(dinv, i), pi) : pi);
  }
}

// I2 / I4: y = A x; partials of (w, y) [I2: w = rhat] or of (y, w) and
// (y, y) [I4: w = s]
template <typename V, bool I4>
__global__ void __launch_bounds__(kThreads)
    k_spmv(int64_t n, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
           const V* __restrict__ vals, const V* __restrict__ x, V* y, const V* __restrict__ w,
           KState k) {
  __shared__ double2 sh[33];
  if (k.status[0] != 0) return;
  const int lane = threadIdx.x & 31;
  const int64_t gw = ((int64_t)blockIdx.x * kThreads + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * kThreads) >> 5;
  double2 p0 = make_double2(0.0, 0.0), p1 = p0;
  for (int64_t i = gw; i < n; i += nw) {
    const double2 yi = row_dot(indptr, indices, vals, x, i, lane);
    if (lane == 0) {
      st(y, i, yi);
      const double2 wi = ld(w, i);
      if (!I4) {
        const double2 d = cdotc(wi, yi);  // (rhat, v) = sum conj(rhat) v
        p0.x += d.x;
        p0.y += d.y;
      } else {
        const double2 d = cdotc(yi, wi);  // (t, s) = sum conj(t) s
        p0.x += d.x;
        p0.y += d.y;
        p1.x += yi.x * yi.x + yi.y * yi.y;
      }
    }
  }
  write_part(k, I4 ? P_TS : P_RHV, p0, sh);
  if (I4) {
    __syncthreads();
    write_part(k, P_TT, p1, sh);
  }
}

// I3: alpha and s = r - alpha v (in r); shat = M^-1 s
template <typename V>
__global__ void __launch_bounds__(kThreads)
    k_alpha(int64_t n, V* r, const V* __restrict__ v, V* shat, const V* __restrict__ dinv,
            KState k) {
  __shared__ double2 sh[33];
  if (k.status[0] != 0) return;
  const double2 rho_new = reduce_part(k, P_RHR, sh);
  const double2 rv = reduce_part(k, P_RHV, sh);
  if (rv.x == 0.0 && rv.y == 0.0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) k.status[0] = -1;
    return;
  }
  const double2 alpha = cdiv(rho_new, rv);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 ri = ld(r, i), av = cmul(alpha, ld(v, i));
    const double2 si = make_double2(ri.x - av.x, ri.y - av.y);
    st(r, i, si);
    if (shat) st(shat, i, dinv ? cmul(ld(dinv, i), si) : si);
  }
  // the readers of the old rho and alpha (k_dir) ran before this kernel
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    k.sc[SC_RHO] = rho_new;
    k.sc[SC_ALPHA] = alpha;
  }
}

// I5: omega, x += alpha phat + omega shat, r = s - omega t; partials
// (rhat, r), (r, r)
template <typename V>
__global__ void __launch_bounds__(kThreads)
    k_omega(int64_t n, V* x, V* r, const V* __restrict__ t, const V* __restrict__ phat,
            const V* __restrict__ shat, const V* __restrict__ rhat, KState k) {
  __shared__ double2 sh[33];
  if (k.status[0] != 0) return;
  const double2 ts = reduce_part(k, P_TS, sh);
  const double2 tt = reduce_part(k, P_TT, sh);
  const double2 omega = tt.x == 0.0 ? make_double2(0.0, 0.0) : cdiv(ts, tt);
  const double2 alpha = k.sc[SC_ALPHA];
  double2 prh = make_double2(0.0, 0.0), prr = prh;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 xi = ld(x, i), a = cmul(alpha, ld(phat, i)), o = cmul(omega, ld(shat, i));
    st(x, i, make_double2(xi.x + a.x + o.x, xi.y + a.y + o.y));
    const double2 si = ld(r, i), ot = cmul(omega, ld(t, i));
    const double2 ri = make_double2(si.x - ot.x, si.y - ot.y);
    st(r, i, ri);
    const double2 d = cdotc(ld(rhat, i), ri);
    prh.x += d.x;
    prh.y += d.y;
    prr.x += ri.x * ri.x + ri.y * ri.y;
  }
  write_part(k, P_RHR, prh, sh);
  __syncthreads();
  write_part(k, P_RR, prr, sh);
  if (blockIdx.x == 0 && threadIdx.x == 0) k.sc[SC_OMEGA] = omega;
}

// I6 (one block): convergence and breakdown; counts the iteration
__global__ void __launch_bounds__(kThreads) k_check(KState k, double tol2, int maxit, int count) {
  __shared__ double2 sh[33];
  if (k.status[0] != 0) return;
  const double2 rr = reduce_part(k, P_RR, sh);
  const double2 bb = reduce_part(k, P_BB, sh);
  const double2 rh = reduce_part(k, P_RHR, sh);
  if (threadIdx.x != 0) return;
  const int it = k.status[1] + count;
  k.status[1] = it;
  if (rr.x <= tol2 * bb.x)
    k.status[0] = 1;
  else if (count && k.sc[SC_OMEGA].x == 0.0 && k.sc[SC_OMEGA].y == 0.0)
    k.status[0] = -2;
  else if (rh.x == 0.0 && rh.y == 0.0)
    k.status[0] = -1;
  else if (it >= maxit)
    k.status[0] = 2;
}

struct Bufs {
  void *r, *rhat, *p, *v, *phat, *shat, *t, *dinv;
  KState k;
};

int64_t part_blocks(int64_t n, int sms) {
  const int64_t want = (n + kThreads - 1) / kThreads;
  return want < 2 * (int64_t)sms ? (want < 1 ? 1 : want) : 2 * (int64_t)sms;
}

}  // namespace
}  // namespace sucem

namespace {
using namespace sucem;

int64_t work_bytes_for(int64_t n, int elem, int64_t nb) {
  const int64_t vec = ((n * elem + 255) / 256) * 256;
  return 8 * vec + (int64_t)kNP * nb * 16 + 16 * SC_N + 256;
}

template <typename T>
int run(int64_t n, const int32_t* indptr, const int32_t* indices, const void* vals_,
        const void* b_, void* x_, int precond, sucem_lu* lu, double tol, int maxit, int batch,
        void* work, int64_t work_bytes, double* info, cudaStream_t st) {
  using V = typename CT<T>::V;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t nb = part_blocks(n, sms);
  if (work_bytes < work_bytes_for(n, sizeof(V), nb))
    return fail("sucem_bicgstab: work buffer too small (see sucem_bicgstab_work_bytes)",
                SUCEM_ERR_ARG);
  const int64_t vec = ((n * (int64_t)sizeof(V) + 255) / 256) * 256;
  uint8_t* w = static_cast<uint8_t*>(work);
  V* r = (V*)(w + 0 * vec);
  V* rhat = (V*)(w + 1 * vec);
  V* p = (V*)(w + 2 * vec);
  V* v = (V*)(w + 3 * vec);
  V* phat = (V*)(w + 4 * vec);
  V* shat = (V*)(w + 5 * vec);
  V* t = (V*)(w + 6 * vec);
  V* dinv = precond == 1 ? (V*)(w + 7 * vec) : nullptr;
  KState k;
  k.part = (double2*)(w + 8 * vec);
  k.sc = k.part + kNP * nb;
  k.status = (int*)(k.sc + SC_N);
  k.nb = (int)nb;
  const V* vals = (const V*)vals_;
  const V* b = (const V*)b_;
  V* x = (V*)x_;
  const unsigned grid = (unsigned)nb;
  // M^-1 applied by the direction / alpha kernels (none, diagonal), or by
  // LU solves enqueued between them
  V* ph_k = precond == 2 ? nullptr : phat;
  V* sh_k = precond == 2 ? nullptr : shat;
  const int io = sizeof(T) == 4 ? SUCEM_C64 : SUCEM_C128;
  auto iteration = [&](cudaStream_t s) -> int {
    k_dir<V><<<grid, kThreads, 0, s>>>(n, r, p, v, ph_k, dinv, k);
    if (precond == 2) {
      const int rc = sucem_lu_solve(lu, io, p, phat, s);
      if (rc != SUCEM_OK) return rc;
    }
    k_spmv<V, false><<<grid, kThreads, 0, s>>>(n, indptr, indices, vals, phat, v, rhat, k);
    k_alpha<V><<<grid, kThreads, 0, s>>>(n, r, v, sh_k, dinv, k);
    if (precond == 2) {
      const int rc = sucem_lu_solve(lu, io, r, shat, s);
      if (rc != SUCEM_OK) return rc;
    }
    k_spmv<V, true><<<grid, kThreads, 0, s>>>(n, indptr, indices, vals, shat, t, r, k);
    k_omega<V><<<grid, kThreads, 0, s>>>(n, x, r, t, phat, shat, rhat, k);
    k_check<<<1, kThreads, 0, s>>>(k, tol * tol, maxit, 1);
    count_launch(6);
    return SUCEM_OK;
  };
  k_init<V><<<grid, kThreads, 0, st>>>(n, indptr, indices, vals, b, x, r, rhat, p, v, dinv, k);
  k_check<<<1, kThreads, 0, st>>>(k, tol * tol, maxit, 0);
  count_launch(2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "sucem_bicgstab");
  int h_status[2] = {0, 0};
  int syncs = 0;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap = nullptr;
  if (precond != 2 && batch > 1) {
    // capture `batch` iterations once on a private stream, replay on st
    e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    cudaGraph_t g = nullptr;
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      for (int i = 0; i < batch; ++i) iteration(cap);
      e = cudaStreamEndCapture(cap, &g);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      if (cap) cudaStreamDestroy(cap);
      return cuda_fail(e, "sucem_bicgstab: graph capture");
    }
  }
  int rc = SUCEM_OK;
  while (true) {
    e = cudaMemcpyAsync(h_status, k.status, sizeof(h_status), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    ++syncs;
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "sucem_bicgstab");
      break;
    }
    if (h_status[0] != 0) break;
    if (exec) {
      e = cudaGraphLaunch(exec, st);
      count_launch(6 * batch);
      if (e != cudaSuccess) {
        rc = cuda_fail(e, "sucem_bicgstab: graph launch");
        break;
      }
    } else {
      const int nb_it = precond == 2 ? 1 : (batch < 1 ? 1 : batch);
      for (int i = 0; i < nb_it && rc == SUCEM_OK; ++i) rc = iteration(st);
      if (rc != SUCEM_OK) break;
    }
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (cap) cudaStreamDestroy(cap);
  if (rc != SUCEM_OK) return rc;
  // final relative residual ||r|| / ||b|| from the partials (host side)
  double2 part_rr_bb[2] = {{0, 0}, {0, 0}};
  {
    double2* hp = new double2[kNP * nb];
    e = cudaMemcpy(hp, k.part, sizeof(double2) * kNP * nb, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
      for (int64_t i = 0; i < nb; ++i) {
        part_rr_bb[0].x += hp[P_RR * nb + i].x;
        part_rr_bb[1].x += hp[P_BB * nb + i].x;
      }
    delete[] hp;
    if (e != cudaSuccess) return cuda_fail(e, "sucem_bicgstab");
  }
  if (info) {
    info[0] = h_status[1];
    info[1] = part_rr_bb[1].x > 0 ? std::sqrt(part_rr_bb[0].x / part_rr_bb[1].x) : 0.0;
    info[2] = h_status[0];
    info[3] = syncs;
  }
  return SUCEM_OK;
}

}  // namespace

extern "C" {

int64_t sucem_bicgstab_work_bytes(int64_t n, int dtype) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int elem = dtype == SUCEM_C64 ? 8 : 16;
  return work_bytes_for(n, elem, part_blocks(n, sms));
}

int sucem_bicgstab(int64_t n, const int32_t* indptr, const int32_t* indices, int dtype,
                   const void* vals, const void* b, void* x, int precond, sucem_lu* lu,
                   double tol, int maxit, int batch, void* work, int64_t work_bytes, double* info,
                   void* stream) {
  if (!indptr || !indices || !vals || !b || !x || !work) return fail("null argument", SUCEM_ERR_ARG);
  if (n < 1 || maxit < 0 || tol < 0) return fail("bad size or tolerance", SUCEM_ERR_ARG);
  if (precond < 0 || precond > 2 || (precond == 2 && !lu))
    return fail("precond: 0 none, 1 diagonal, 2 LU (needs the LU handle)", SUCEM_ERR_ARG);
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == SUCEM_C64)
    return run<float>(n, indptr, indices, vals, b, x, precond, lu, tol, maxit, batch, work,
                      work_bytes, info, st);
  if (dtype == SUCEM_C128)
    return run<double>(n, indptr, indices, vals, b, x, precond, lu, tol, maxit, batch, work,
                       work_bytes, info, st);
  return fail("sucem_bicgstab: complex dtypes only (SUCEM_C64, SUCEM_C128)", SUCEM_ERR_ARG);
}

}  // extern "C"
