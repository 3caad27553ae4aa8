// Tensor-core (tcgen05) Schur-block update of complex single-precision
// fronts, included by mf_numeric.cu inside its anonymous namespace (uses
// DNode and the row-major front arena).
//
// Complex64 fronts are factorised in super-panels; when the super-panel
// [sp0, bnd) of a front is finished (its last 64-column panel factorised),
// the trailing block takes, over one 128 x 128 tile per CTA,
//   F[bnd:f, bnd:f] -= F[bnd:f, sp0:bnd] * F[sp0:bnd, bnd:f]
// (the last super-panel's trailing block is the Schur complement).
//
// Arithmetic: complex FP32 operands are split into TF32 pairs x = hi + lo
// (hi = x rounded to TF32, lo = x - hi), and every real product is formed as
// hi*hi + hi*lo + lo*hi (the 3xTF32 scheme, ~2^-21 relative), so one complex
// K-step is 12 tcgen05.mma.kind::tf32 instructions (M = 128, N = 128, K = 8)
// accumulating Re and Im in two FP32 TMEM blocks; the -Im*Im terms use the
// instruction's A-negation bit.
//
// Pipeline: K is consumed in chunks of 16; all 256 threads load a chunk
// (A: 128 rows x 16, B: 16 x 128 columns; two chunks ahead, through two
// register buffers), split it and store eight K-major
// operand planes (Re/Im x hi/lo for A and B) in the canonical no-swizzle
// core-matrix layout (8 rows x 16 bytes per core matrix, 128 bytes apart
// along K, 512 bytes apart along M/N) into one of three stages; one thread
// issues the chunk's 24 MMAs and commits them to the stage's mbarrier, which
// gates the stage's reuse three chunks later.  Every wait is bounded: on a
// timeout the kernel raises *err and skips the write-back.
namespace tc {

constexpr int BM = 128;                        // tile rows (TMEM lanes)
constexpr int BN = 128;                        // tile columns (complex)
constexpr int KC = 16;                         // K per chunk
constexpr int STAGES = 3;
constexpr int THREADS = 256;
constexpr int PLANE = BM * KC * 4;             // bytes of one operand plane (BN == BM)
constexpr int STAGE_BYTES = 8 * PLANE;         // A: Re hi/lo, Im hi/lo; then B likewise
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 256;
constexpr int TMEM_COLS = 2 * BN;              // Re then Im accumulators
constexpr int kWaitLimit = 1 << 24;            // polls of one mbarrier before giving up
static_assert(BN == BM, "planes share one size");

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of element (r, k) in a K-major no-swizzle plane of KC columns
__device__ __forceinline__ int core_off(int r, int kgroup) {
  return ((r >> 3) * (KC / 4) + kgroup) * 128 + (r & 7) * 16;
}

// shared-memory matrix descriptor: start address, leading (K) byte offset
// 128, stride (M/N) byte offset 512, fixed field 0b001 at bit 46, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) |
         ((uint64_t)((KC / 4) * 128 >> 4) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor, kind::tf32: D f32, A/B tf32, K-major A and B
__host__ __device__ constexpr uint32_t idesc(bool neg_a) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((neg_a ? 1u : 0u) << 13) |
         ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id,
                                    uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(id), "r"(acc));
}

__device__ __forceinline__ bool wait_parity(uint32_t bar, uint32_t parity) {
  uint32_t done = 0;
  for (int it = 0; it < kWaitLimit; ++it) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity));
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// split four complex values into Re/Im hi/lo quads and store them at `off`
// of the four planes starting at `planes`
__device__ __forceinline__ void store_split(uint8_t* planes, int off, const float2* v) {
  float4 rh, rl, ih, il;
  float* prh = &rh.x;
  float* prl = &rl.x;
  float* pih = &ih.x;
  float* pil = &il.x;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    prh[q] = tf32_hi(v[q].x);
    prl[q] = tf32_hi(v[q].x - prh[q]);
    pih[q] = tf32_hi(v[q].y);
    pil[q] = tf32_hi(v[q].y - pih[q]);
  }
  *reinterpret_cast<float4*>(planes + 0 * PLANE + off) = rh;
  *reinterpret_cast<float4*>(planes + 1 * PLANE + off) = rl;
  *reinterpret_cast<float4*>(planes + 2 * PLANE + off) = ih;
  *reinterpret_cast<float4*>(planes + 3 * PLANE + off) = il;
}

// one output tile: rows [row0, row0 + nrow) x columns [col0, col0 + ncol) of
// the front take -= F[rows, kk0:kk0+K] * F[kk0:kk0+K, columns]
struct Tile {
  int row0, nrow, col0, ncol, kk0, K;
};

// tile `bx` of the trailing block [bnd, f)^2 with K = bnd - sp0 of the
// super-panel [sp0, bnd) of width sp that ends with the panel at p0 (false:
// the front's super-panel does not end there, or no such tile)
__device__ __forceinline__ bool tile_of(const DNode& nd, int p0, int sp, int nbt, int bx,
                                        Tile& t) {
  if (p0 >= nd.k) return false;
  const int sp0 = (p0 / sp) * sp;
  const int bnd = min(nd.k, sp0 + sp);
  if (p0 + min(nbt, nd.k - p0) != bnd) return false;
  t.kk0 = sp0;
  t.K = bnd - sp0;
  const int mn = nd.f - bnd;
  if (mn <= 0 || t.K <= 0) return false;
  const int tpd = (mn + BM - 1) / BM;
  if (bx >= tpd * tpd) return false;
  t.row0 = bnd + (bx / tpd) * BM;
  t.col0 = bnd + (bx % tpd) * BN;
  t.nrow = min(BM, nd.f - t.row0);
  t.ncol = min(BN, nd.f - t.col0);
  return true;
}

}  // namespace tc

// the trailing update of every listed front, one 128 x 128 output tile per
// block (blockIdx.x: tile, blockIdx.y: front)
__global__ void __launch_bounds__(tc::THREADS, 1)
    tc_update_kernel(const int32_t* __restrict__ list, int count, const DNode* __restrict__ nodes,
                     float2* __restrict__ arena, int p0, int sp, int nbt, int* __restrict__ err) {
  using namespace tc;
  extern __shared__ __align__(128) uint8_t tc_smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(tc_smem_raw) + 127) & ~(uintptr_t)127);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mbar + STAGES);

  const int fi = blockIdx.y;
  if (fi >= count) return;
  const DNode nd = nodes[list[fi]];
  Tile tl;
  if (!tile_of(nd, p0, sp, nbt, (int)blockIdx.x, tl)) return;
  const int kk0 = tl.kk0, K = tl.K;
  float2* F = arena + nd.off;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // staging roles: A row ar (8 consecutive k from akh*8), B column bn (8
  // consecutive k from bkh*8)
  const int ar = tid % BM, akh = tid / BM;
  const int bn = tid % BN, bkh = tid / BN;
  const bool arow_ok = ar < tl.nrow, bcol_ok = bn < tl.ncol;
  const float2* Arow = F + (int64_t)(tl.row0 + (arow_ok ? ar : 0)) * nd.f + kk0;
  const float2* Bcol = F + (int64_t)kk0 * nd.f + tl.col0 + (bcol_ok ? bn : 0);

  if (tid == 0) {
#pragma unroll
    for (int s = 0; s < STAGES; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[s])));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = *tmem_slot;

  const int nchunks = (K + KC - 1) / KC;
  const float2 zero = make_float2(0.f, 0.f);
  // two register buffers: chunk c + 2 is loaded while chunk c is stored
  float2 av0[8], bv0[8], av1[8], bv1[8];
  auto gload = [&](float2* av, float2* bv, int c) {
    const int ka = c * KC + akh * 8, kb = c * KC + bkh * 8;
#pragma unroll
    for (int j = 0; j < 8; ++j) av[j] = (arow_ok && ka + j < K) ? Arow[ka + j] : zero;
#pragma unroll
    for (int j = 0; j < 8; ++j)
      bv[j] = (bcol_ok && kb + j < K) ? Bcol[(int64_t)(kb + j) * nd.f] : zero;
  };
  bool ok = true;
  auto step = [&](float2* av, float2* bv, int c) {
    const int s = c % STAGES;
    if (c >= STAGES) ok = wait_parity(smem_u32(&mbar[s]), ((c / STAGES) - 1) & 1) && ok;
    uint8_t* st = smem + s * STAGE_BYTES;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      store_split(st, core_off(ar, akh * 2 + h), av + 4 * h);
      store_split(st + 4 * PLANE, core_off(bn, bkh * 2 + h), bv + 4 * h);
    }
    if (c + 2 < nchunks) gload(av, bv, c + 2);
    asm volatile("fence.proxy.async.shared::cta;");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t base = smem_u32(st);
#pragma unroll
      for (int ks = 0; ks < KC / 8; ++ks) {
        uint64_t a[4], b[4];
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          a[p] = sdesc(base + p * PLANE + ks * 256);
          b[p] = sdesc(base + (4 + p) * PLANE + ks * 256);
        }
        const uint32_t first = (c > 0 || ks > 0) ? 1u : 0u;
        const uint32_t pos = idesc(false), neg = idesc(true);
        const uint32_t dre = tmem, dim = tmem + BN;
        // Re += Are*Bre - Aim*Bim
        mma(dre, a[0], b[0], pos, first);
        mma(dre, a[0], b[1], pos, 1);
        mma(dre, a[1], b[0], pos, 1);
        mma(dre, a[2], b[2], neg, 1);
        mma(dre, a[2], b[3], neg, 1);
        mma(dre, a[3], b[2], neg, 1);
        // Im += Are*Bim + Aim*Bre
        mma(dim, a[0], b[2], pos, first);
        mma(dim, a[0], b[3], pos, 1);
        mma(dim, a[1], b[2], pos, 1);
        mma(dim, a[2], b[0], pos, 1);
        mma(dim, a[2], b[1], pos, 1);
        mma(dim, a[3], b[0], pos, 1);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_u32(&mbar[s])));
    }
  };
  gload(av0, bv0, 0);
  if (nchunks > 1) gload(av1, bv1, 1);
  for (int c = 0; c < nchunks; c += 2) {
    step(av0, bv0, c);
    if (c + 1 < nchunks) step(av1, bv1, c + 1);
  }
  // the last commit covers every MMA of the tile
  const int cl = nchunks - 1;
  ok = wait_parity(smem_u32(&mbar[cl % STAGES]), (cl / STAGES) & 1) && ok;
  ok = __syncthreads_and(ok);  // uniform: the TMEM loads below are warp-collective
  if (!ok && tid == 0) atomicExch(err, 1);
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (ok) {
    // warp w reads TMEM lanes 32 (w % 4) .. +31 (tile rows) and columns
    // 64 (w / 4) .. +63 of both accumulators, 16 at a time
    const int q = warp & 3, half = warp >> 2;
    const int row = q * 32 + lane;
    float2* Crow = F + (int64_t)(tl.row0 + (row < tl.nrow ? row : 0)) * nd.f + tl.col0;
#pragma unroll 1
    for (int cc = 0; cc < 4; ++cc) {
      const int col0 = half * 64 + cc * 16;
      uint32_t re[16], im[16];
      const uint32_t tre = tmem + ((uint32_t)(q * 32) << 16) + col0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(re[0]), "=r"(re[1]), "=r"(re[2]), "=r"(re[3]), "=r"(re[4]), "=r"(re[5]),
            "=r"(re[6]), "=r"(re[7]), "=r"(re[8]), "=r"(re[9]), "=r"(re[10]), "=r"(re[11]),
            "=r"(re[12]), "=r"(re[13]), "=r"(re[14]), "=r"(re[15])
          : "r"(tre));
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(im[0]), "=r"(im[1]), "=r"(im[2]), "=r"(im[3]), "=r"(im[4]), "=r"(im[5]),
            "=r"(im[6]), "=r"(im[7]), "=r"(im[8]), "=r"(im[9]), "=r"(im[10]), "=r"(im[11]),
            "=r"(im[12]), "=r"(im[13]), "=r"(im[14]), "=r"(im[15])
          : "r"(tre + BN));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      if (row < tl.nrow) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int col = col0 + j;
          if (col < tl.ncol) {
            float2 v = Crow[col];
            v.x -= __uint_as_float(re[j]);
            v.y -= __uint_as_float(im[j]);
            Crow[col] = v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS));
}
