// Tensor-core (tcgen05) trailing update of single-precision fronts, real
// (float) or complex (float2), included by mf_numeric.cu inside its
// anonymous namespace (uses DNode and the row-major front arena).
//
// Single-precision fronts are factorised in super-panels; when the
// super-panel [sp0, bnd) of a front is finished (its last 64-column panel
// factorised), the trailing block takes
//   F[bnd:f, bnd:f] -= F[bnd:f, sp0:bnd] * F[sp0:bnd, bnd:f]
// (the last super-panel's trailing block is the Schur complement), and on
// levels with large pivot blocks every 64-column panel p0 applies its
// K = 64 update to the rows and columns of its super-panel outside the
// deferred block.  A launch covers a list of 128 x 128 output tiles, each
// given by its own descriptor (front, rows, columns, K range), planned on
// the host.
//
// Arithmetic: FP32 operands are split into TF32 pairs x = hi + lo (hi = x
// rounded to TF32, lo = x - hi rounded to TF32), and every real product is
// formed as hi*hi + hi*lo + lo*hi (the 3xTF32 scheme, ~2^-21 relative):
// a real K-step is 3 tcgen05.mma.kind::tf32 instructions (M = 128, N = 128,
// K = 8) into one FP32 TMEM accumulator; a complex K-step is 12, Re and Im
// in two accumulators, the -Im*Im terms through the instruction's
// A-negation bit.
//
// Operands are split once per launch by tc_presplit_kernel: every strip of
// A (128 rows x K) and of B (K x 128 columns) that the launch's tiles use
// is written, K-chunk by K-chunk (16), as the exact shared-memory image the
// MMAs read: the K-major operand planes (real: hi/lo; complex: Re/Im x
// hi/lo) in the canonical no-swizzle core-matrix layout (8 rows x 16 bytes
// per core matrix, 128 bytes apart along K, 512 bytes apart along M/N).
//
// Structure: a persistent, warp-specialised kernel, one CTA per SM walking
// the tile list round-robin.
//   warp 8, one thread (producer): per K-chunk of a tile, waits for the
//     stage's "empty" barrier, announces the stage's bytes on its "full"
//     barrier and issues two bulk asynchronous copies (the A and the B
//     chunk image, cp.async.bulk) that complete on "full";
//   warp 9, one thread (MMA issuer): per chunk, waits for "full", issues
//     the chunk's MMAs into the tile's TMEM accumulator(s) and commits them
//     to the stage's "empty" barrier (the producers' permission to refill
//     it); after a tile's last chunk it commits to the accumulator's
//     "acc_full" barrier;
//   warps 0-7 (epilogue, two per TMEM lane quarter, one per column half):
//     request the first 16 columns of their C block, wait for "acc_full",
//     read their 32 TMEM lanes (tile rows) 16 columns at a time (each
//     block's C requested before its TMEM reads), turn them
//     through shared memory so that a warp's accesses to C cover two rows of
//     16 consecutive columns, apply C -= D and arrive on "acc_empty".
// Two accumulator sets let the epilogue of one tile run under the main
// loop of the next.  Every wait is bounded: on a timeout the kernel raises
// *err, every role stops, and all meet at the final barrier.
namespace tc {

constexpr int BM = 128;                        // tile rows (TMEM lanes)
constexpr int BN = 128;                        // tile columns
constexpr int KC = 16;                         // K per chunk
constexpr int STAGES = 3;
constexpr int EPI_WARPS = 8;                   // two per TMEM lane quarter (column halves)
constexpr int THREADS = 32 * (EPI_WARPS + 2);  // epilogue warps, 1 producer warp, 1 MMA warp
constexpr int PRODUCER_WARP = EPI_WARPS;
constexpr int MMA_WARP = EPI_WARPS + 1;
constexpr int TD = 12;                         // ints per tile descriptor
constexpr int PLANE = BM * KC * 4;             // bytes of one operand plane (BN == BM)
constexpr int EPI_BYTES = EPI_WARPS * 32 * 17 * 8;  // per epilogue warp: 32 rows x 16 (+1) values
constexpr int kWaitLimit = 1 << 24;            // polls of one mbarrier before giving up
static_assert(BN == BM, "planes share one size");

// per element type: operand planes of A (and of B), accumulators per tile
template <typename S>
struct Cfg;
template <>
struct Cfg<float2> {
  static constexpr int NP = 4;                 // Re hi, Re lo, Im hi, Im lo
  static constexpr int NACC = 2;               // Re, Im
};
template <>
struct Cfg<float> {
  static constexpr int NP = 2;                 // hi, lo
  static constexpr int NACC = 1;
};
template <typename S>
__host__ __device__ constexpr int chunk_bytes() { return Cfg<S>::NP * PLANE; }  // one operand's K-chunk image
template <typename S>
__host__ __device__ constexpr int stage_bytes() { return 2 * chunk_bytes<S>(); }  // A planes, then B planes
template <typename S>
__host__ __device__ constexpr int smem_bytes() { return STAGES * stage_bytes<S>() + EPI_BYTES + 512; }
template <typename S>
__host__ __device__ constexpr int acc_cols() { return Cfg<S>::NACC * BN; }  // the accumulators of one tile
template <typename S>
__host__ __device__ constexpr int tmem_cols() { return 2 * acc_cols<S>(); }  // two tiles in flight

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// byte offset of row r, K-group kgroup (4 consecutive K) in a K-major
// no-swizzle plane of KC columns
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

__device__ __forceinline__ void commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar));
}

__device__ __forceinline__ void arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar));
}

// arrive on `bar` and add `bytes` to the transaction count its phase waits for
__device__ __forceinline__ void arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

// bulk asynchronous copy global -> shared (16-byte aligned, size a multiple
// of 16), completing `bytes` transactions on `bar`
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes,
                                          uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// bounded wait for the phase with the given parity; with backoff, a failed
// poll sleeps briefly (for waiters that are not on the critical path);
// false after `limit` failed polls
__device__ __forceinline__ bool wait_parity(uint32_t bar, uint32_t parity, bool backoff = false,
                                            int limit = kWaitLimit) {
  uint32_t done = 0;
  for (int it = 0; it < limit; ++it) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity));
    if (done) return true;
    if (backoff) __nanosleep(256);
  }
  return false;
}

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// split four real values into hi/lo quads and store them at `off` of the
// two planes starting at `planes`
__device__ __forceinline__ void store_split(uint8_t* planes, int off, const float* v) {
  float4 h, l;
  float* ph = &h.x;
  float* pl = &l.x;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    ph[q] = tf32_hi(v[q]);
    pl[q] = tf32_hi(v[q] - ph[q]);
  }
  *reinterpret_cast<float4*>(planes + 0 * PLANE + off) = h;
  *reinterpret_cast<float4*>(planes + 1 * PLANE + off) = l;
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

// a tile from its descriptor: TD ints {front node, row0, col0, nrow, ncol,
// kk0, K, first chunk image of its A strip, of its B strip, 0, 0, 0}
__device__ __forceinline__ Tile tile_of(const int32_t* td) {
  Tile t;
  t.row0 = td[1];
  t.col0 = td[2];
  t.nrow = td[3];
  t.ncol = td[4];
  t.kk0 = td[5];
  t.K = td[6];
  return t;
}

}  // namespace tc

// One block per K-chunk image of a launch: strip descriptors of 8 ints
// {front node, first row (A) or column (B), rows/columns in use (<= 128),
// kk0, K, first chunk image, side (0: A rows, 1: B columns), 0} and the
// strip of every chunk image.  Values outside the strip (rows past n, K
// past the range) are zero.
template <typename S>
__global__ void __launch_bounds__(256)
    tc_presplit_kernel(const int32_t* __restrict__ strips, const int32_t* __restrict__ chunk_strip,
                       const DNode* __restrict__ nodes, const S* __restrict__ arena,
                       uint8_t* __restrict__ img) {
  pdl_wait();  // launched with programmatic dependent launch
  pdl_trigger();
  using namespace tc;
  const int32_t* sd = strips + 8 * __ldg(&chunk_strip[blockIdx.x]);
  const DNode nd = nodes[sd[0]];
  const int r0 = sd[1], n = sd[2], kk0 = sd[3], K = sd[4], side = sd[6];
  const int c = (int)blockIdx.x - sd[5];
  const S* F = arena + nd.off;
  uint8_t* dst = img + (int64_t)blockIdx.x * chunk_bytes<S>();
  S zero;
  if constexpr (std::is_same<S, float2>::value) zero = make_float2(0.f, 0.f); else zero = 0.f;
  for (int it = threadIdx.x; it < BM * (KC / 4); it += blockDim.x) {
    // A: four threads per row (consecutive K groups, 128 contiguous bytes);
    // B: consecutive threads on consecutive columns
    const int r = side == 0 ? it >> 2 : it & (BM - 1);
    const int kg = side == 0 ? it & 3 : it >> 7;
    S v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = c * KC + 4 * kg + j;
      if (r < n && k < K)
        v[j] = side == 0 ? F[(int64_t)(r0 + r) * nd.f + kk0 + k] : F[(int64_t)(kk0 + k) * nd.f + r0 + r];
      else
        v[j] = zero;
    }
    store_split(dst, core_off(r, kg), v);
  }
}

// the listed tiles (TD-int descriptors, see tile_of), each CTA taking tiles
// blockIdx.x, blockIdx.x + gridDim.x, ...; S = float or float2; img: the
// launch's chunk images (tc_presplit_kernel)
template <typename S>
__global__ void __launch_bounds__(tc::THREADS, 1)
    tc_update_kernel(const int32_t* __restrict__ tiles, int ntiles,
                     const DNode* __restrict__ nodes, S* __restrict__ arena,
                     const uint8_t* __restrict__ img, int* __restrict__ err) {
  using namespace tc;
  constexpr bool CPLX = std::is_same<S, float2>::value;
  constexpr int NP = Cfg<S>::NP, SB = stage_bytes<S>(), CB = chunk_bytes<S>(), ACC = acc_cols<S>(),
                TM = tmem_cols<S>();
  extern __shared__ __align__(128) uint8_t tc_smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(tc_smem_raw) + 127) & ~(uintptr_t)127);
  S* epi = reinterpret_cast<S*>(smem + STAGES * SB);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * SB + EPI_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* acc_full = empty + STAGES;
  uint64_t* acc_empty = acc_full + 2;
  uint64_t* drain = acc_empty + 2;  // give-up path: completion of issued MMAs
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* fail = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[s])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
    }
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&acc_full[b])));
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&acc_empty[b])),
                   "r"(32 * EPI_WARPS));
    }
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(drain)));
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TM));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  // launched with programmatic dependent launch: the barrier and TMEM setup
  // above overlap the kernel before; the arena and the chunk images are
  // read only after this
  pdl_wait();
  pdl_trigger();
  const uint32_t tmem = *tmem_slot;
  auto raise = [&]() {
    *fail = 1;
    atomicExch(err, 1);
  };

  if (warp == PRODUCER_WARP) {
    // ---- producer: one thread fills each stage with two bulk copies ----
    if (lane == 0) {
      int g = 0;  // chunk counter over all tiles of this CTA
      bool ok = true;
      for (int it = blockIdx.x; it < ntiles && ok; it += gridDim.x) {
        const int32_t* td = tiles + TD * it;
        const int nch = (td[6] + KC - 1) / KC;
        const uint8_t* ia = img + (int64_t)td[7] * CB;
        const uint8_t* ib = img + (int64_t)td[8] * CB;
        for (int c = 0; c < nch; ++c, ++g) {
          const int s = g % STAGES;
          if (*fail || (g >= STAGES && !wait_parity(smem_u32(&empty[s]), ((g / STAGES) - 1) & 1))) {
            ok = false;
            break;
          }
          const uint32_t st = smem_u32(smem + s * SB), fb = smem_u32(&full[s]);
          arrive_expect_tx(fb, 2 * CB);
          bulk_copy(st, ia + (int64_t)c * CB, CB, fb);
          bulk_copy(st + CB, ib + (int64_t)c * CB, CB, fb);
        }
        if (*fail) ok = false;
      }
      if (!ok) {
        raise();
        // giving up: let the copies this thread issued land before the
        // shared memory is released (bounded waits on their stages)
        for (int q = g - STAGES; q < g; ++q)
          if (q >= 0) wait_parity(smem_u32(&full[q % STAGES]), (q / STAGES) & 1);
      }
    }
    __syncwarp();
  } else if (warp == MMA_WARP) {
    // ---- MMA issuer ----
    if (lane == 0) {
      int g = 0, i = 0;
      bool ok = true;
      const uint32_t pos = idesc(false), neg = idesc(true);
      for (int it = blockIdx.x; it < ntiles && ok; it += gridDim.x, ++i) {
        const Tile tl = tile_of(tiles + TD * it);
        const int nch = (tl.K + KC - 1) / KC;
        const int b = i & 1;
        if (i >= 2 && !wait_parity(smem_u32(&acc_empty[b]), ((i / 2) - 1) & 1)) {
          ok = false;
          raise();
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t dre = tmem + b * ACC;
        for (int c = 0; c < nch; ++c, ++g) {
          const int s = g % STAGES;
          if (!wait_parity(smem_u32(&full[s]), (g / STAGES) & 1)) {
            ok = false;
            raise();
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t base = smem_u32(smem + s * SB);
#pragma unroll
          for (int ks = 0; ks < KC / 8; ++ks) {
            uint64_t a[NP], bb[NP];
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              a[p] = sdesc(base + p * PLANE + ks * 256);
              bb[p] = sdesc(base + (NP + p) * PLANE + ks * 256);
            }
            const uint32_t first = (c > 0 || ks > 0) ? 1u : 0u;
            if constexpr (CPLX) {
              const uint32_t dim = dre + BN;
              // Re += Are*Bre - Aim*Bim
              mma(dre, a[0], bb[0], pos, first);
              mma(dre, a[0], bb[1], pos, 1);
              mma(dre, a[1], bb[0], pos, 1);
              mma(dre, a[2], bb[2], neg, 1);
              mma(dre, a[2], bb[3], neg, 1);
              mma(dre, a[3], bb[2], neg, 1);
              // Im += Are*Bim + Aim*Bre
              mma(dim, a[0], bb[2], pos, first);
              mma(dim, a[0], bb[3], pos, 1);
              mma(dim, a[1], bb[2], pos, 1);
              mma(dim, a[2], bb[0], pos, 1);
              mma(dim, a[2], bb[1], pos, 1);
              mma(dim, a[3], bb[0], pos, 1);
            } else {
              mma(dre, a[0], bb[0], pos, first);
              mma(dre, a[0], bb[1], pos, 1);
              mma(dre, a[1], bb[0], pos, 1);
            }
          }
          commit(smem_u32(&empty[s]));
        }
        if (!ok) break;
        commit(smem_u32(&acc_full[b]));
        if (*fail) ok = false;
      }
      if (!ok) {
        // giving up: MMAs already issued may still be writing TMEM, which is
        // freed after the final barrier; track them all with one more commit
        // and wait (bounded) until they have completed
        commit(smem_u32(drain));
        wait_parity(smem_u32(drain), 0);
      }
    }
    __syncwarp();
  } else {
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (tile rows),
    // columns of half w / 4 ----
    int i = 0;
    for (int it = blockIdx.x; it < ntiles; it += gridDim.x, ++i) {
      const DNode nd = nodes[tiles[TD * it]];
      const Tile tl = tile_of(tiles + TD * it);
      const int b = i & 1;
      S* buf = epi + warp * 32 * 17;  // [32 rows][17]
      // TMEM lanes (tile rows) 32 q .. 32 q + 31, columns [64 h, 64 h + 64)
      const int q = warp & 3, h = warp >> 2;
      S* Cw = arena + nd.off + (int64_t)(tl.row0 + q * 32) * nd.f + tl.col0;
      // C of each 16-column block is requested before that block's TMEM
      // reads (the first one before the accumulator is ready): C is not
      // touched by the tile's main loop, so its load latency overlaps them
      S cv[16];
      auto load_c = [&](int cc) {
#pragma unroll
        for (int t = 0; t < 16; ++t) {
          const int r = 2 * t + (lane >> 4), col = cc * 16 + (lane & 15);
          if (q * 32 + r < tl.nrow && col < tl.ncol)
            cv[t] = Cw[(int64_t)r * nd.f + col];
          else if constexpr (CPLX)
            cv[t] = make_float2(0.f, 0.f);
          else
            cv[t] = 0.f;
        }
      };
      const int cc0 = h * (BN / 32);
      load_c(cc0);
      // uniform per warp: the TMEM loads below are warp-collective
      const bool got =
          __all_sync(~0u, wait_parity(smem_u32(&acc_full[b]), (i / 2) & 1, true));
      if (!got || *fail) {
        if (lane == 0) raise();
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t tre = tmem + b * ACC + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
      for (int cc = cc0; cc < cc0 + BN / 32; ++cc) {
        if (cc > cc0) load_c(cc);
        uint32_t re[16], im[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(re[0]), "=r"(re[1]), "=r"(re[2]), "=r"(re[3]), "=r"(re[4]), "=r"(re[5]),
              "=r"(re[6]), "=r"(re[7]), "=r"(re[8]), "=r"(re[9]), "=r"(re[10]), "=r"(re[11]),
              "=r"(re[12]), "=r"(re[13]), "=r"(re[14]), "=r"(re[15])
            : "r"(tre + cc * 16));
        if constexpr (CPLX)
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
              : "=r"(im[0]), "=r"(im[1]), "=r"(im[2]), "=r"(im[3]), "=r"(im[4]), "=r"(im[5]),
                "=r"(im[6]), "=r"(im[7]), "=r"(im[8]), "=r"(im[9]), "=r"(im[10]), "=r"(im[11]),
                "=r"(im[12]), "=r"(im[13]), "=r"(im[14]), "=r"(im[15])
              : "r"(tre + BN + cc * 16));
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        // lane = row: park the 16 values, then read them back column-major
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          if constexpr (CPLX)
            buf[lane * 17 + j] = make_float2(__uint_as_float(re[j]), __uint_as_float(im[j]));
          else
            buf[lane * 17 + j] = __uint_as_float(re[j]);
        }
        __syncwarp();
#pragma unroll
        for (int t = 0; t < 16; ++t) {
          const int r = 2 * t + (lane >> 4), col = cc * 16 + (lane & 15);
          if (q * 32 + r < tl.nrow && col < tl.ncol) {
            const S dv = buf[r * 17 + (lane & 15)];
            if constexpr (CPLX)
              Cw[(int64_t)r * nd.f + col] = make_float2(cv[t].x - dv.x, cv[t].y - dv.y);
            else
              Cw[(int64_t)r * nd.f + col] = cv[t] - dv;
          }
        }
        __syncwarp();
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      arrive(smem_u32(&acc_empty[b]));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == MMA_WARP)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TM));
}
