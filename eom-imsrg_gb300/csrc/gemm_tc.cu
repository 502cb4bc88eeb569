// Mixed-precision channel contractions on the 5th-generation tensor cores (tcgen05).
//
// Operands are FP64 matrices split into S bfloat16 slices (x = x0 + x1 [+ x2], each
// slice the bf16 rounding of the remainder), stored K-major as 128-row x 64-column
// tiles in one buffer per slice.  One persistent, warp-specialised kernel computes
// C = sum_terms sign_t * A_t B_t^T over a static tile list:
//   warp 0    : TMA producer (cp.async.bulk.tensor 2D, 128B swizzle) into a smem ring
//   warp 1    : allocates TMEM, issues tcgen05.mma (kind::f16, BF16 in, FP32 accumulate)
//               for the slice products (S=2: 3 products, S=3: 6 products)
//   warps 2-5 : epilogue, tcgen05.ld of the FP32 accumulator, FP64 / FP32 stores
// Two TMEM accumulators let the epilogue of one tile overlap the MMAs of the next.
// Every wait is bounded (globaltimer); a timeout sets an error word and the kernel
// drains its copies, frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "dev.cuh"
#include "engine.h"
#include "kernels.h"
#include "comm122.h"
#include "pair_groups.h"
#include "recouple.h"
#include "split.cuh"
#include "tc.h"

namespace imsrg {

namespace {

constexpr int BM = 128;
constexpr int TILE_BYTES = BM * 128;  // 128 rows of 128 bytes: 16 KiB, one TMA box
constexpr int NUM_THREADS = 320;  // TMA warp, MMA warp, 8 epilogue warps

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait on a barrier phase.  Returns false (after recording `code`) when it has waited
// more than limit_ns, or when another role has already aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, int* err,
                                          int code, unsigned long long limit_ns) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  while (true) {
    if (mbar_test(bar, parity)) return true;
    if (*abort_flag) return false;
    if (globaltimer() - t0 > limit_ns) {
      atomicCAS(err, 0, code);
      *abort_flag = 1;
      return false;
    }
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// shared-memory matrix descriptor: K-major operand tile, 128-byte rows, 128B swizzle,
// 8-row groups 1024 bytes apart (SBO); LBO is unused for swizzled K-major layouts.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;             // LBO (16 bytes, ignored)
  d |= (uint64_t)(1024 >> 4) << 32;   // SBO
  d |= (uint64_t)1 << 46;             // descriptor version (tcgen05)
  d |= (uint64_t)2 << 61;             // 128-byte swizzle
  return d;
}

// Operand element kinds of the tensor-core products: split-BF16 (tcgen05.mma kind::f16, A and
// B both BF16) or split-TF32 (kind::tf32, FP32 words rounded to TF32).  A tile row is 128
// bytes in both: 64 BF16 or 32 TF32 values of K, and one MMA consumes 32 bytes of it (K = 16
// BF16 or 8 TF32), so the shared-memory descriptors step the same way.
enum TcKind : int { kKindBF16 = 0, kKindTF32 = 1 };
constexpr int kMmaPerRow = 4;  // MMAs per 128-byte tile row

// instruction descriptor (kind::f16 / kind::tf32): FP32 D (bits 4-5 = 1), A and B types in
// bits 7-9 / 10-12 (BF16 = 1, TF32 = 2), both K-major, N >> 3 at bit 17 (the tile's width n,
// a multiple of 16 up to 256), M >> 4 at bit 24 (M = 128)
template <int KIND>
__host__ __device__ constexpr uint32_t umma_idesc(bool negate_a, int n) {
  constexpr uint32_t t = KIND == kKindTF32 ? 2u : 1u;
  return (1u << 4) | (t << 7) | (t << 10) | ((negate_a ? 1u : 0u) << 13) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

template <int KIND>
__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
  if constexpr (KIND == kKindTF32)
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
  else
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ bool term_negated(int code, int hL, int hR) {
  bool neg = (code & kSignNeg) != 0;
  if ((code & kSignHL) && hL < 0) neg = !neg;
  if ((code & kSignHR) && hR < 0) neg = !neg;
  return neg;
}

template <int S>
struct SliceProducts;
template <>
struct SliceProducts<2> {
  static constexpr int n = 3;
  __device__ static int a(int p) { return p == 2 ? 1 : 0; }
  __device__ static int b(int p) { return p == 1 ? 1 : 0; }
};
template <>
struct SliceProducts<3> {
  static constexpr int n = 6;
  // small products first: (2,0) (1,1) (0,2) (1,0) (0,1) (0,0)
  __device__ static int a(int p) { return (p == 0) ? 2 : (p == 1 || p == 3) ? 1 : 0; }
  __device__ static int b(int p) { return (p == 2) ? 2 : (p == 1 || p == 4) ? 1 : 0; }
};

// A stage holds S A boxes (128 rows) and S B tiles of WMAX rows (WMAX / 128 boxes each).
template <int S, int WMAX>
constexpr int stage_bytes() { return S * TILE_BYTES * (1 + WMAX / 128); }
template <int S, int WMAX>
constexpr int stages_for() {
  return (200 * 1024) / stage_bytes<S, WMAX>() > 4 ? 4 : (200 * 1024) / stage_bytes<S, WMAX>();
}
template <int S, int WMAX>
constexpr size_t smem_bytes() {
  return (size_t)stages_for<S, WMAX>() * stage_bytes<S, WMAX>() + 1024 /*align*/ + 256 /*barriers*/;
}

}  // namespace

// WMAX: the widest tile (128 or 256 columns); each tile carries its own width (TcTile::w), which
// goes into the instruction descriptor, so one launch mixes wide and narrow tiles.
template <int S, int KIND, int WMAX>
__global__ void __launch_bounds__(NUM_THREADS, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tmap, int64_t slice_rows, const TcProb* __restrict__ probs,
              const TcTile* __restrict__ tiles, int ntiles, TcOut out, int hL, int hR, int* err,
              unsigned long long wait_ns, int unarmed_it) {
  constexpr int ST = stages_for<S, WMAX>();
  static_assert(ST >= 2, "at least two pipeline stages");
  constexpr int NP = SliceProducts<S>::n;
  constexpr int BBYTES = TILE_BYTES * (WMAX / 128);  // one B slice of a stage
  constexpr int SBYTES = stage_bytes<S, WMAX>();
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* ring = smem;  // stage s: A slices [S] (16 KiB each), then B slices [S] (BBYTES each)
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)ST * SBYTES);
  uint64_t* empty = full + ST;
  uint64_t* tfull = empty + ST;
  uint64_t* tempty = tfull + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + 2);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  volatile int* consumed = reinterpret_cast<volatile int*>(tmem_slot + 2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < ST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(&tfull[a], 1);
      mbar_init(&tempty[a], 8);
    }
    *abort_flag = 0;
    *consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {  // 2 accumulators x WMAX FP32 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * WMAX)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      int it = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const TcTile tile = tiles[t];
        const TcProb& P = probs[tile.prob];
        const int nbox = (tile.w + 127) >> 7;  // B boxes of this tile (1, or 2 for tiles wider than 128)
        for (int term = 0; term < P.nterm && ok; ++term) {
          const int abase = P.t[term].a_tile + (tile.m0 / BM) * P.nkb;
          const int bbase = P.t[term].b_tile + (tile.n0 >> 7) * P.nkb;
          for (int kb = 0; kb < P.nkb; ++kb, ++it) {
            const int s = it % ST;
            if (!mbar_wait(&empty[s], ((it / ST) & 1) ^ 1, abort_flag, err, 1, wait_ns)) { ok = false; break; }
            // test switch (imsrg_test_unarmed_stage): CTA 0 leaves this stage unarmed -- no copy
            // is issued for it and nothing arrives on its barrier -- so the MMA warp's bounded
            // wait on it runs out
            if (it == unarmed_it && blockIdx.x == 0) continue;
            mbar_expect_tx(&full[s], (uint32_t)(S * (1 + nbox) * TILE_BYTES));
            uint8_t* stage = ring + (size_t)s * SBYTES;
            for (int sl = 0; sl < S; ++sl) {
              tma_load_2d(smem_u32(stage + (size_t)sl * TILE_BYTES), &tmap, 0,
                          (int)(sl * slice_rows + (int64_t)(abase + kb) * BM), &full[s]);
              for (int bx = 0; bx < nbox; ++bx)
                tma_load_2d(smem_u32(stage + (size_t)S * TILE_BYTES + (size_t)sl * BBYTES + (size_t)bx * TILE_BYTES),
                            &tmap, 0, (int)(sl * slice_rows + (int64_t)(bbase + bx * P.nkb + kb) * BM), &full[s]);
            }
          }
        }
      }
      if (!ok) {
        // drain: wait (bounded) for every issued stage the MMA warp did not consume
        const unsigned long long t0 = globaltimer();
        for (int j = *consumed; j < it; ++j) {
          while (!mbar_test(&full[j % ST], (j / ST) & 1)) {
            if (globaltimer() - t0 > wait_ns) break;
          }
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      int it = 0, local = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++local) {
        const TcTile tile = tiles[t];
        const TcProb& P = probs[tile.prob];
        const int acc = local & 1;
        if (!mbar_wait(&tempty[acc], ((local >> 1) & 1) ^ 1, abort_flag, err, 2, wait_ns)) { ok = false; break; }
        tc_fence_after();
        const uint32_t d_tmem = tmem_base + (uint32_t)(acc * WMAX);
        bool first = true;
        // the problem's fields in registers (the MMA asm clobbers memory); for a segmented K the
        // instruction descriptor of each segment, stepped by a counter of K steps (an MMA takes
        // 16 BF16 or 8 TF32 elements of K)
        constexpr int KSTEP = (KIND == kKindTF32) ? 8 : 16;
        const int nkb = P.nkb, nterm = P.nterm, seg_steps = P.kseg / KSTEP;
        uint32_t sd0 = 0, sd1 = 0, sd2 = 0, sd3 = 0;
        if (seg_steps) {
          sd0 = umma_idesc<KIND>(term_negated(P.t[0].sign, hL, hR), tile.w);
          sd1 = umma_idesc<KIND>(term_negated(P.t[1].sign, hL, hR), tile.w);
          sd2 = umma_idesc<KIND>(term_negated(P.t[2].sign, hL, hR), tile.w);
          sd3 = umma_idesc<KIND>(term_negated(P.t[3].sign, hL, hR), tile.w);
        }
        for (int term = 0; term < nterm && ok; ++term) {
          const uint32_t idesc = umma_idesc<KIND>(term_negated(P.t[term].sign, hL, hR), tile.w);
          int segi = 0, left = seg_steps;
          for (int kb = 0; kb < nkb; ++kb, ++it) {
            uint32_t idk[kMmaPerRow];
#pragma unroll
            for (int ks = 0; ks < kMmaPerRow; ++ks) {
              idk[ks] = seg_steps ? (segi == 0 ? sd0 : segi == 1 ? sd1 : segi == 2 ? sd2 : sd3) : idesc;
              if (seg_steps && --left == 0) {  // K past the fourth segment is zero padding
                segi = min(segi + 1, 3);
                left = seg_steps;
              }
            }
            const int s = it % ST;
            if (!mbar_wait(&full[s], (it / ST) & 1, abort_flag, err, 3, wait_ns)) { ok = false; break; }
            tc_fence_after();
            const uint32_t stage = smem_u32(ring + (size_t)s * SBYTES);
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              const uint32_t a0 = stage + (uint32_t)(SliceProducts<S>::a(p) * TILE_BYTES);
              const uint32_t b0 = stage + (uint32_t)(S * TILE_BYTES + SliceProducts<S>::b(p) * BBYTES);
#pragma unroll
              for (int ks = 0; ks < kMmaPerRow; ++ks) {
                umma<KIND>(d_tmem, umma_desc(a0 + ks * 32), umma_desc(b0 + ks * 32), idk[ks], first ? 0u : 1u);
                first = false;
              }
            }
            umma_commit(&empty[s]);  // frees the stage once these MMAs have read it
            *consumed = it + 1;
          }
        }
        if (ok) umma_commit(&tfull[acc]);
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue (warps 2..9)
    const int quad = warp & 3;          // TMEM lanes 32*quad .. 32*quad+31
    const int half = (warp - 2) >> 2;   // accumulator columns 32*(2c+half) .. +31, c = 0, 1, ...
    int local = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++local) {
      const TcTile tile = tiles[t];
      const TcProb& P = probs[tile.prob];
      const int acc = local & 1;
      if (!mbar_wait(&tfull[acc], (local >> 1) & 1, abort_flag, err, 4, wait_ns)) break;
      tc_fence_after();
      const int m = tile.m0 + quad * 32 + lane;
      for (int c0 = half * 32; c0 < tile.w; c0 += 64) {
        uint32_t r[32];
        tmem_ld32(tmem_base + (uint32_t)(acc * WMAX + c0) + ((uint32_t)(quad * 32) << 16), r);
        if (m < P.M) {
          if (P.out_f32) {
            float* C = (P.out_f32 == 1 ? out.f32 : out.f32b) + P.c_off;
            // the columns of this warp's 32-row segment that anything reads (one bit each)
            // (m < M here; a chunk at or past column N stores nothing and reads no mask word)
            unsigned keep = 0xffffffffu;
            if (P.xmask)
              keep = tile.n0 + c0 < P.N ? __ldg(out.xmask + (P.xmask - 1) + ((tile.m0 >> 5) + quad) * ((P.N + 31) >> 5) +
                                                ((tile.n0 + c0) >> 5))
                                        : 0u;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const int n = tile.n0 + c0 + j;
              if (n < P.N && ((keep >> j) & 1u)) C[m + (int64_t)n * P.ldc] = __uint_as_float(r[j]);
            }
          } else if (out.w1f && P.c_id == kOpW1) {
            float* C = out.w1f + P.c_off;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const int n = tile.n0 + c0 + j;
              if (n < P.N) C[m + (int64_t)n * P.ldc] = __uint_as_float(r[j]);
            }
          } else {
            double* C = out.f64[P.c_id] + P.c_off;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const int n = tile.n0 + c0 + j;
              if (n < P.N) C[m + (int64_t)n * P.ldc] = f32_to_f64(__uint_as_float(r[j]));
            }
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[acc]);
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  __syncwarp();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(2 * WMAX) : "memory");
}

// ---------------------------------------------------------------- operand split
// Chunked split: one block per run of rows of one operand, each thread converts 8
// consecutive k of one row and writes them as one vector (16 bytes of BF16, 32 of TF32) into
// every slice.  T: the operand type (split.cuh).
template <int S, typename T>
__global__ void __launch_bounds__(256) k_split_chunks(const TcSplitOp* __restrict__ ops,
                                                      const SplitChunk* __restrict__ chunks,
                                                      const double* __restrict__ L, const double* __restrict__ R,
                                                      void* __restrict__ bufv, int64_t slice_elems) {
  T* buf = static_cast<T*>(bufv);
  const SplitChunk ch = chunks[blockIdx.x];
  const TcSplitOp o = ops[ch.op];
  const double* src = (o.src == 0 ? L : R) + o.src_off;
  const int nvec = (o.K + 7) >> 3;
  const int nr = ch.r1 - ch.r0;
  const int total = nr * nvec;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    // rows fastest for transposed sources (coalesced reads down a column), K fastest otherwise
    const int r = o.trans ? ch.r0 + t % nr : ch.r0 + t / nvec;
    const int k0 = (o.trans ? t / nr : t - (r - ch.r0) * nvec) << 3;
    float x[8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
      x[u] = (k0 + u < o.K)
                 ? f64_to_f32(o.trans ? src[r + (int64_t)(k0 + u) * o.ld] : src[k0 + u + (int64_t)r * o.K])
                 : 0.0f;
    const int64_t dst = split_offset<T>(o.tile_base, o.nkb, r, k0);
#pragma unroll
    for (int sl = 0; sl < S; ++sl) {
      __align__(32) T h[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) h[u] = SplitElem<T>::take(x[u]);
      uint4* d = reinterpret_cast<uint4*>(buf + sl * slice_elems + dst);
#pragma unroll
      for (int v = 0; v < (int)(8 * sizeof(T) / 16); ++v) d[v] = reinterpret_cast<const uint4*>(h)[v];
    }
  }
}

// ---------------------------------------------------------------- small-K FP32 GEMM
// The K = nhh problems of 222_pp_hh (every W2 product): FP32 SIMT, FP64 in and out.
// C = sum of alpha op(A) op(B) in FP32 on the SIMT cores, stored as TO (double, or float at
// the same element offsets of the output buffer)
template <typename TO>
__device__ __forceinline__ void gemm_f32_tile(const GemmProb* __restrict__ probs, const GemmTile* __restrict__ tiles,
                                              const GemmOperands& ops) {
  __shared__ float As[16][65];
  __shared__ float Bs[16][65];
  const GemmTile tile = tiles[blockIdx.x];
  const GemmProb& P = probs[tile.prob];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  float acc[4][4] = {};
  for (int t = 0; t < P.nterm; ++t) {
    const GemmTerm& T = P.t[t];
    const double* A = ops.in[T.a_id] + T.a_off;
    const double* B = ops.in[T.b_id] + T.b_off;
    const int sel = T.alpha & 3;
    float alpha = (sel == kAlphaHL) ? (float)ops.hL : (sel == kAlphaHR ? (float)ops.hR : 1.0f);
    if (T.alpha & kAlphaNeg) alpha = -alpha;
    for (int k0 = 0; k0 < T.K; k0 += 16) {
#pragma unroll
      for (int s = 0; s < 4; ++s) {
        int m, k;
        if (T.ta == 0) { m = tid & 63; k = (tid >> 6) + 4 * s; }
        else { k = tid & 15; m = (tid >> 4) + 16 * s; }
        const int gm = tile.m0 + m, gk = k0 + k;
        double v = 0.0;
        if (gm < P.M && gk < T.K) v = T.ta == 0 ? A[gm + (int64_t)gk * T.lda] : A[gk + (int64_t)gm * T.lda];
        As[k][m] = alpha * (float)v;
        int n;
        if (T.tb == 0) { k = tid & 15; n = (tid >> 4) + 16 * s; }
        else { n = tid & 63; k = (tid >> 6) + 4 * s; }
        const int gn = tile.n0 + n, gk2 = k0 + k;
        double w = 0.0;
        if (gn < P.N && gk2 < T.K) w = T.tb == 0 ? B[gk2 + (int64_t)gn * T.ldb] : B[gn + (int64_t)gk2 * T.ldb];
        Bs[k][n] = (float)w;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < 16; ++kk) {
        float a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
      }
      __syncthreads();
    }
  }
  TO* C = reinterpret_cast<TO*>(ops.out[P.c_id]) + P.c_off;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gm = tile.m0 + tx + 16 * i, gn = tile.n0 + ty + 16 * j;
      if (gm < P.M && gn < P.N) C[gm + (int64_t)gn * P.ldc] = (TO)acc[i][j];
    }
}
__global__ void __launch_bounds__(256) k_gemm_f32(const GemmProb* __restrict__ probs, const GemmTile* __restrict__ tiles,
                                                  GemmOperands ops) {
  gemm_f32_tile<double>(probs, tiles, ops);
}
// the same with FP32 outputs (the mixed commutator's W2)
__global__ void __launch_bounds__(256) k_gemm_f32_w(const GemmProb* __restrict__ probs,
                                                    const GemmTile* __restrict__ tiles, GemmOperands ops) {
  gemm_f32_tile<float>(probs, tiles, ops);
}

}  // namespace imsrg

// ====================================================================== host side
using namespace imsrg;

namespace imsrg {

cudaError_t tc_gemm_smem_attrs(int S, int kind);

struct TcState {
  int S = 0;
  int kind = kKindBF16;  // operand type of the slices (TcKind)
  int tile_k = 64;       // K values per 128-byte tile row: 64 BF16, 32 TF32
  void* buf = nullptr;
  int64_t slice_rows = 0, slice_elems = 0;
  int total_tiles = 0;
  CUtensorMap tmap;
  // 222_pp_hh: split table, K = npp products on tensor cores, K = nhh products on FP32 SIMT
  std::vector<TcSplitOp> split_ops;
  std::vector<int64_t> split_prefix;
  std::vector<TcProb> pphh_probs;
  std::vector<TcTile> pphh_tiles;
  std::vector<GemmProb> small_probs;
  std::vector<GemmTile> small_tiles;
  // particle-hole: X(q) = phi phi Z - pm Zs with Z(q) = hL LCC RCC^T - hR RCC LCC^T (recouple.cu)
  std::vector<int> cc_tile_A, cc_tile_B, cc_nkb, cc_seg, swap_row;
  std::vector<TcProb> z_probs;
  std::vector<TcTile> z_tiles;
  void* d_mem = nullptr;
  const TcSplitOp* d_split_ops = nullptr;
  const int64_t* d_split_prefix = nullptr;
  const TcProb* d_pphh_probs = nullptr;
  const TcTile* d_pphh_tiles = nullptr;
  const GemmProb* d_small_probs = nullptr;
  const GemmTile* d_small_tiles = nullptr;
  const TcProb* d_z_probs = nullptr;
  const TcTile* d_z_tiles = nullptr;
  std::vector<PandyaChunk> pandya_chunks;  // chunks of the cross-coupled channels for k_pandya_tc
  const PandyaChunk* d_pandya_chunks = nullptr;
  const int* d_cc_tile_A = nullptr;
  const int* d_cc_tile_B = nullptr;
  const int* d_cc_nkb = nullptr;
  const int* d_cc_seg = nullptr;
  const int* d_swap_row = nullptr;
  float* zbuf = nullptr;  // X, the recoupling input (FP32, wcc layout)
  int* d_err = nullptr;
  // orbit quadruples (i<=j, k<=l) of the particle-hole recoupling, j fastest
  std::vector<uint64_t> quads;
  const uint64_t* d_quads = nullptr;
  std::vector<int> xcol;              // X column offset of every pair and J' (recouple.cu)
  std::vector<unsigned> xmask;        // the X elements the recoupling reads (store masks, recouple.cu)
  const unsigned* d_xmask = nullptr;
  const int* d_xcol = nullptr;
  int recouple_minb = 6;              // launch-bounds variant of k_recouple_q
  int recouple_ctas = 0;              // CTAs of k_recouple_q
  std::vector<SplitChunk> chunks;
  const SplitChunk* d_chunks = nullptr;
  // commutator_122 by pair-group sub-blocks (comm122.cu): the plan, its launch order for the
  // current caps (tc_g122_partition) and its device copies (tasks and runs sized for all tasks)
  G122Plan g122;
  G122Task* d_g122_tasks = nullptr;
  int2* d_g122_items = nullptr;
  const unsigned* d_g122_codes = nullptr;
  int* d_g122_counter = nullptr;
  PairGroupsDev g122_w{};
  int g122_nspb = 0, g122_nblk2 = 0, g122_per_sm = 1;
  // tuned launch parameters (imsrg_autotune): GEMM tile order and shape
  int gemm_order = 0;  // 0: longest K first, 1: problem order
  // tile shape of each list: widest output tile (128 or 256 columns) and narrow last column
  // tiles (only as wide as needed, a multiple of 16): [0] ladder, [1] X, [2] merged
  int wmax[3] = {128, 128, 128};
  bool narrow[3] = {true, true, true};
  bool merged = true;  // ladder and X products in one launch (else two launches)
  // the merged list of one commutator: the K = npp ladder problems, then the X problems, in one
  // persistent launch (tile lists in device memory sized for the largest tile count)
  std::vector<TcProb> all_probs;
  std::vector<TcTile> all_tiles;
  const TcProb* d_all_probs = nullptr;
  TcTile* d_tile_mem = nullptr;  // [pphh tiles | X tiles | merged tiles]
  size_t tile_cap_pphh = 0, tile_cap_z = 0, tile_cap_all = 0;
  std::vector<int> g_start, g_n, g_orb, g_b1, g_b2, g_blk_off;
  float2* g122_fb = nullptr;  // (fL, fR)(x, y) on every (l, j, tz) block
  int num_sms = 148;
};

}  // namespace imsrg

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int ceil_div(int a, int b) { return (a + b - 1) / b; }

// the output tiles of a problem list: 128 rows by up to wmax columns (narrow: the last
// column tile only as wide as its columns need, in steps of 16), longest K first
// whether any element of the tile (rows m0.., columns n0.. n0 + w - 1) is to be stored: always,
// unless the problem has a store mask (TcProb::xmask) with no bit set in the tile
bool tile_stored(const TcProb& P, const std::vector<unsigned>* mask, int m0, int n0, int w) {
  if (!P.xmask || !mask) return true;
  const int nwc = (P.N + 31) >> 5;
  for (int b = m0 >> 5; b < std::min((m0 + BM + 31) >> 5, (P.M + 31) >> 5); ++b)
    for (int c = n0 >> 5; c < std::min((n0 + w + 31) >> 5, nwc); ++c)
      if ((*mask)[(size_t)(P.xmask - 1) + (size_t)b * nwc + c]) return true;
  return false;
}

std::vector<TcTile> make_tiles(const std::vector<TcProb>& probs, int wmax, bool narrow,
                               const std::vector<unsigned>* mask = nullptr) {
  std::vector<TcTile> t;
  for (int p = 0; p < (int)probs.size(); ++p)
    for (int m0 = 0; m0 < probs[p].M; m0 += BM)
      for (int n0 = 0; n0 < probs[p].N; n0 += wmax) {
        const int w = tc_tile_width(probs[p].N, n0, wmax, narrow);
        if (tile_stored(probs[p], mask, m0, n0, w)) t.push_back(TcTile{p, m0, n0, w});
      }
  std::stable_sort(t.begin(), t.end(), [&](const TcTile& a, const TcTile& b) {
    return probs[a.prob].nkb * probs[a.prob].nterm > probs[b.prob].nkb * probs[b.prob].nterm;
  });
  return t;
}

struct DevPacker {
  std::vector<char> buf;
  std::vector<std::pair<size_t, const void**>> fix;
  template <class T>
  void add(const std::vector<T>& v, const T** dst) {
    size_t o = (buf.size() + 255) & ~size_t(255);
    buf.resize(o + std::max<size_t>(v.size() * sizeof(T), 1));
    if (!v.empty()) std::memcpy(buf.data() + o, v.data(), v.size() * sizeof(T));
    fix.push_back({o, reinterpret_cast<const void**>(dst)});
  }
};

}  // namespace

void Ctx::tc_release() {
  if (!tc) return;
  if (tc->buf) cudaFree(tc->buf);
  if (tc->d_mem) cudaFree(tc->d_mem);
  if (tc->zbuf) cudaFree(tc->zbuf);
  if (tc->d_err) cudaFree(tc->d_err);
  if (tc->g122_fb) cudaFree(tc->g122_fb);
  if (tc->d_g122_tasks) cudaFree(tc->d_g122_tasks);
  if (tc->d_g122_items) cudaFree(tc->d_g122_items);
  if (tc->d_g122_counter) cudaFree(tc->d_g122_counter);
  if (tc->d_tile_mem) cudaFree(tc->d_tile_mem);
  delete tc;
  tc = nullptr;
}

imsrg_status Ctx::tc_prepare(int mode) {
  const int S = (mode == IMSRG_PREC_BF16X6) ? 3 : 2;
  const int kind = (mode == IMSRG_PREC_TF32X3) ? kKindTF32 : kKindBF16;
  if (tc && tc->S == S && tc->kind == kind) return IMSRG_OK;
  tc_release();
  int cc_major = 0;
  cudaDeviceGetAttribute(&cc_major, cudaDevAttrComputeCapabilityMajor, device);
  if (cc_major < 10) return fail(IMSRG_ERR_UNSUPPORTED, "tensor-core path needs a Blackwell (sm_10x) GPU");
  tc = new TcState();
  tc->S = S;
  tc->kind = kind;
  tc->tile_k = kind == kKindTF32 ? 32 : 64;
  const int BK = tc->tile_k;
  cudaDeviceGetAttribute(&tc->num_sms, cudaDevAttrMultiProcessorCount, device);
  const Layout& l = L;
  int tiles = 0;
  // ---- 222_pp_hh operands: columns of gam(1..3) of L and R, K = npp
  // operand index: [q][src][g]  (g = 0 pppp, 1 ppph, 2 pphh)
  std::vector<int> opnd_tile(l.nblocks * 6, -1);
  for (int q = 0; q < l.nblocks; ++q) {
    const int np = l.ncls[q][0];
    if (np == 0) continue;
    for (int src = 0; src < 2; ++src)
      for (int g = 0; g < 3; ++g) {
        const int cols = l.gn2[q * 6 + g];
        if (cols == 0) continue;
        TcSplitOp o{};
        o.src = src;
        o.src_off = l.goff[q * 6 + g];
        o.rows = cols;
        o.K = np;
        o.nkb = ceil_div(np, BK);
        o.tile_base = tiles;
        opnd_tile[q * 6 + src * 3 + g] = tiles;
        tiles += ceil_div(cols, BM) * o.nkb;
        tc->split_ops.push_back(o);
      }
  }
  for (int op = 0; op < (int)tc->split_ops.size(); ++op) {
    const TcSplitOp& o = tc->split_ops[op];
    const int rows_per = std::max(1, 4096 / std::max(o.K, 1));
    for (int r0 = 0; r0 < o.rows; r0 += rows_per) tc->chunks.push_back(SplitChunk{op, r0, std::min(o.rows, r0 + rows_per)});
  }
  tc->split_prefix.push_back(0);
  for (auto& o : tc->split_ops) tc->split_prefix.push_back(tc->split_prefix.back() + (int64_t)o.rows * o.K);
  auto T = [&](int q, int src, int g) { return opnd_tile[q * 6 + src * 3 + g]; };
  const int hl = kSignHL, hr = kSignHR, ng = kSignNeg;
  for (int q = 0; q < l.nblocks; ++q) {
    const int np = l.ncls[q][0], nb = l.ncls[q][1], nh = l.ncls[q][2];
    if (np == 0) continue;
    const int nkb = ceil_div(np, BK);
    auto prob = [&](int M, int N, int g_out, int ldc, TcTermDesc t0, int nt, TcTermDesc t1) {
      TcProb p{};
      p.M = M; p.N = N; p.nkb = nkb; p.nterm = nt;
      p.t[0] = t0; p.t[1] = t1;
      p.out_f32 = 0; p.c_id = kOpW1; p.c_off = l.goff[q * 6 + g_out]; p.ldc = ldc;
      tc->pphh_probs.push_back(p);
    };
    // rows of op(A) are columns of the stored array; when op(A) is a square array itself,
    // its rows are herm * its columns (the sign joins the term's sign).
    // W1_pppp = L_pppp . R_pppp
    prob(np, np, 0, np, TcTermDesc{T(q, 0, 0), T(q, 1, 0), hl}, 1, TcTermDesc{});
    if (nh) {
      // W1_hhhh = hL L_pphh^T . R_pphh
      prob(nh, nh, 4, nh, TcTermDesc{T(q, 0, 2), T(q, 1, 2), hl}, 1, TcTermDesc{});
      // W1_pphh = L_pppp . R_pphh - R_pppp . L_pphh
      prob(np, nh, 2, np, TcTermDesc{T(q, 0, 0), T(q, 1, 2), hl}, 2, TcTermDesc{T(q, 1, 0), T(q, 0, 2), ng | hr});
    }
    if (nb) {
      // W1_phph = hL L_ppph^T . R_ppph
      prob(nb, nb, 3, nb, TcTermDesc{T(q, 0, 1), T(q, 1, 1), hl}, 1, TcTermDesc{});
      // W1_ppph = L_pppp . R_ppph - R_pppp . L_ppph
      prob(np, nb, 1, np, TcTermDesc{T(q, 0, 0), T(q, 1, 1), hl}, 2, TcTermDesc{T(q, 1, 0), T(q, 0, 1), ng | hr});
    }
    if (nb && nh) {
      // W1_phhh = hL L_ppph^T . R_pphh - hR R_ppph^T . L_pphh
      prob(nb, nh, 5, nb, TcTermDesc{T(q, 0, 1), T(q, 1, 2), hl}, 2, TcTermDesc{T(q, 1, 1), T(q, 0, 2), ng | hr});
    }
  }
  // K = nhh products (all W2 arrays), from the FP64 problem list
  for (const GemmProb& p : pphh_probs)
    if (p.c_id == kOpW2) tc->small_probs.push_back(p);
  tc->small_tiles = build_tiles(tc->small_probs, 64, 64);

  // ---- particle-hole: LCC / RCC rows r, K = nph, written by the Pandya pass with the row
  //      sign phi(r), and the same rows unsigned at the swapped position (row r(a,b) holding
  //      row r(b,a)): phiL, phiR, Ls, Rs.  One FP32 product per channel,
  //        X = hL phiL phiR^T - hR phiR phiL^T - hR Ls Rs^T + hL Rs Ls^T
  //          = phi phi Z - pm Z(s, s),   Z = hL LCC RCC^T - hR RCC LCC^T, pm = hL hR,
  //      is the input of the recoupling (recouple.cu).  The four terms are one product over a
  //      K of four segments, each nph rounded up to 16: A = [phiL | phiR | Ls | Rs] and
  //      B = [phiR | phiL | Rs | Ls], the segment signs (hL, -hR, -hR, hL) in the MMAs, so K is
  //      padded to whole tiles once instead of once per term.
  tc->cc_tile_A.assign(l.ncc, 0);
  tc->cc_tile_B.assign(l.ncc, 0);
  tc->cc_nkb.assign(l.ncc, 0);
  tc->cc_seg.assign(l.ncc, 0);
  tc->swap_row.assign(std::max<size_t>(l.cc_ra.size(), 1), 0);
  for (int q = 0; q < l.ncc; ++q)
    for (int r = 0; r < l.cc_rlen[q]; ++r) {
      const int a = l.cc_ra[l.cc_row_off[q] + r], b = l.cc_rb[l.cc_row_off[q] + r];
      const int rs = l.ccr[((size_t)b * l.N + a) * l.NJ + l.cc_J[q] / 2];
      if (rs < 0) return fail(IMSRG_ERR_MISMATCH, "swapped pair outside its cross-coupled channel");
      tc->swap_row[l.cc_row_off[q] + r] = rs;
    }
  for (int q = 0; q < l.ncc; ++q) {
    const int r = l.cc_rlen[q], nb = l.cc_nph[q];
    if (r == 0 || nb == 0) continue;
    const int seg = ceil_div(nb, 16) * 16;
    const int nkb = ceil_div(4 * seg, BK);
    const int blk = ceil_div(r, BM) * nkb;
    tc->cc_nkb[q] = nkb;
    tc->cc_seg[q] = seg;
    tc->cc_tile_A[q] = tiles; tiles += blk;
    tc->cc_tile_B[q] = tiles; tiles += blk;
    TcProb p{};
    p.M = r; p.N = r; p.nkb = nkb; p.nterm = 1; p.kseg = seg;
    p.t[0] = TcTermDesc{tc->cc_tile_A[q], tc->cc_tile_B[q], hl};
    p.t[1] = TcTermDesc{0, 0, ng | hr};
    p.t[2] = TcTermDesc{0, 0, ng | hr};
    p.t[3] = TcTermDesc{0, 0, hl};
    p.out_f32 = 1;
    p.c_id = 0; p.c_off = l.wcc_off[q]; p.ldc = r;
    tc->z_probs.push_back(p);
  }
  tc->total_tiles = tiles;
  if (l.JM + 1 > 26) return fail(IMSRG_ERR_UNSUPPORTED, "mixed recoupling supports 2j <= 25 (eMax <= 12)");
  // ---- Pandya chunks: at most 1024 elements of one cross-coupled channel each (both operators)
  for (int q = 0; q < l.ncc; ++q) {
    const int64_t n = l.cc_off[q + 1] - l.cc_off[q];
    const int nph = l.cc_nph[q];
    if (n <= 0) continue;
    if (n * (int64_t)nph >= (1ll << 32)) return fail(IMSRG_ERR_UNSUPPORTED, "cross-coupled channel too large");
    const unsigned m = (unsigned)(((1ull << 32) + (unsigned)nph - 1) / (unsigned)nph);
    for (int64_t e0 = 0; e0 < n; e0 += 1024)
      tc->pandya_chunks.push_back(PandyaChunk{q, (int)e0, (int)std::min<int64_t>(1024, n - e0), m});
  }
  // ---- commutator_122 tasks: the group pairs G1 <= G2 of each channel
  {
    PairGroups pg;
    build_pair_groups(pg, l);
    tc->g_start = pg.spb_start; tc->g_n = pg.spb_n; tc->g_orb = pg.spb_orb;
    tc->g_b1 = pg.grp_b1; tc->g_b2 = pg.grp_b2; tc->g_blk_off = pg.blk_off;
    tc->g122_nspb = pg.nspb;
    tc->g122_nblk2 = pg.nblk2;
    const std::string e = build_g122_plan(l, pg, tc->g122);
    if (!e.empty()) return fail(IMSRG_ERR_UNSUPPORTED, e);
  }
  // ---- recoupling quadruples: bra (i<=j) of class c1, ket (k<=l) of class c2, with
  //      c1 < c2, or c1 == c2 and (i,j) <= (k,l) (the unique stored elements), matching
  //      2Tz and parity and sharing at least one J
  {
    const int N = l.N;
    std::vector<std::vector<int>> by_tp(4);  // orbits grouped by (tz, l parity)
    for (int o = 0; o < N; ++o) by_tp[((l.tz[o] + 1) / 2) * 2 + (l.ll[o] & 1)].push_back(o);
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < N; ++k)
        for (int ll2 = k; ll2 < N; ++ll2) {
          const int tzj = l.tz[k] + l.tz[ll2] - l.tz[i];
          if (tzj != -1 && tzj != 1) continue;
          const int par = ((l.ll[k] + l.ll[ll2] - l.ll[i]) % 2 + 2) % 2;
          const int c2 = l.con[k] + l.con[ll2];
          const int kl_lo = std::abs(l.jj[k] - l.jj[ll2]), kl_hi = l.jj[k] + l.jj[ll2];
          for (int j : by_tp[((tzj + 1) / 2) * 2 + par]) {
            if (j < i) continue;
            const int c1 = l.con[i] + l.con[j];
            if (c1 > c2) continue;
            if (c1 == c2 && (i > k || (i == k && j > ll2))) continue;
            const int lo = std::max(std::abs(l.jj[i] - l.jj[j]), kl_lo), hi = std::min(l.jj[i] + l.jj[j], kl_hi);
            if (lo > hi) continue;
            tc->quads.push_back((uint64_t)i | ((uint64_t)j << 16) | ((uint64_t)k << 32) | ((uint64_t)ll2 << 48));
          }
        }
    // within the quadruples of one orbit i, by (jj, jk, jl): neighbouring threads then share their J and J' ranges and
    // 6j rows, so a warp's loops run with its lanes in step (the X rows read for one i are the same in any order)
    auto shape = [&](uint64_t qd) {
      return (l.jj[(qd >> 16) & 0xFFFF] * 64 + l.jj[(qd >> 32) & 0xFFFF]) * 64 + l.jj[(qd >> 48) & 0xFFFF];
    };
    for (size_t a = 0; a < tc->quads.size();) {
      size_t b = a;
      while (b < tc->quads.size() && (tc->quads[b] & 0xFFFF) == (tc->quads[a] & 0xFFFF)) ++b;
      std::stable_sort(tc->quads.begin() + a, tc->quads.begin() + b,
                       [&](uint64_t x, uint64_t y) { return shape(x) < shape(y); });
      a = b;
    }
  }
  // X stores only where the recoupling reads: the masks of the 32-row column segments
  {
    std::vector<int> moff;
    tc->xmask = build_x_read_mask(l, tc->quads, moff);
    for (TcProb& p : tc->z_probs)
      for (int q = 0; q < l.ncc; ++q)
        if (l.cc_rlen[q] == p.M && l.wcc_off[q] == p.c_off && moff[q] >= 0) p.xmask = moff[q] + 1;
  }
  tc->slice_rows = (int64_t)tiles * BM;
  tc->slice_elems = tc->slice_rows * BK;
  if ((int64_t)S * tc->slice_rows >= (int64_t)1 << 31) return fail(IMSRG_ERR_UNSUPPORTED, "operand buffer too large for 32-bit TMA rows");

  const size_t bytes = (size_t)tc_elem_bytes() * (size_t)S * tc->slice_elems;
  CK_TC(cuda(cudaMalloc(&tc->buf, std::max<size_t>(bytes, 256)), "cudaMalloc(tc operands)"));
  CK_TC(cuda(cudaMemset(tc->buf, 0, std::max<size_t>(bytes, 256)), "memset(tc operands)"));
  CK_TC(cuda(cudaMalloc(&tc->zbuf, sizeof(float) * std::max<int64_t>(l.wcc_size, 1)), "cudaMalloc(X)"));
  CK_TC(cuda(cudaMemset(tc->zbuf, 0, sizeof(float) * std::max<int64_t>(l.wcc_size, 1)), "memset(X)"));
  CK_TC(cuda(cudaMalloc(&tc->d_err, sizeof(int)), "cudaMalloc(err)"));
  CK_TC(cuda(cudaMalloc(&tc->g122_fb, sizeof(float2) * std::max(tc->g122_nblk2, 1)), "cudaMalloc(122 blocks)"));
  CK_TC(cuda(cudaMemset(tc->d_err, 0, sizeof(int)), "memset(err)"));
  DevPacker pk;
  pk.add(tc->split_ops, &tc->d_split_ops);
  pk.add(tc->split_prefix, &tc->d_split_prefix);
  pk.add(tc->pphh_probs, &tc->d_pphh_probs);
  pk.add(tc->small_probs, &tc->d_small_probs);
  pk.add(tc->small_tiles, &tc->d_small_tiles);
  pk.add(tc->z_probs, &tc->d_z_probs);
  tc->all_probs = tc->pphh_probs;
  for (TcProb p : tc->z_probs) tc->all_probs.push_back(p);
  pk.add(tc->all_probs, &tc->d_all_probs);
  pk.add(tc->cc_tile_A, &tc->d_cc_tile_A);
  pk.add(tc->pandya_chunks, &tc->d_pandya_chunks);
  pk.add(tc->cc_tile_B, &tc->d_cc_tile_B);
  pk.add(tc->cc_nkb, &tc->d_cc_nkb);
  pk.add(tc->cc_seg, &tc->d_cc_seg);
  pk.add(tc->swap_row, &tc->d_swap_row);
  pk.add(tc->quads, &tc->d_quads);
  tc->xcol = build_xcol(l);
  pk.add(tc->xcol, &tc->d_xcol);
  pk.add(tc->xmask, &tc->d_xmask);
  pk.add(tc->chunks, &tc->d_chunks);
  pk.add(tc->g_start, &tc->g122_w.spb_start);
  pk.add(tc->g_n, &tc->g122_w.spb_n);
  pk.add(tc->g_orb, &tc->g122_w.spb_orb);
  pk.add(tc->g_b1, &tc->g122_w.grp_b1);
  pk.add(tc->g_b2, &tc->g122_w.grp_b2);
  pk.add(tc->g_blk_off, &tc->g122_w.blk_off);
  pk.add(tc->g122.codes, &tc->d_g122_codes);

  CK_TC(cuda(cudaMalloc(&tc->d_mem, pk.buf.size()), "cudaMalloc(tc tables)"));
  CK_TC(cuda(cudaMemcpy(tc->d_mem, pk.buf.data(), pk.buf.size(), cudaMemcpyHostToDevice), "cudaMemcpy(tc tables)"));
  for (auto& f : pk.fix) *f.second = static_cast<const char*>(tc->d_mem) + f.first;
  CK_TC(cuda(cudaMalloc(&tc->d_g122_tasks, sizeof(G122Task) * std::max<size_t>(tc->g122.all.size(), 1)),
             "cudaMalloc(122 tasks)"));
  CK_TC(cuda(cudaMalloc(&tc->d_g122_items, sizeof(int2) * std::max<size_t>(tc->g122.all.size(), 1)),
             "cudaMalloc(122 runs)"));
  CK_TC(cuda(cudaMalloc(&tc->d_g122_counter, sizeof(int)), "cudaMalloc(122 counter)"));
  CK_TC(cuda(cudaMemset(tc->d_g122_counter, 0, sizeof(int)), "cudaMemset(122 counter)"));
  CK_TC(tc_g122_partition(tc->g122.tiny_cap, tc->g122.warp_cap));
  tc->recouple_ctas = tc->num_sms * 32;
  // tile lists: the most tiles come with 128-wide tiles
  tc->tile_cap_pphh = make_tiles(tc->pphh_probs, 128, false).size();
  tc->tile_cap_z = make_tiles(tc->z_probs, 128, false).size();
  tc->tile_cap_all = tc->tile_cap_pphh + tc->tile_cap_z;
  CK_TC(cuda(cudaMalloc(&tc->d_tile_mem, sizeof(TcTile) * std::max<size_t>(tc->tile_cap_all * 2, 1)),
             "cudaMalloc(GEMM tiles)"));
  tc->d_pphh_tiles = tc->d_tile_mem;
  tc->d_z_tiles = tc->d_tile_mem + tc->tile_cap_pphh;
  CK_TC(tc_set_tiles(tc->wmax, tc->narrow, tc->gemm_order));

  // tensor map over the whole operand buffer: rows of 64 bf16 (128 bytes), box 64 x 128
  CK_TC(tc_encode_map(&tc->tmap, tc->buf, (int64_t)S * tc->slice_rows));
  CK_TC(cuda(tc_gemm_smem_attrs(S, kind), "smem attr (tensor-core GEMM)"));
  return IMSRG_OK;
}

imsrg_status Ctx::tc_gemm(const TcProb* probs, const TcTile* tiles, int ntiles, TcOut out, int hL, int hR, int wmax) {
  return tc_gemm_on(tc->tmap, tc->slice_rows, probs, tiles, ntiles, out, hL, hR, wmax);
}

int Ctx::tc_slices() const { return tc ? tc->S : 0; }
int Ctx::tc_tile_k() const { return tc ? tc->tile_k : 64; }
int Ctx::tc_elem_bytes() const { return (tc && tc->kind == kKindTF32) ? 4 : 2; }
int Ctx::tc_kind() const { return tc ? tc->kind : kKindBF16; }

namespace {
template <int S, int KIND, int WMAX>
void launch_tc_gemm(int grid, cudaStream_t st, const CUtensorMap& map, int64_t slice_rows, const TcProb* probs,
                    const TcTile* tiles, int ntiles, TcOut out, int hL, int hR, int* err, unsigned long long wait_ns,
                    int unarmed) {
  k_tc_gemm<S, KIND, WMAX><<<grid, NUM_THREADS, smem_bytes<S, WMAX>(), st>>>(map, slice_rows, probs, tiles, ntiles,
                                                                           out, hL, hR, err, wait_ns, unarmed);
}
template <int S, int KIND, int WMAX>
cudaError_t set_gemm_smem() {
  return cudaFuncSetAttribute(k_tc_gemm<S, KIND, WMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)smem_bytes<S, WMAX>());
}
}  // namespace

// the kernel instances of one slice count and operand type: widest tile 128, and 256 where two
// stages of S x (16 + 32) KiB fit (S = 2)
cudaError_t imsrg::tc_gemm_smem_attrs(int S, int kind) {
  cudaError_t e;
  if (kind == kKindTF32) {
    if ((e = set_gemm_smem<2, kKindTF32, 128>()) != cudaSuccess) return e;
    return set_gemm_smem<2, kKindTF32, 256>();
  }
  if (S == 3) return set_gemm_smem<3, kKindBF16, 128>();
  if ((e = set_gemm_smem<2, kKindBF16, 128>()) != cudaSuccess) return e;
  return set_gemm_smem<2, kKindBF16, 256>();
}

// the persistent tensor-core GEMM over any operand buffer of this context's slice count and
// operand type; the tile list must have been built for the widest tile wmax
imsrg_status Ctx::tc_gemm_on(const CUtensorMap& map, int64_t slice_rows, const TcProb* probs, const TcTile* tiles,
                             int ntiles, TcOut out, int hL, int hR, int wmax) {
  if (ntiles == 0) return IMSRG_OK;
  if (wmax != 128 && !(wmax == 256 && tc->S == 2)) return fail(IMSRG_ERR_INVALID_ARGUMENT, "unsupported tile width");
  const int grid = std::min(ntiles, tc->num_sms);
  const int unarmed = tc_unarmed_next ? 0 : -1;  // one-shot test switch
  tc_unarmed_next = 0;
  auto go = [&](auto launcher) {
    launcher(grid, stream, map, slice_rows, probs, tiles, ntiles, out, hL, hR, tc->d_err, tc_wait_ns, unarmed);
  };
  if (tc->kind == kKindTF32)
    wmax == 256 ? go(launch_tc_gemm<2, kKindTF32, 256>) : go(launch_tc_gemm<2, kKindTF32, 128>);
  else if (tc->S == 2)
    wmax == 256 ? go(launch_tc_gemm<2, kKindBF16, 256>) : go(launch_tc_gemm<2, kKindBF16, 128>);
  else
    go(launch_tc_gemm<3, kKindBF16, 128>);
  return launched("k_tc_gemm");
}

// rows of 128 bytes over total_rows rows, box 128 bytes x 128 rows, 128-byte swizzle.  The map
// moves bytes: it is described as rows of 64 BF16 values for BF16 and TF32 operands alike
// (the swizzle permutes 16-byte chunks by row and does not depend on the element type).
imsrg_status Ctx::tc_encode_map(CUtensorMap* map, void* buf, int64_t total_rows) {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  CK_TC(cuda(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q),
             "cudaGetDriverEntryPointByVersion"));
  if (!fn || q != cudaDriverEntryPointSuccess) return fail(IMSRG_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  const cuuint64_t gdim[2] = {64, (cuuint64_t)std::max<int64_t>(total_rows, BM)};
  const cuuint64_t gstride[1] = {128};
  const cuuint32_t box[2] = {64, (cuuint32_t)BM};
  const cuuint32_t estride[2] = {1, 1};
  CUresult r = reinterpret_cast<EncodeTiledFn>(fn)(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, buf, gdim, gstride, box,
                                                    estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(IMSRG_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return IMSRG_OK;
}

// operand split of any op / chunk list into a buffer of this context's slice count
imsrg_status Ctx::tc_split_on(const TcSplitOp* ops, const SplitChunk* chunks, int nchunks, const double* Lp,
                              const double* Rp, void* buf, int64_t slice_elems) {
  if (nchunks == 0) return IMSRG_OK;
  if (tc->kind == kKindTF32)
    k_split_chunks<2, float><<<nchunks, 256, 0, stream>>>(ops, chunks, Lp, Rp, buf, slice_elems);
  else if (tc->S == 2)
    k_split_chunks<2, __nv_bfloat16><<<nchunks, 256, 0, stream>>>(ops, chunks, Lp, Rp, buf, slice_elems);
  else
    k_split_chunks<3, __nv_bfloat16><<<nchunks, 256, 0, stream>>>(ops, chunks, Lp, Rp, buf, slice_elems);
  return launched("k_split_chunks");
}

imsrg_status Ctx::tc_pphh(const double* Lp, int hL, const double* Rp, int hR, double* w1, double* w2) {
  if (!tc->chunks.empty()) {
    const int grid = (int)tc->chunks.size();
    CK_TC(tc_split_on(tc->d_split_ops, tc->d_chunks, grid, Lp, Rp, tc->buf, tc->slice_elems));
  }
  mark(kPhasePphhSplit);
  TcOut out{};
  out.f64[kOpW1] = w1;
  out.f64[kOpW2] = w2;
  CK_TC(tc_gemm(tc->d_pphh_probs, tc->d_pphh_tiles, (int)tc->pphh_tiles.size(), out, hL, hR, tc->wmax[0]));
  mark(kPhasePphhGemm);
  if (!tc->small_tiles.empty()) {
    GemmOperands ops{};
    ops.in[kOpL] = Lp; ops.in[kOpR] = Rp;
    ops.out[kOpW1] = w1; ops.out[kOpW2] = w2;
    ops.hL = hL; ops.hR = hR;
    k_gemm_f32<<<(int)tc->small_tiles.size(), 256, 0, stream>>>(tc->d_small_probs, tc->d_small_tiles, ops);
    CK_TC(launched("k_gemm_f32"));
  }
  mark(kPhasePphhSmall);
  return IMSRG_OK;
}

imsrg_status Ctx::tc_error() {
  if (!tc) return IMSRG_OK;
  int e = 0;
  CK_TC(cuda(cudaMemcpyAsync(&e, tc->d_err, sizeof(int), cudaMemcpyDeviceToHost, stream), "D2H tc error"));
  CK_TC(cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize"));
  if (e) {
    cudaMemsetAsync(tc->d_err, 0, sizeof(int), stream);
    static const char* role[] = {"", "producer (stage free)", "MMA (accumulator free)", "MMA (stage loaded)",
                                 "epilogue (accumulator ready)"};
    return fail(IMSRG_ERR_TIMEOUT, std::string("tensor-core GEMM: a bounded wait ran out in the ") +
                                       (e >= 1 && e <= 4 ? role[e] : "kernel") + " (code " + std::to_string(e) + ")");
  }
  return IMSRG_OK;
}

imsrg_status Ctx::tc_wcc(const double*, const double*, double*) {
  return fail(IMSRG_ERR_UNSUPPORTED, "the piecewise 222_ph entry point runs in FP64");
}

// The whole [L,R] with the channel contractions on tensor cores and the gathers in FP32
// (same call order as the FP64 path).
imsrg_status Ctx::tc_commutator(const double* Lp, int hL, const double* Rp, int hR, double* RES, int hRES,
                                bool with_e0) {
  const int64_t ncc = L.cc_size;
  mark(kPhaseStart);
  // operands of both tensor-core products: the Pandya tiles (particle-hole) and the split
  // columns of the ladder arrays; then one persistent launch computes the K = npp ladder
  // products W1 and the recoupling input X over the merged tile list
  if (ncc) {
    const PandyaOps ops{{Rp, Lp}, {hR, hL}, tc->d_cc_tile_A, tc->d_cc_tile_B, tc->d_cc_nkb, tc->d_cc_seg};
    launch_pandya_tc(tc->S, tc->kind, (int)tc->pandya_chunks.size(), stream, D, tc->d_pandya_chunks, ops, tc->buf,
                     tc->slice_elems, tc->d_swap_row);
    CK_TC(launched("k_pandya_tc"));
  }
  mark(kPhasePandya);
  // W1 and W2 of the ladder in FP32, in the first half of the FP64 workspaces
  float* w1f = reinterpret_cast<float*>(d_w1);
  float* w2f = reinterpret_cast<float*>(d_w2);
  CK_TC(pphh_clear_f(w1f, w2f));
  if (!tc->chunks.empty()) CK_TC(tc_split_on(tc->d_split_ops, tc->d_chunks, (int)tc->chunks.size(), Lp, Rp, tc->buf,
                                             tc->slice_elems));
  mark(kPhasePphhSplit);
  TcOut gout{};
  gout.w1f = w1f;
  gout.xmask = tc->d_xmask;
  gout.f32 = tc->zbuf;
  if (tc->merged)
    CK_TC(tc_gemm(tc->d_all_probs, tc->d_tile_mem + tc->tile_cap_all, (int)tc->all_tiles.size(), gout, hL, hR,
                  tc->wmax[2]));
  else
    CK_TC(tc_gemm(tc->d_pphh_probs, tc->d_pphh_tiles, (int)tc->pphh_tiles.size(), gout, hL, hR, tc->wmax[0]));
  mark(kPhasePphhGemm);
  if (with_e0) CK_TC(e0(Lp, hL, Rp, hR, RES, nullptr));
  {  // commutator_111 block by block (one-body operators only couple orbits of one (l, j, tz) block)
    const int n = L.A * L.A + L.P * L.A + L.P * L.P;
    k_comm111f<<<(n + 255) / 256, 256, 0, stream>>>(D, Lp, hL, Rp, hR, RES);
    CK_TC(launched("k_comm111f"));
  }
  CK_TC(c121(Lp, hL, Rp, hR, RES, hRES));
  mark(kPhaseOneBody);
  if (L.n_unique) {
    k_comm122_fb2<<<tc->g122_nspb, 64, 0, stream>>>(D, tc->g122_w, tc->g122_nspb, Lp, hL, Rp, hR, tc->g122_fb,
                                                     tc->d_g122_counter);
    CK_TC(launched("k_comm122_fb2"));
    const G122Plan& P = tc->g122;
    // the big tasks, then enough eight-warp CTAs to fill the GPU at the occupancy the shared
    // memory allows (the warps take the runs from the counter)
    const int grid = P.nbig + tc->num_sms * std::max(1, tc->g122_per_sm);
    launch_comm122(grid, P.smem_bytes, stream, D, tc->d_g122_tasks, tc->d_g122_items, (int)P.items.size(), P.nbig,
                   tc->d_g122_counter, tc->d_g122_codes, std::max(P.warp_cap, 4 * P.tiny_cap), P.tiny_cap, Lp, hL,
                   Rp, hR, RES, hRES, tc->g122_fb);
    CK_TC(launched("k_comm122_sub"));
  }
  mark(kPhase122);
  if (!tc->small_tiles.empty()) {  // the K = nhh products (W2) on FP32 SIMT
    GemmOperands ops{};
    ops.in[kOpL] = Lp; ops.in[kOpR] = Rp;
    ops.out[kOpW1] = d_w1; ops.out[kOpW2] = d_w2;  // FP32 stores at the same element offsets
    ops.hL = hL; ops.hR = hR;
    k_gemm_f32_w<<<(int)tc->small_tiles.size(), 256, 0, stream>>>(tc->d_small_probs, tc->d_small_tiles, ops);
    CK_TC(launched("k_gemm_f32_w"));
  }
  mark(kPhasePphhSmall);
  CK_TC(c221_f(hL, hR, RES, hRES, w1f, w2f));
  mark(kPhase221);
  if (!tc->merged) {
    CK_TC(tc_gemm(tc->d_z_probs, tc->d_z_tiles, (int)tc->z_tiles.size(), gout, hL, hR, tc->wmax[1]));
    mark(kPhasePhGemm);
  }
  if (!tc->quads.empty()) {
    const int64_t nq = (int64_t)tc->quads.size();
    const int grid = (int)std::min<int64_t>((nq + 255) / 256, tc->recouple_ctas);
    launch_recouple_q(tc->recouple_minb, grid, stream, D, tc->d_quads, nq, tc->d_xcol, tc->zbuf, RES);
    CK_TC(launched("k_recouple_q"));
  }
  mark(kPhaseRecouple);
  // the ladder's contribution last (additions commute), with the lower triangles of the square
  // arrays written from the updated upper ones in the same pass
  if (!upd_tiles.empty()) {
    k_pphh_update_mirror_f<<<(int)upd_tiles.size(), 256, 0, stream>>>(D, d_upd_tiles, RES, w1f, w2f,
                                                                     (float)(hL * hR), hRES);
    CK_TC(launched("k_pphh_update_mirror_f"));
  }
  mark(kPhasePphhUpdate);
  return IMSRG_OK;
}

// ---------------------------------------------------------------- autotuner
// Splits the 122 tasks into [tiny | warp | cta] runs by size, keeping channel order inside
// each run, and uploads the list.  The caps must keep the per-CTA shared memory of the
// 8-lane and warp kernels within the 48 KiB default.
imsrg_status Ctx::tc_g122_partition(int tiny_cap, int small_cap) {
  G122Plan& P = tc->g122;
  const int bt = P.tiny_cap, bw = P.warp_cap;
  const std::string e = g122_partition(P, tiny_cap, small_cap);
  if (!e.empty()) {
    g122_partition(P, bt, bw);  // keep the previous caps
    return fail(IMSRG_ERR_INVALID_ARGUMENT, e);
  }
  if (!P.tasks.empty()) {
    CK_TC(cuda(cudaMemcpyAsync(tc->d_g122_tasks, P.tasks.data(), sizeof(G122Task) * P.tasks.size(),
                               cudaMemcpyHostToDevice, stream), "cudaMemcpyAsync(122 tasks)"));
    if (!P.items.empty())
      CK_TC(cuda(cudaMemcpyAsync(tc->d_g122_items, P.items.data(), sizeof(int2) * P.items.size(),
                                 cudaMemcpyHostToDevice, stream), "cudaMemcpyAsync(122 runs)"));
    CK_TC(cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize(122 tasks)"));
  }
  CK_TC(cuda(g122_smem_attr(P.smem_bytes), "smem attr (122)"));
  CK_TC(cuda(g122_blocks_per_sm(P.smem_bytes, &tc->g122_per_sm), "occupancy (122)"));
  return IMSRG_OK;
}

// Tile lists of the persistent GEMMs for their tile shapes and an order: per list ([0] ladder,
// [1] X, [2] the merged list) the widest tile wmax (128, or 256 with two slices) and narrow last
// column tiles or not; order 0 = longest K first (LPT), 1 = problem order.  No output element
// depends on these choices.
imsrg_status Ctx::tc_set_tiles(const int* wmax, const bool* narrow, int order) {
  for (int x = 0; x < 3; ++x)
    if (wmax[x] != 128 && !(wmax[x] == 256 && tc->S == 2)) return fail(IMSRG_ERR_INVALID_ARGUMENT, "unsupported tile width");
  auto build = [&](const std::vector<TcProb>& probs, int x) {
    std::vector<TcTile> t = make_tiles(probs, wmax[x], narrow[x], &tc->xmask);
    if (order == 1)
      std::stable_sort(t.begin(), t.end(), [](const TcTile& a, const TcTile& b) {
        return a.prob != b.prob ? a.prob < b.prob : (a.m0 != b.m0 ? a.m0 < b.m0 : a.n0 < b.n0);
      });
    return t;
  };
  tc->pphh_tiles = build(tc->pphh_probs, 0);
  tc->z_tiles = build(tc->z_probs, 1);
  tc->all_tiles = build(tc->all_probs, 2);
  if (tc->pphh_tiles.size() > tc->tile_cap_pphh || tc->z_tiles.size() > tc->tile_cap_z ||
      tc->all_tiles.size() > tc->tile_cap_all)
    return fail(IMSRG_ERR_MISMATCH, "GEMM tile list larger than its allocation");
  TcTile* d_all = tc->d_tile_mem + tc->tile_cap_all;
  auto put = [&](TcTile* dst, const std::vector<TcTile>& v) -> imsrg_status {
    if (v.empty()) return IMSRG_OK;
    return cuda(cudaMemcpyAsync(dst, v.data(), sizeof(TcTile) * v.size(), cudaMemcpyHostToDevice, stream),
                "cudaMemcpyAsync(GEMM tiles)");
  };
  CK_TC(put(tc->d_tile_mem, tc->pphh_tiles));
  CK_TC(put(tc->d_tile_mem + tc->tile_cap_pphh, tc->z_tiles));
  CK_TC(put(d_all, tc->all_tiles));
  CK_TC(cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize(GEMM tiles)"));
  for (int x = 0; x < 3; ++x) {
    tc->wmax[x] = wmax[x];
    tc->narrow[x] = narrow[x];
  }
  tc->gemm_order = order;
  return IMSRG_OK;
}

// Times one mixed commutator [L, R] per candidate launch configuration on this basis and keeps
// the fastest: the 122 task caps, the recoupling kernel, then the tensor-core GEMM's tile shape
// and order jointly.  Every
// candidate computes the same result: no output element depends on the partition, the grid or
// the tile order.  A captured Magnus-step graph is dropped, so the next step re-captures it.
imsrg_status Ctx::tc_autotune(const double* Lp, int hL, const double* Rp, int hR, double* RES, imsrg_tune_info* info) {
  if (!tc) return fail(IMSRG_ERR_UNSUPPORTED, "autotune needs a mixed-precision context");
  const int hRES = -hL * hR;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CK_TC(cuda(cudaEventCreate(&e0), "cudaEventCreate"));
  CK_TC(cuda(cudaEventCreate(&e1), "cudaEventCreate"));
  auto time_one = [&](float* ms) -> imsrg_status {
    CK_TC(commutator(Lp, hL, Rp, hR, RES, hRES, true));  // warm-up
    CK_TC(cuda(cudaEventRecord(e0, stream), "cudaEventRecord"));
    for (int r = 0; r < 3; ++r) CK_TC(commutator(Lp, hL, Rp, hR, RES, hRES, true));
    CK_TC(cuda(cudaEventRecord(e1, stream), "cudaEventRecord"));
    CK_TC(cuda(cudaEventSynchronize(e1), "cudaEventSynchronize"));
    CK_TC(cuda(cudaEventElapsedTime(ms, e0, e1), "cudaEventElapsedTime"));
    *ms /= 3.0f;
    return IMSRG_OK;
  };
  imsrg_status st = IMSRG_OK;
  float base = 0.0f, best = 0.0f;
  do {
    if ((st = time_one(&base)) != IMSRG_OK) break;
    best = base;
    // 122 caps
    static const int caps[][2] = {{32, 256}, {64, 256}, {32, 512}, {64, 512}, {64, 1024}};
    int bt = tc->g122.tiny_cap, bs = tc->g122.warp_cap;
    for (const auto& c : caps) {
      if ((st = tc_g122_partition(c[0], c[1])) != IMSRG_OK) break;
      float ms;
      if ((st = time_one(&ms)) != IMSRG_OK) break;
      if (ms < best) { best = ms; bt = c[0]; bs = c[1]; }
    }
    if (st != IMSRG_OK || (st = tc_g122_partition(bt, bs)) != IMSRG_OK) break;
    // recoupling: the launch-bounds variant and the CTA count (no output depends on them)
    {
      int bm = tc->recouple_minb, bc = tc->recouple_ctas;
      float ms;
      for (int minb : {4, 6, 8}) {
        for (int mult : {16, 32, 64}) {
          tc->recouple_minb = minb;
          tc->recouple_ctas = tc->num_sms * mult;
          if ((st = time_one(&ms)) != IMSRG_OK) break;
          if (ms < best) { best = ms; bm = minb; bc = tc->recouple_ctas; }
        }
        if (st != IMSRG_OK) break;
      }
      if (st != IMSRG_OK) break;
      tc->recouple_minb = bm;
      tc->recouple_ctas = bc;
    }
    // tensor-core GEMM: one merged launch with its tile shape, or two launches with a tile shape
    // each (the ladder's first, then X's), and the tile order
    {
      std::vector<std::pair<int, bool>> shapes = {{128, false}, {128, true}};
      if (tc->S == 2) { shapes.push_back({256, false}); shapes.push_back({256, true}); }
      int bw[3], bo = tc->gemm_order;
      bool bn[3], bmg = tc->merged;
      for (int x = 0; x < 3; ++x) { bw[x] = tc->wmax[x]; bn[x] = tc->narrow[x]; }
      auto trial = [&](bool merged, const int* w, const bool* n, int order) -> imsrg_status {
        tc->merged = merged;
        CK_TC(tc_set_tiles(w, n, order));
        float ms;
        CK_TC(time_one(&ms));
        if (ms < best) {
          best = ms;
          bmg = merged;
          bo = order;
          for (int x = 0; x < 3; ++x) { bw[x] = w[x]; bn[x] = n[x]; }
        }
        return IMSRG_OK;
      };
      for (int order : {0, 1}) {
        for (const auto& sh : shapes) {  // merged
          int w[3] = {bw[0], bw[1], sh.first};
          bool n[3] = {bn[0], bn[1], sh.second};
          if ((st = trial(true, w, n, order)) != IMSRG_OK) break;
        }
        if (st != IMSRG_OK) break;
        for (int list = 0; list < 2 && st == IMSRG_OK; ++list)  // separate: ladder shape, then X shape
          for (const auto& sh : shapes) {
            int w[3] = {bw[0], bw[1], bw[2]};
            bool n[3] = {bn[0], bn[1], bn[2]};
            w[list] = sh.first;
            n[list] = sh.second;
            if ((st = trial(false, w, n, order)) != IMSRG_OK) break;
          }
        if (st != IMSRG_OK) break;
      }
      if (st != IMSRG_OK) break;
      tc->merged = bmg;
      if ((st = tc_set_tiles(bw, bn, bo)) != IMSRG_OK) break;
    }
    float after = 0.0f;
    if ((st = time_one(&after)) != IMSRG_OK) break;
    if (info) {
      info->tiny_cap = tc->g122.tiny_cap;
      info->small_cap = tc->g122.warp_cap;
      info->recouple_kind = 1;
      info->recouple_min_blocks = tc->recouple_minb;
      info->recouple_ctas = tc->recouple_ctas;
      const int gl = tc->merged ? 2 : 0;
      info->gemm_wmax = tc->wmax[gl];
      info->gemm_narrow = tc->narrow[gl] ? 1 : 0;
      info->gemm_wmax_x = tc->wmax[1];
      info->gemm_narrow_x = tc->narrow[1] ? 1 : 0;
      info->gemm_merged = tc->merged ? 1 : 0;
      info->gemm_order = tc->gemm_order;
      info->ms_before = base;
      info->ms_after = after;
    }
  } while (false);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st == IMSRG_OK) graph_release();
  return st;
}

extern "C" imsrg_status imsrg_recouple_traffic(imsrg_ctx* ctx, int64_t* x_reads, int64_t* x_distinct,
                                               int64_t* res_elems, int64_t* aux_bytes) {
  if (!ctx || !x_reads || !x_distinct || !res_elems || !aux_bytes) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (c->device < 0) return c->fail(IMSRG_ERR_UNSUPPORTED, "host-only context (device < 0)");
  if (c->precision == IMSRG_PREC_FP64) return c->fail(IMSRG_ERR_UNSUPPORTED, "the recoupling kernel runs in the mixed modes");
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(IMSRG_ERR_CUDA, "cudaSetDevice");
  CK_TC(c->tc_prepare(c->precision));
  const RecoupleTraffic t = recouple_traffic(c->L, c->tc->quads);
  *x_reads = t.x_reads;
  *x_distinct = t.x_distinct;
  *res_elems = t.res_elems;
  *aux_bytes = t.aux_bytes;
  return IMSRG_OK;
}

extern "C" imsrg_status imsrg_set_tuning(imsrg_ctx* ctx, const imsrg_tune_info* cfg) {
  if (!ctx || !cfg) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (c->device < 0) return c->fail(IMSRG_ERR_UNSUPPORTED, "host-only context (device < 0)");
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(IMSRG_ERR_CUDA, "cudaSetDevice");
  if (c->precision == IMSRG_PREC_FP64) return c->fail(IMSRG_ERR_UNSUPPORTED, "tuning applies to the mixed modes");
  // recouple_kind 1 (one thread per quadruple) is the only recoupling kernel
  if (cfg->recouple_kind != 1 || cfg->gemm_order < 0 || cfg->gemm_order > 1 || cfg->recouple_ctas < 1 ||
      (cfg->recouple_min_blocks != 4 && cfg->recouple_min_blocks != 6 && cfg->recouple_min_blocks != 8))
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_set_tuning: value out of range");
  CK_TC(c->ensure_workspace());
  CK_TC(c->tc_prepare(c->precision));
  CK_TC(c->tc_g122_partition(cfg->tiny_cap, cfg->small_cap));
  {
    const bool m = cfg->gemm_merged != 0;
    const int wx = cfg->gemm_wmax_x ? cfg->gemm_wmax_x : cfg->gemm_wmax;
    int w[3] = {cfg->gemm_wmax, wx, cfg->gemm_wmax};
    bool n[3] = {cfg->gemm_narrow != 0, (cfg->gemm_wmax_x ? cfg->gemm_narrow_x : cfg->gemm_narrow) != 0,
                 cfg->gemm_narrow != 0};
    if (m) { w[0] = c->tc->wmax[0]; n[0] = c->tc->narrow[0]; w[1] = c->tc->wmax[1]; n[1] = c->tc->narrow[1]; }
    CK_TC(c->tc_set_tiles(w, n, cfg->gemm_order));
    c->tc->merged = m;
  }
  c->tc->recouple_minb = cfg->recouple_min_blocks;
  c->tc->recouple_ctas = cfg->recouple_ctas;
  c->graph_release();
  return IMSRG_OK;
}

extern "C" imsrg_status imsrg_autotune(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES,
                                       imsrg_tune_info* info) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (c->device < 0) return c->fail(IMSRG_ERR_UNSUPPORTED, "host-only context (device < 0)");
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(IMSRG_ERR_CUDA, "cudaSetDevice");
  if (!L || !R || !RES || L->owner != c || R->owner != c || RES->owner != c || RES == L || RES == R)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_autotune: operators of this context, RES distinct");
  if (c->precision == IMSRG_PREC_FP64) return c->fail(IMSRG_ERR_UNSUPPORTED, "autotune applies to the mixed modes");
  CK_TC(c->ensure_workspace());
  CK_TC(c->tc_prepare(c->precision));
  return c->tc_autotune(L->d, L->herm, R->d, R->herm, RES->d, info);
}
