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
#include "pair_groups.h"
#include "tc.h"

namespace imsrg {

namespace {

constexpr int BM = 128, BN = 128, BK = 64;
constexpr int TILE_BYTES = BM * BK * 2;  // 16 KiB, identical for A and B tiles
constexpr int NUM_THREADS = 320;  // TMA warp, MMA warp, 8 epilogue warps
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s

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
// Bounded wait on a barrier phase.  Returns false (after recording `code`) on timeout or
// when another role has already aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, int* err,
                                          int code) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  while (true) {
    if (mbar_test(bar, parity)) return true;
    if (*abort_flag) return false;
    if (globaltimer() - t0 > kWaitLimitNs) {
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

// instruction descriptor, kind::f16: BF16 A/B, FP32 D, both K-major, M=128, N=128
__host__ __device__ constexpr uint32_t umma_idesc(bool negate_a) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((negate_a ? 1u : 0u) << 13) | ((uint32_t)(BN >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
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

template <int S>
constexpr int stages_for() { return S == 2 ? 3 : 2; }

template <int S>
constexpr size_t smem_bytes() {
  return (size_t)stages_for<S>() * 2 * S * TILE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
}

}  // namespace

template <int S>
__global__ void __launch_bounds__(NUM_THREADS, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tmap, int64_t slice_rows, const TcProb* __restrict__ probs,
              const TcTile* __restrict__ tiles, int ntiles, TcOut out, int hL, int hR, int* err) {
  constexpr int ST = stages_for<S>();
  constexpr int NP = SliceProducts<S>::n;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* ring = smem;  // stage s: A slices [S] then B slices [S], 16 KiB each
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)ST * 2 * S * TILE_BYTES);
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
  if (warp == 1) {  // 2 accumulators x 128 FP32 columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * BN)
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
        for (int term = 0; term < P.nterm && ok; ++term) {
          const int abase = P.t[term].a_tile + (tile.m0 / BM) * P.nkb;
          const int bbase = P.t[term].b_tile + (tile.n0 / BN) * P.nkb;
          for (int kb = 0; kb < P.nkb; ++kb, ++it) {
            const int s = it % ST;
            if (!mbar_wait(&empty[s], ((it / ST) & 1) ^ 1, abort_flag, err, 1)) { ok = false; break; }
            mbar_expect_tx(&full[s], (uint32_t)(2 * S * TILE_BYTES));
            uint8_t* stage = ring + (size_t)s * 2 * S * TILE_BYTES;
            for (int sl = 0; sl < S; ++sl) {
              tma_load_2d(smem_u32(stage + (size_t)sl * TILE_BYTES), &tmap, 0,
                          (int)(sl * slice_rows + (int64_t)(abase + kb) * BM), &full[s]);
              tma_load_2d(smem_u32(stage + (size_t)(S + sl) * TILE_BYTES), &tmap, 0,
                          (int)(sl * slice_rows + (int64_t)(bbase + kb) * BN), &full[s]);
            }
          }
        }
      }
      if (!ok) {
        // drain: wait (bounded) for every issued stage the MMA warp did not consume
        const unsigned long long t0 = globaltimer();
        for (int j = *consumed; j < it; ++j) {
          while (!mbar_test(&full[j % ST], (j / ST) & 1)) {
            if (globaltimer() - t0 > kWaitLimitNs) break;
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
        if (!mbar_wait(&tempty[acc], ((local >> 1) & 1) ^ 1, abort_flag, err, 2)) { ok = false; break; }
        tc_fence_after();
        const uint32_t d_tmem = tmem_base + (uint32_t)(acc * BN);
        bool first = true;
        for (int term = 0; term < P.nterm && ok; ++term) {
          const uint32_t idesc = umma_idesc(term_negated(P.t[term].sign, hL, hR));
          for (int kb = 0; kb < P.nkb; ++kb, ++it) {
            const int s = it % ST;
            if (!mbar_wait(&full[s], (it / ST) & 1, abort_flag, err, 3)) { ok = false; break; }
            tc_fence_after();
            const uint32_t stage = smem_u32(ring + (size_t)s * 2 * S * TILE_BYTES);
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              const uint32_t a0 = stage + (uint32_t)(SliceProducts<S>::a(p) * TILE_BYTES);
              const uint32_t b0 = stage + (uint32_t)((S + SliceProducts<S>::b(p)) * TILE_BYTES);
#pragma unroll
              for (int ks = 0; ks < BK / 16; ++ks) {
                umma(d_tmem, umma_desc(a0 + ks * 32), umma_desc(b0 + ks * 32), idesc, first ? 0u : 1u);
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
    const int half = (warp - 2) >> 2;   // accumulator columns 64*half .. 64*half+63
    int local = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++local) {
      const TcTile tile = tiles[t];
      const TcProb& P = probs[tile.prob];
      const int acc = local & 1;
      if (!mbar_wait(&tfull[acc], (local >> 1) & 1, abort_flag, err, 4)) break;
      tc_fence_after();
      const int m = tile.m0 + quad * 32 + lane;
      for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 32) {
        uint32_t r[32];
        tmem_ld32(tmem_base + (uint32_t)(acc * BN + c0) + ((uint32_t)(quad * 32) << 16), r);
        if (m < P.M) {
          if (P.out_f32) {
            float* C = (P.out_f32 == 1 ? out.f32 : out.f32b) + P.c_off;
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
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(2 * BN) : "memory");
}

// ---------------------------------------------------------------- operand split
// FP64 columns of the stored arrays -> S bf16 slices, K-major 128x64 tiles.
template <int S>
__global__ void k_split_cols(const TcSplitOp* __restrict__ ops, const int64_t* __restrict__ prefix, int nops,
                             const double* __restrict__ L, const double* __restrict__ R, __nv_bfloat16* __restrict__ buf,
                             int64_t slice_elems) {
  const int64_t total = prefix[nops];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nops;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (prefix[mid] <= e) lo = mid; else hi = mid;
    }
    while (prefix[lo + 1] <= e) ++lo;
    const TcSplitOp& o = ops[lo];
    const int64_t loc = e - prefix[lo];
    const int r = (int)(loc / o.K), k = (int)(loc - (int64_t)r * o.K);
    const float x = f64_to_f32((o.src == 0 ? L : R)[o.src_off + k + (int64_t)r * o.K]);
    const int64_t dst = ((int64_t)(o.tile_base + (r / BM) * o.nkb + k / BK) * BM + (r % BM)) * BK + (k % BK);
    float rem = x;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const __nv_bfloat16 h = __float2bfloat16_rn(rem);
      buf[s * slice_elems + dst] = h;
      rem -= __bfloat162float(h);
    }
  }
}

// Chunked split: one block per run of rows of one operand, each thread converts 8
// consecutive k of one row and writes 16-byte bf16 vectors into every slice.
template <int S>
__global__ void __launch_bounds__(256) k_split_chunks(const TcSplitOp* __restrict__ ops,
                                                      const SplitChunk* __restrict__ chunks,
                                                      const double* __restrict__ L, const double* __restrict__ R,
                                                      __nv_bfloat16* __restrict__ buf, int64_t slice_elems) {
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
    const int64_t dst = ((int64_t)(o.tile_base + (r / BM) * o.nkb + k0 / BK) * BM + (r % BM)) * BK + (k0 % BK);
#pragma unroll
    for (int sl = 0; sl < S; ++sl) {
      __align__(16) __nv_bfloat16 h[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        h[u] = __float2bfloat16_rn(x[u]);
        x[u] -= __bfloat162float(h[u]);
      }
      *reinterpret_cast<uint4*>(buf + sl * slice_elems + dst) = *reinterpret_cast<const uint4*>(h);
    }
  }
}

// ---------------------------------------------------------------- small-K FP32 GEMM
// The K = nhh problems of 222_pp_hh (every W2 product): FP32 SIMT, FP64 in and out.
__global__ void __launch_bounds__(256) k_gemm_f32(const GemmProb* __restrict__ probs, const GemmTile* __restrict__ tiles,
                                                  GemmOperands ops) {
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
  double* C = ops.out[P.c_id] + P.c_off;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gm = tile.m0 + tx + 16 * i, gn = tile.n0 + ty + 16 * j;
      if (gm < P.M && gn < P.N) C[gm + (int64_t)gn * P.ldc] = (double)acc[i][j];
    }
}

}  // namespace imsrg

// ====================================================================== host side
using namespace imsrg;

namespace imsrg {

struct TcState {
  int S = 0;
  __nv_bfloat16* buf = nullptr;
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
  // particle-hole: Z(q) = hL LCC RCC^T - hR RCC LCC^T
  std::vector<int> cc_tile_L, cc_tile_R, cc_tile_Ls, cc_tile_Rs, cc_nkb, swap_row;
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
  const int* d_cc_tile_L = nullptr;
  const int* d_cc_tile_R = nullptr;
  const int* d_cc_nkb = nullptr;
  const int* d_cc_tile_Ls = nullptr;
  const int* d_cc_tile_Rs = nullptr;
  const int* d_swap_row = nullptr;
  float* zbuf = nullptr;
  float* ybuf = nullptr;
  int* d_err = nullptr;
  // orbit quadruples (i<=j, k<=l) of the particle-hole recoupling, j fastest
  std::vector<uint64_t> quads;
  const uint64_t* d_quads = nullptr;
  std::vector<SplitChunk> chunks;
  const SplitChunk* d_chunks = nullptr;
  // commutator_122 by pair groups: sub-blocks of at most g122_small elements go one per warp,
  // the larger ones one per CTA (tasks in channel order, so a channel's L and R stay in L2)
  // (tiny sub-blocks, up to g122_tiny elements, go to 8-lane groups, four per warp)
  // All tasks in channel order with their sizes; the device list holds them partitioned into
  // [tiny | warp | cta] runs by the current caps (tc_g122_partition).
  std::vector<int4> g122_all;
  std::vector<int64_t> g122_elems;
  int4* d_g122_tasks = nullptr;
  int g122_ntiny = 0, g122_nwarp = 0, g122_ncta = 0;
  PairGroupsDev g122_t{}, g122_w{}, g122_c{};
  int g122_tiny_cap = 64, g122_small = 256, g122_nmax2 = 1, g122_nmax4 = 1, g122_nspb = 0, g122_nblk2 = 0;
  // tuned launch parameters (imsrg_autotune): CTAs of the recoupling kernel, GEMM tile order
  int recouple_ctas = 152 * 16;
  int recouple_minb = 4;  // launch-bounds variant of k_recouple_y
  int gemm_order = 0;  // 0: longest K first, 1: problem order
  std::vector<TcTile> pphh_tiles_lpt, z_tiles_lpt;
  std::vector<int> g_start, g_n, g_orb, g_b1, g_b2, g_blk_off;
  float* g122_fb = nullptr;  // f(x, y) of L and R on every (l, j, tz) block
  int num_sms = 148;
};

}  // namespace imsrg

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int ceil_div(int a, int b) { return (a + b - 1) / b; }

std::vector<TcTile> make_tiles(const std::vector<TcProb>& probs) {
  std::vector<TcTile> t;
  for (int p = 0; p < (int)probs.size(); ++p)
    for (int m0 = 0; m0 < probs[p].M; m0 += BM)
      for (int n0 = 0; n0 < probs[p].N; n0 += BN) t.push_back(TcTile{p, m0, n0, 0});
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
  if (tc->ybuf) cudaFree(tc->ybuf);
  if (tc->d_err) cudaFree(tc->d_err);
  if (tc->g122_fb) cudaFree(tc->g122_fb);
  if (tc->d_g122_tasks) cudaFree(tc->d_g122_tasks);
  delete tc;
  tc = nullptr;
}

imsrg_status Ctx::tc_prepare(int mode) {
  const int S = (mode == IMSRG_PREC_BF16X6) ? 3 : 2;
  if (tc && tc->S == S) return IMSRG_OK;
  tc_release();
  int cc_major = 0;
  cudaDeviceGetAttribute(&cc_major, cudaDevAttrComputeCapabilityMajor, device);
  if (cc_major < 10) return fail(IMSRG_ERR_UNSUPPORTED, "tensor-core path needs a Blackwell (sm_10x) GPU");
  tc = new TcState();
  tc->S = S;
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
  tc->pphh_tiles = make_tiles(tc->pphh_probs);
  // K = nhh products (all W2 arrays), from the FP64 problem list
  for (const GemmProb& p : pphh_probs)
    if (p.c_id == kOpW2) tc->small_probs.push_back(p);
  tc->small_tiles = build_tiles(tc->small_probs, 64, 64);

  // ---- particle-hole: LCC / RCC rows r, K = nph, each also with its rows swapped
  //      (row r(a,b) holding row r(b,a)); Z(q) = hL LCC RCC^T - hR RCC LCC^T and its
  //      row-swapped copy Y(q) = hL LCCs RCC^T - hR RCCs LCC^T
  tc->cc_tile_L.assign(l.ncc, 0);
  tc->cc_tile_R.assign(l.ncc, 0);
  tc->cc_tile_Ls.assign(l.ncc, 0);
  tc->cc_tile_Rs.assign(l.ncc, 0);
  tc->cc_nkb.assign(l.ncc, 0);
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
    const int nkb = ceil_div(nb, BK);
    const int blk = ceil_div(r, BM) * nkb;
    tc->cc_nkb[q] = nkb;
    tc->cc_tile_L[q] = tiles; tiles += blk;
    tc->cc_tile_R[q] = tiles; tiles += blk;
    tc->cc_tile_Ls[q] = tiles; tiles += blk;
    tc->cc_tile_Rs[q] = tiles; tiles += blk;
    for (int which = 0; which < 2; ++which) {
      TcProb p{};
      p.M = r; p.N = r; p.nkb = nkb; p.nterm = 2;
      const int aL = which ? tc->cc_tile_Ls[q] : tc->cc_tile_L[q];
      const int aR = which ? tc->cc_tile_Rs[q] : tc->cc_tile_R[q];
      p.t[0] = TcTermDesc{aL, tc->cc_tile_R[q], hl};
      p.t[1] = TcTermDesc{aR, tc->cc_tile_L[q], ng | hr};
      p.out_f32 = 1 + which;  // 1 -> Z, 2 -> Y
      p.c_id = 0; p.c_off = l.wcc_off[q]; p.ldc = r;
      tc->z_probs.push_back(p);
    }
  }
  tc->z_tiles = make_tiles(tc->z_probs);
  tc->total_tiles = tiles;
  if (l.JM + 1 > 26) return fail(IMSRG_ERR_UNSUPPORTED, "mixed recoupling supports 2j <= 25 (eMax <= 12)");
  // ---- commutator_122 tasks: the group pairs G1 <= G2 of each channel
  {
    PairGroups pg;
    build_pair_groups(pg, l);
    tc->g_start = pg.spb_start; tc->g_n = pg.spb_n; tc->g_orb = pg.spb_orb;
    tc->g_b1 = pg.grp_b1; tc->g_b2 = pg.grp_b2; tc->g_blk_off = pg.blk_off;
    tc->g122_nspb = pg.nspb;
    tc->g122_nblk2 = pg.nblk2;
    tc->g122_nmax2 = pg.nmax * pg.nmax;
    tc->g122_nmax4 = tc->g122_nmax2 * tc->g122_nmax2;
    for (int q = 0; q < l.nblocks; ++q)
      for (int G2 = pg.grp_first[q]; G2 < pg.grp_first[q + 1]; ++G2)
        for (int G1 = pg.grp_first[q]; G1 <= G2; ++G1) {
          const int4 t = make_int4(q, G1, G2, 0);
          tc->g122_all.push_back(t);
          tc->g122_elems.push_back(pg.elems(G1, G2));
        }
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
  }
  tc->slice_rows = (int64_t)tiles * BM;
  tc->slice_elems = tc->slice_rows * BK;
  if ((int64_t)S * tc->slice_rows >= (int64_t)1 << 31) return fail(IMSRG_ERR_UNSUPPORTED, "operand buffer too large for 32-bit TMA rows");

  const size_t bytes = sizeof(__nv_bfloat16) * (size_t)S * tc->slice_elems;
  CK_TC(cuda(cudaMalloc(&tc->buf, std::max<size_t>(bytes, 256)), "cudaMalloc(tc operands)"));
  CK_TC(cuda(cudaMemset(tc->buf, 0, std::max<size_t>(bytes, 256)), "memset(tc operands)"));
  CK_TC(cuda(cudaMalloc(&tc->zbuf, sizeof(float) * std::max<int64_t>(l.wcc_size, 1)), "cudaMalloc(Z)"));
  CK_TC(cuda(cudaMemset(tc->zbuf, 0, sizeof(float) * std::max<int64_t>(l.wcc_size, 1)), "memset(Z)"));
  CK_TC(cuda(cudaMalloc(&tc->ybuf, sizeof(float) * std::max<int64_t>(l.wcc_size, 1)), "cudaMalloc(Y)"));
  CK_TC(cuda(cudaMemset(tc->ybuf, 0, sizeof(float) * std::max<int64_t>(l.wcc_size, 1)), "memset(Y)"));
  CK_TC(cuda(cudaMalloc(&tc->d_err, sizeof(int)), "cudaMalloc(err)"));
  CK_TC(cuda(cudaMalloc(&tc->g122_fb, sizeof(float) * 2 * std::max(tc->g122_nblk2, 1)), "cudaMalloc(122 blocks)"));
  CK_TC(cuda(cudaMemset(tc->d_err, 0, sizeof(int)), "memset(err)"));
  DevPacker pk;
  pk.add(tc->split_ops, &tc->d_split_ops);
  pk.add(tc->split_prefix, &tc->d_split_prefix);
  pk.add(tc->pphh_probs, &tc->d_pphh_probs);
  pk.add(tc->pphh_tiles, &tc->d_pphh_tiles);
  pk.add(tc->small_probs, &tc->d_small_probs);
  pk.add(tc->small_tiles, &tc->d_small_tiles);
  pk.add(tc->z_probs, &tc->d_z_probs);
  pk.add(tc->z_tiles, &tc->d_z_tiles);
  pk.add(tc->cc_tile_L, &tc->d_cc_tile_L);
  pk.add(tc->cc_tile_R, &tc->d_cc_tile_R);
  pk.add(tc->cc_nkb, &tc->d_cc_nkb);
  pk.add(tc->cc_tile_Ls, &tc->d_cc_tile_Ls);
  pk.add(tc->cc_tile_Rs, &tc->d_cc_tile_Rs);
  pk.add(tc->swap_row, &tc->d_swap_row);
  pk.add(tc->quads, &tc->d_quads);
  pk.add(tc->chunks, &tc->d_chunks);
  pk.add(tc->g_start, &tc->g122_w.spb_start);
  pk.add(tc->g_n, &tc->g122_w.spb_n);
  pk.add(tc->g_orb, &tc->g122_w.spb_orb);
  pk.add(tc->g_b1, &tc->g122_w.grp_b1);
  pk.add(tc->g_b2, &tc->g122_w.grp_b2);
  pk.add(tc->g_blk_off, &tc->g122_w.blk_off);

  CK_TC(cuda(cudaMalloc(&tc->d_mem, pk.buf.size()), "cudaMalloc(tc tables)"));
  CK_TC(cuda(cudaMemcpy(tc->d_mem, pk.buf.data(), pk.buf.size(), cudaMemcpyHostToDevice), "cudaMemcpy(tc tables)"));
  for (auto& f : pk.fix) *f.second = static_cast<const char*>(tc->d_mem) + f.first;
  CK_TC(cuda(cudaMalloc(&tc->d_g122_tasks, sizeof(int4) * std::max<size_t>(tc->g122_all.size(), 1)),
             "cudaMalloc(122 tasks)"));
  tc->g122_t = tc->g122_c = tc->g122_w;
  CK_TC(tc_g122_partition(tc->g122_tiny_cap, tc->g122_small));
  tc->recouple_ctas = tc->num_sms * 16;
  tc->pphh_tiles_lpt = tc->pphh_tiles;
  tc->z_tiles_lpt = tc->z_tiles;

  // tensor map over the whole operand buffer: rows of 64 bf16 (128 bytes), box 64 x 128
  CK_TC(tc_encode_map(&tc->tmap, tc->buf, (int64_t)S * tc->slice_rows));
  const size_t sm = S == 2 ? smem_bytes<2>() : smem_bytes<3>();
  if (S == 2)
    CK_TC(cuda(cudaFuncSetAttribute(k_tc_gemm<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm), "smem attr"));
  else
    CK_TC(cuda(cudaFuncSetAttribute(k_tc_gemm<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm), "smem attr"));
  return IMSRG_OK;
}

imsrg_status Ctx::tc_gemm(const TcProb* probs, const TcTile* tiles, int ntiles, TcOut out, int hL, int hR) {
  return tc_gemm_on(tc->tmap, tc->slice_rows, probs, tiles, ntiles, out, hL, hR);
}

int Ctx::tc_slices() const { return tc ? tc->S : 0; }

// the persistent split-BF16 GEMM over any operand buffer of this context's slice count
imsrg_status Ctx::tc_gemm_on(const CUtensorMap& map, int64_t slice_rows, const TcProb* probs, const TcTile* tiles,
                             int ntiles, TcOut out, int hL, int hR) {
  if (ntiles == 0) return IMSRG_OK;
  const int grid = std::min(ntiles, tc->num_sms);
  if (tc->S == 2)
    k_tc_gemm<2><<<grid, NUM_THREADS, smem_bytes<2>(), stream>>>(map, slice_rows, probs, tiles, ntiles, out, hL, hR,
                                                                  tc->d_err);
  else
    k_tc_gemm<3><<<grid, NUM_THREADS, smem_bytes<3>(), stream>>>(map, slice_rows, probs, tiles, ntiles, out, hL, hR,
                                                                  tc->d_err);
  return launched("k_tc_gemm");
}

// rows of 64 bf16 (128 bytes) over total_rows rows, box 64 x 128, 128-byte swizzle
imsrg_status Ctx::tc_encode_map(CUtensorMap* map, void* buf, int64_t total_rows) {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  CK_TC(cuda(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q),
             "cudaGetDriverEntryPointByVersion"));
  if (!fn || q != cudaDriverEntryPointSuccess) return fail(IMSRG_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  const cuuint64_t gdim[2] = {(cuuint64_t)BK, (cuuint64_t)std::max<int64_t>(total_rows, BM)};
  const cuuint64_t gstride[1] = {(cuuint64_t)(BK * sizeof(__nv_bfloat16))};
  const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)BM};
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
                              const double* Rp, __nv_bfloat16* buf, int64_t slice_elems) {
  if (nchunks == 0) return IMSRG_OK;
  if (tc->S == 2)
    k_split_chunks<2><<<nchunks, 256, 0, stream>>>(ops, chunks, Lp, Rp, buf, slice_elems);
  else
    k_split_chunks<3><<<nchunks, 256, 0, stream>>>(ops, chunks, Lp, Rp, buf, slice_elems);
  return launched("k_split_chunks");
}

imsrg_status Ctx::tc_pphh(const double* Lp, int hL, const double* Rp, int hR, double* w1, double* w2) {
  if (!tc->chunks.empty()) {
    const int grid = (int)tc->chunks.size();
    if (tc->S == 2)
      k_split_chunks<2><<<grid, 256, 0, stream>>>(tc->d_split_ops, tc->d_chunks, Lp, Rp, tc->buf, tc->slice_elems);
    else
      k_split_chunks<3><<<grid, 256, 0, stream>>>(tc->d_split_ops, tc->d_chunks, Lp, Rp, tc->buf, tc->slice_elems);
    CK_TC(launched("k_split_chunks"));
  }
  mark(kPhasePphhSplit);
  TcOut out{};
  out.f64[kOpW1] = w1;
  out.f64[kOpW2] = w2;
  CK_TC(tc_gemm(tc->d_pphh_probs, tc->d_pphh_tiles, (int)tc->pphh_tiles.size(), out, hL, hR));
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
    return fail(IMSRG_ERR_CUDA, "tensor-core GEMM wait timed out (code " + std::to_string(e) + ")");
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
  if (ncc) {
    const int grid = (int)std::min<int64_t>((ncc + 255) / 256, 152 * 16);
    launch_pandya_tc(tc->S, grid, stream, D, Rp, hR, tc->buf, tc->slice_elems, tc->d_cc_tile_R, tc->d_cc_tile_Rs,
                     tc->d_cc_nkb, tc->d_swap_row);
    launch_pandya_tc(tc->S, grid, stream, D, Lp, hL, tc->buf, tc->slice_elems, tc->d_cc_tile_L, tc->d_cc_tile_Ls,
                     tc->d_cc_nkb, tc->d_swap_row);
    CK_TC(launched("k_pandya_tc"));
  }
  mark(kPhasePandya);
  if (with_e0) CK_TC(e0(Lp, hL, Rp, hR, RES, nullptr));
  CK_TC(c111(Lp, hL, Rp, hR, RES));
  CK_TC(c121(Lp, hL, Rp, hR, RES, hRES));
  mark(kPhaseOneBody);
  if (L.n_unique) {
    k_comm122_fblocks<<<tc->g122_nspb, 64, 0, stream>>>(D, tc->g122_w, tc->g122_nspb, tc->g122_nblk2, Lp, hL, Rp, hR,
                                                         tc->g122_fb);
    CK_TC(launched("k_comm122_fblocks"));
    if (tc->g122_ntiny) {  // 8 lanes per task, 32 tasks per CTA
      const int nt = tc->g122_ntiny;
      const int grid = std::min((nt + 31) / 32, tc->num_sms * 8);
      const size_t smem = sizeof(float) * 32 * (size_t)(2 * tc->g122_tiny_cap + 4 * tc->g122_nmax2);
      launch_comm122_lanes(8, grid, smem, stream, D, tc->g122_t, nt, tc->g122_tiny_cap, tc->g122_nmax2, Lp, hL, Rp, hR,
                           RES, hRES, tc->g122_fb, tc->g122_nblk2);
      CK_TC(launched("k_comm122_groups_lanes<8>"));
    }
    if (tc->g122_nwarp) {  // a warp per task, 8 tasks per CTA
      const int nt = tc->g122_nwarp;
      const int grid = std::min((nt + 7) / 8, tc->num_sms * 8);
      const size_t smem = sizeof(float) * 8 * (size_t)(2 * tc->g122_small + 4 * tc->g122_nmax2);
      launch_comm122_lanes(32, grid, smem, stream, D, tc->g122_w, nt, tc->g122_small, tc->g122_nmax2, Lp, hL, Rp, hR,
                           RES, hRES, tc->g122_fb, tc->g122_nblk2);
      CK_TC(launched("k_comm122_groups_lanes<32>"));
    }
    if (tc->g122_ncta) {
      const size_t smem = sizeof(float) * (size_t)(2 * tc->g122_nmax4 + 4 * tc->g122_nmax2);
      k_comm122_groups_cta<<<tc->g122_ncta, 256, smem, stream>>>(D, tc->g122_c, tc->g122_nmax4,
                                                                             tc->g122_nmax2, Lp, hL, Rp, hR, RES, hRES,
                                                                             tc->g122_fb, tc->g122_nblk2);
      CK_TC(launched("k_comm122_groups_cta"));
    }
  }
  mark(kPhase122);
  CK_TC(pphh(Lp, hL, Rp, hR, RES, d_w1, d_w2, true));
  CK_TC(c221(hL, hR, RES, hRES, d_w1, d_w2, true));
  mark(kPhase221);
  TcOut zo{};
  zo.f32 = tc->zbuf;
  zo.f32b = tc->ybuf;
  CK_TC(tc_gemm(tc->d_z_probs, tc->d_z_tiles, (int)tc->z_tiles.size(), zo, hL, hR));
  mark(kPhasePhGemm);
  if (!tc->quads.empty()) {
    const int64_t nq = (int64_t)tc->quads.size();
    const int grid = (int)std::min<int64_t>((nq + 255) / 256, tc->recouple_ctas);
    launch_recouple_y(tc->recouple_minb, grid, stream, D, tc->d_quads, nq, tc->zbuf, tc->ybuf, RES, hL * hR);
    CK_TC(launched("k_recouple_y"));
  }
  if (!upd_tiles.empty()) {
    k_mirror_square<<<(int)upd_tiles.size(), 256, 0, stream>>>(D, d_upd_tiles, RES, hRES);
    CK_TC(launched("k_mirror_square"));
  }
  mark(kPhaseRecouple);
  return IMSRG_OK;
}

// ---------------------------------------------------------------- autotuner
// Splits the 122 tasks into [tiny | warp | cta] runs by size, keeping channel order inside
// each run, and uploads the list.  The caps must keep the per-CTA shared memory of the
// 8-lane and warp kernels within the 48 KiB default.
imsrg_status Ctx::tc_g122_partition(int tiny_cap, int small_cap) {
  const size_t lim = 48 * 1024;
  if (tiny_cap < 1 || small_cap < tiny_cap ||
      sizeof(float) * 32 * (size_t)(2 * tiny_cap + 4 * tc->g122_nmax2) > lim ||
      sizeof(float) * 8 * (size_t)(2 * small_cap + 4 * tc->g122_nmax2) > lim)
    return fail(IMSRG_ERR_INVALID_ARGUMENT, "122 task caps out of range");
  const size_t n = tc->g122_all.size();
  std::vector<int4> v;
  v.reserve(n);
  int nt = 0, nw = 0;
  for (size_t i = 0; i < n; ++i)
    if (tc->g122_elems[i] <= tiny_cap) { v.push_back(tc->g122_all[i]); ++nt; }
  for (size_t i = 0; i < n; ++i)
    if (tc->g122_elems[i] > tiny_cap && tc->g122_elems[i] <= small_cap) { v.push_back(tc->g122_all[i]); ++nw; }
  for (size_t i = 0; i < n; ++i)
    if (tc->g122_elems[i] > small_cap) v.push_back(tc->g122_all[i]);
  if (n) {
    CK_TC(cuda(cudaMemcpyAsync(tc->d_g122_tasks, v.data(), sizeof(int4) * n, cudaMemcpyHostToDevice, stream),
               "cudaMemcpyAsync(122 tasks)"));
    CK_TC(cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize(122 tasks)"));
  }
  tc->g122_ntiny = nt;
  tc->g122_nwarp = nw;
  tc->g122_ncta = (int)n - nt - nw;
  tc->g122_t.tasks = tc->d_g122_tasks;
  tc->g122_w.tasks = tc->d_g122_tasks + nt;
  tc->g122_c.tasks = tc->d_g122_tasks + nt + nw;
  tc->g122_tiny_cap = tiny_cap;
  tc->g122_small = small_cap;
  return IMSRG_OK;
}

// Order of the persistent GEMM tile lists: 0 = longest K first, 1 = problem order.
imsrg_status Ctx::tc_set_gemm_order(int order) {
  auto sorted = [&](const std::vector<TcTile>& lpt) {
    std::vector<TcTile> t = lpt;
    if (order == 1)
      std::stable_sort(t.begin(), t.end(), [](const TcTile& a, const TcTile& b) {
        return a.prob != b.prob ? a.prob < b.prob : (a.m0 != b.m0 ? a.m0 < b.m0 : a.n0 < b.n0);
      });
    return t;
  };
  tc->pphh_tiles = sorted(tc->pphh_tiles_lpt);
  tc->z_tiles = sorted(tc->z_tiles_lpt);
  if (!tc->pphh_tiles.empty())
    CK_TC(cuda(cudaMemcpyAsync(const_cast<TcTile*>(tc->d_pphh_tiles), tc->pphh_tiles.data(),
                               sizeof(TcTile) * tc->pphh_tiles.size(), cudaMemcpyHostToDevice, stream),
               "cudaMemcpyAsync(GEMM tiles)"));
  if (!tc->z_tiles.empty())
    CK_TC(cuda(cudaMemcpyAsync(const_cast<TcTile*>(tc->d_z_tiles), tc->z_tiles.data(),
                               sizeof(TcTile) * tc->z_tiles.size(), cudaMemcpyHostToDevice, stream),
               "cudaMemcpyAsync(GEMM tiles)"));
  CK_TC(cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize(GEMM tiles)"));
  tc->gemm_order = order;
  return IMSRG_OK;
}

// Times one mixed commutator [L, R] per candidate launch configuration on this basis and keeps
// the fastest, one knob at a time (122 task caps, recoupling CTAs, GEMM tile order).  Every
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
    static const int caps[][2] = {{16, 256}, {32, 128}, {32, 256}, {64, 256}, {64, 512}};
    int bt = tc->g122_tiny_cap, bs = tc->g122_small;
    for (const auto& c : caps) {
      if ((st = tc_g122_partition(c[0], c[1])) != IMSRG_OK) break;
      float ms;
      if ((st = time_one(&ms)) != IMSRG_OK) break;
      if (ms < best) { best = ms; bt = c[0]; bs = c[1]; }
    }
    if (st != IMSRG_OK || (st = tc_g122_partition(bt, bs)) != IMSRG_OK) break;
    // recoupling: launch-bounds variant and CTA count together (the best CTA count depends on
    // how many CTAs of the variant are resident)
    int bm = tc->recouple_minb, br = tc->recouple_ctas;
    for (int minb : {4, 5, 6, 8}) {
      for (int mult : {4, 8, 16, 32, 64, 128}) {
        tc->recouple_minb = minb;
        tc->recouple_ctas = tc->num_sms * mult;
        float ms;
        if ((st = time_one(&ms)) != IMSRG_OK) break;
        if (ms < best) { best = ms; bm = minb; br = tc->recouple_ctas; }
      }
      if (st != IMSRG_OK) break;
    }
    tc->recouple_minb = bm;
    tc->recouple_ctas = br;
    if (st != IMSRG_OK) break;
    // GEMM tile order
    int bo = tc->gemm_order;
    for (int order : {0, 1}) {
      if ((st = tc_set_gemm_order(order)) != IMSRG_OK) break;
      float ms;
      if ((st = time_one(&ms)) != IMSRG_OK) break;
      if (ms < best) { best = ms; bo = order; }
    }
    if (st != IMSRG_OK || (st = tc_set_gemm_order(bo)) != IMSRG_OK) break;
    float after = 0.0f;
    if ((st = time_one(&after)) != IMSRG_OK) break;
    if (info) {
      info->tiny_cap = tc->g122_tiny_cap;
      info->small_cap = tc->g122_small;
      info->recouple_ctas = tc->recouple_ctas;
      info->recouple_min_blocks = tc->recouple_minb;
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
