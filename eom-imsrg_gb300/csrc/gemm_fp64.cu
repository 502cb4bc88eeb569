// Grouped FP64 GEMM over a static problem/tile list (the plain-FP64 path).
//
// One CTA per 64x64 output tile, 256 threads each accumulating a 4x4 sub-tile with
// DFMA; K is staged through shared memory in chunks of 16 with loads coalesced along
// whichever dimension is contiguous for the operand's transpose flag.  On GB300 the
// FP64 pipe, not HBM, bounds this kernel, so the tile only has to keep DFMA busy.
#include "gemm.h"
#include "kernels.h"

namespace imsrg {

namespace {
constexpr int BM = 64, BN = 64, BK = 16;

__device__ __forceinline__ double alpha_of(int code, int hL, int hR) {
  const int sel = code & 3;
  double a = (sel == kAlphaHL) ? (double)hL : (sel == kAlphaHR ? (double)hR : 1.0);
  return (code & kAlphaNeg) ? -a : a;
}
}  // namespace

__global__ void __launch_bounds__(256) k_gemm_fp64(const GemmProb* __restrict__ probs,
                                                   const GemmTile* __restrict__ tiles, GemmOperands ops) {
  __shared__ double As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  const GemmTile tile = tiles[blockIdx.x];
  const GemmProb& P = probs[tile.prob];
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  for (int t = 0; t < P.nterm; ++t) {
    const GemmTerm& T = P.t[t];
    const double* A = ops.in[T.a_id] + T.a_off;
    const double* B = ops.in[T.b_id] + T.b_off;
    const double alpha = alpha_of(T.alpha, ops.hL, ops.hR);
    for (int k0 = 0; k0 < T.K; k0 += BK) {
      // A tile: op(A)(m, k), m in [m0, m0+64), k in [k0, k0+16)
      if (T.ta == 0) {
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          const int m = tid & 63, k = (tid >> 6) + 4 * s;
          const int gm = tile.m0 + m, gk = k0 + k;
          As[k][m] = (gm < P.M && gk < T.K) ? alpha * A[gm + (int64_t)gk * T.lda] : 0.0;
        }
      } else {
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          const int k = tid & 15, m = (tid >> 4) + 16 * s;
          const int gm = tile.m0 + m, gk = k0 + k;
          As[k][m] = (gm < P.M && gk < T.K) ? alpha * A[gk + (int64_t)gm * T.lda] : 0.0;
        }
      }
      // B tile: op(B)(k, n)
      if (T.tb == 0) {
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          const int k = tid & 15, n = (tid >> 4) + 16 * s;
          const int gn = tile.n0 + n, gk = k0 + k;
          Bs[k][n] = (gn < P.N && gk < T.K) ? B[gk + (int64_t)gn * T.ldb] : 0.0;
        }
      } else {
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          const int n = tid & 63, k = (tid >> 6) + 4 * s;
          const int gn = tile.n0 + n, gk = k0 + k;
          Bs[k][n] = (gn < P.N && gk < T.K) ? B[gn + (int64_t)gk * T.ldb] : 0.0;
        }
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < BK; ++kk) {
        double a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
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
      if (gm < P.M && gn < P.N) {
        double* c = C + gm + (int64_t)gn * P.ldc;
        *c = P.accum ? *c + acc[i][j] : acc[i][j];
      }
    }
}

}  // namespace imsrg
