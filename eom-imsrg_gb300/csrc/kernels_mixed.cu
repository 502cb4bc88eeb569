// FP32-arithmetic companions of the FP64 kernels for the mixed-precision commutator.
// Operators stay FP64 in HBM; these kernels read FP64, compute in FP32 and accumulate
// the result into FP64 (GB300's FP64 pipe is ~1/64 of its FP32 rate).
#include <cuda_bf16.h>

#include "dev.cuh"
#include "kernels.h"

namespace imsrg {

__device__ __forceinline__ float d_sixjf(const DevLayout& D, int j1, int j2, int j3, int j4, int j5, int j6) {
  if (!(d_tri(j1, j2, j3) && d_tri(j4, j5, j3) && d_tri(j1, j5, j6) && d_tri(j4, j2, j6))) return 0.0f;
  const int nh = D.sj_nh;
  const int k = (((j1 >> 1) * nh + (j2 >> 1)) * nh + (j4 >> 1)) * nh + (j5 >> 1);
  return __ldg(D.sj_valf + D.sj_off[k] + ((j3 - D.sj_j3min[k]) >> 1) * D.sj_n6[k] + ((j6 - D.sj_j6min[k]) >> 1));
}

// Pandya transform (calculate_cross_coupled, src/cross_coupled.f90:1190-1300) in FP32,
// written straight into the K-major split-BF16 operand tiles of the cross-coupled GEMM:
// row r of the tile block of channel q, column ph.  Threads run along ph so the writes
// into each 128-byte tile row are contiguous.
template <int S>
__global__ void k_pandya_tc(DevLayout D, const double* __restrict__ op, int herm, __nv_bfloat16* __restrict__ buf,
                            int64_t slice_elems, const int* __restrict__ tile_base, const int* __restrict__ nkb) {
  const int64_t total = D.cc_size;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = D.ncc;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (D.cc_off[mid] <= e) lo = mid; else hi = mid;
    }
    while (D.cc_off[lo + 1] <= e) ++lo;
    const int q = lo;
    const int nph = D.cc_nph[q];
    const int64_t loc = e - D.cc_off[q];
    const int r = (int)(loc / nph);
    const int nbx = (int)(loc - (int64_t)r * nph);
    const int JC = D.cc_J[q];
    const int p = D.cc_cp[D.cc_col_off[q] + nbx], h = D.cc_ch[D.cc_col_off[q] + nbx];
    const int a = D.cc_ra[D.cc_row_off[q] + r], b = D.cc_rb[D.cc_row_off[q] + r];
    const int jp = D.jj[p], jh = D.jj[h], ja = D.jj[a], jb = D.jj[b];
    float val = 0.0f;
    if (((D.ll[a] + D.ll[h]) & 1) == ((D.ll[b] + D.ll[p]) & 1) && D.tz[a] + D.tz[h] == D.tz[b] + D.tz[p]) {
      const int Jmin = max(abs(jp - jb), abs(ja - jh)), Jmax = min(jp + jb, ja + jh);
      float sm = 0.0f;
      VRef rf;
      for (int JT = Jmin; JT <= Jmax; JT += 2) {
        if (!d_vref(D, h, a, p, b, JT, rf)) continue;
        const float v = (float)op[rf.idx] * (float)(rf.herm ? herm * rf.pre : rf.pre);
        sm += ((JT & 2) ? -1.0f : 1.0f) * (float)(JT + 1) * d_sixjf(D, jp, jh, JC, ja, jb, JT) * v;
      }
      val = sm * (((jh + jb + JC) & 2) ? -1.0f : 1.0f) * sqrtf((float)(JC + 1));
    }
    const int64_t dst =
        ((int64_t)(tile_base[q] + (r >> 7) * nkb[q] + (nbx >> 6)) * 128 + (r & 127)) * 64 + (nbx & 63);
    float rem = val;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const __nv_bfloat16 hv = __float2bfloat16_rn(rem);
      buf[s * slice_elems + dst] = hv;
      rem -= __bfloat162float(hv);
    }
  }
}
void launch_pandya_tc(int S, int grid, cudaStream_t stream, const DevLayout& D, const double* op, int herm,
                      __nv_bfloat16* buf, int64_t slice_elems, const int* tile_base, const int* nkb) {
  if (S == 2)
    k_pandya_tc<2><<<grid, 256, 0, stream>>>(D, op, herm, buf, slice_elems, tile_base, nkb);
  else
    k_pandya_tc<3><<<grid, 256, 0, stream>>>(D, op, herm, buf, slice_elems, tile_base, nkb);
}

// commutator_122 (src/commutators.f90:283-396), FP32 arithmetic -- ASSIGNS every 2b element
__global__ void k_comm122f(DevLayout D, const double* __restrict__ L, int hL, const double* __restrict__ R, int hR,
                           double* __restrict__ RES, int hRES) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < D.n_unique; u += (int64_t)gridDim.x * blockDim.x) {
    int q, g, IX, JX;
    d_unique_decode(D, u, q, g, IX, JX);
    const int c1 = (g < 3) ? 0 : (g == 4 ? 2 : 1);
    const int c2 = (g == 0) ? 0 : ((g == 1 || g == 3) ? 1 : 2);
    const int o1 = D.pair_off[q * 3 + c1] + IX, o2 = D.pair_off[q * 3 + c2] + JX;
    const int a = D.pair_a[o1], b = D.pair_b[o1], c = D.pair_a[o2], d = D.pair_b[o2];
    const int JT = D.lamJ[q];
    float sm = 0.0f;
    VRef r;
    const int who[4] = {a, b, c, d};
#pragma unroll
    for (int slot = 0; slot < 4; ++slot) {
      const int x = who[slot];
      const int s0 = D.same_start[x], n = D.same_count[x];
      for (int t = 0; t < n; ++t) {
        const int i = D.same_list[s0 + t];
        bool ok;
        if (slot == 0) ok = d_vref(D, i, b, c, d, JT, r);
        else if (slot == 1) ok = d_vref(D, a, i, c, d, JT, r);
        else if (slot == 2) ok = d_vref(D, a, b, i, d, JT, r);
        else ok = d_vref(D, a, b, c, i, JT, r);
        if (!ok) continue;
        const float vR = (float)R[r.idx] * (float)(r.herm ? hR * r.pre : r.pre);
        const float vL = (float)L[r.idx] * (float)(r.herm ? hL * r.pre : r.pre);
        if (slot < 2) {
          sm += (float)d_f_elem(D, L, hL, x, i) * vR - (float)d_f_elem(D, R, hR, x, i) * vL;
        } else {
          sm += -(float)d_f_elem(D, L, hL, i, x) * vR + (float)d_f_elem(D, R, hR, i, x) * vL;
        }
      }
    }
    double v = (double)sm;
    if (a == b) v *= 0.7071067811865476;
    if (c == d) v *= 0.7071067811865476;
    const int k = q * 6 + g;
    double* X = RES + D.goff[k];
    const int n1 = D.gn1[k];
    X[IX + (int64_t)JX * n1] = v;
    if (g == 0 || g == 3 || g == 4) X[JX + (int64_t)IX * n1] = v * hRES;
  }
}

// commutator_222_ph recoupling (src/commutators.f90:804-921) reading the antisymmetrised
// cross-coupled product Z(q) = hL LCC RCC^T - hR RCC LCC^T (FP32), which folds the
// reference's four WCC reads per J' into two.  ACCUMULATES into RES.
__global__ void k_comm222ph_z(DevLayout D, const float* __restrict__ Z, double* __restrict__ RES, int hRES) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < D.n_unique; u += (int64_t)gridDim.x * blockDim.x) {
    int q, g, IX, JX;
    d_unique_decode(D, u, q, g, IX, JX);
    const int c1 = (g < 3) ? 0 : (g == 4 ? 2 : 1);
    const int c2 = (g == 0) ? 0 : ((g == 1 || g == 3) ? 1 : 2);
    const int o1 = D.pair_off[q * 3 + c1] + IX, o2 = D.pair_off[q * 3 + c2] + JX;
    const int i = D.pair_a[o1], j = D.pair_b[o1], k = D.pair_a[o2], l = D.pair_b[o2];
    const int ji = D.jj[i], jj = D.jj[j], jk = D.jj[k], jl = D.jj[l];
    const int Jtot = D.lamJ[q];
    const int N = D.N, NJ = D.NJ;
    const float phase = ((ji + jj + jk + jl) & 2) ? -1.0f : 1.0f;
    float sm = 0.0f;
    {
      const int Tz = abs(D.tz[i] - D.tz[k]) >> 1;
      const int PAR = (D.ll[i] + D.ll[k]) & 1;
      const int jmin = max(abs(jj - jl), abs(ji - jk)), jmax = min(jj + jl, ji + jk);
      float acc = 0.0f;
      for (int JP = jmin; JP <= jmax; JP += 2) {
        const int qx = (JP >> 1) + Tz * (D.JM + 1) + PAR * 2 * (D.JM + 1);
        const float* W = Z + D.wcc_off[qx];
        const int64_t rl = D.cc_rlen[qx];
        const int h = JP >> 1;
        const int64_t rjl = D.ccr[(j * N + l) * NJ + h], rik = D.ccr[(i * N + k) * NJ + h];
        const int64_t gjl = D.ccr[(l * N + j) * NJ + h], gik = D.ccr[(k * N + i) * NJ + h];
        if ((rjl | rik | gjl | gik) < 0) continue;
        acc += (W[gik + rjl * rl] + phase * W[gjl + rik * rl]) * d_sixjf(D, ji, jj, Jtot, jl, jk, JP);
      }
      sm -= (((jl + jk + Jtot) & 2) ? -1.0f : 1.0f) * acc;
    }
    {
      const int Tz = abs(D.tz[i] - D.tz[l]) >> 1;
      const int PAR = (D.ll[i] + D.ll[l]) & 1;
      const int jmin = max(abs(ji - jl), abs(jj - jk)), jmax = min(ji + jl, jj + jk);
      for (int JP = jmin; JP <= jmax; JP += 2) {
        const int qx = (JP >> 1) + Tz * (D.JM + 1) + PAR * 2 * (D.JM + 1);
        const float* W = Z + D.wcc_off[qx];
        const int64_t rl = D.cc_rlen[qx];
        const int h = JP >> 1;
        const int64_t ril = D.ccr[(i * N + l) * NJ + h], rjk = D.ccr[(j * N + k) * NJ + h];
        const int64_t gil = D.ccr[(l * N + i) * NJ + h], gjk = D.ccr[(k * N + j) * NJ + h];
        if ((ril | rjk | gil | gjk) < 0) continue;
        sm += (W[gil + rjk * rl] + phase * W[gjk + ril * rl]) * d_sixjf(D, ji, jj, Jtot, jk, jl, JP);
      }
    }
    double v = (double)sm;
    if (i == j) v *= .70710678118;
    if (k == l) v *= .70710678118;
    const int kk = q * 6 + g;
    double* X = RES + D.goff[kk];
    const int n1 = D.gn1[kk];
    const double nv = X[IX + (int64_t)JX * n1] + v;
    X[IX + (int64_t)JX * n1] = nv;
    if (g == 0 || g == 3 || g == 4) X[JX + (int64_t)IX * n1] = nv * hRES;
  }
}

}  // namespace imsrg
