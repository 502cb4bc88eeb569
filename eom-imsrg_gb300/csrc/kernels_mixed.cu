// FP32-arithmetic companions of the FP64 kernels for the mixed-precision commutator.
// Operators stay FP64 in HBM; these kernels read FP64, compute in FP32 and accumulate
// the result into FP64 (GB300's FP64 pipe is ~1/64 of its FP32 rate).
#include <cuda_bf16.h>

#include "dev.cuh"
#include "kernels.h"
#include "pair_groups.h"
#include "split.cuh"

namespace imsrg {

__device__ __forceinline__ float d_sixjf(const DevLayout& D, int j1, int j2, int j3, int j4, int j5, int j6) {
  if (!(d_tri(j1, j2, j3) && d_tri(j4, j5, j3) && d_tri(j1, j5, j6) && d_tri(j4, j2, j6))) return 0.0f;
  const int nh = D.sj_nh;
  const int k = (((j1 >> 1) * nh + (j2 >> 1)) * nh + (j4 >> 1)) * nh + (j5 >> 1);
  return __ldg(D.sj_valf + D.sj_off[k] + ((j3 - D.sj_j3min[k]) >> 1) * D.sj_n6[k] + ((j6 - D.sj_j6min[k]) >> 1));
}

// Pandya transform (calculate_cross_coupled, src/cross_coupled.f90:1190-1300) in FP32,
// written straight into the K-major split operand tiles (BF16 or TF32, split.cuh) of the
// cross-coupled GEMM:
// row r of the tile block of channel q, column ph.  Threads run along ph so the writes
// into each 128-byte tile row are contiguous.
// Each element is written twice: at row r of the operand tiles, times the row sign
// phi(r(a,b)) = (-1)^((ja+jb)/2), and unsigned at row s(r) of the row-swapped copy,
// s(r(a,b)) = r(b,a).  The recoupling input X (gemm_tc.cu) is built from both.
template <int S, typename T>
__global__ void k_pandya_tc(DevLayout D, const double* __restrict__ op, int herm, void* __restrict__ bufv,
                            int64_t slice_elems, const int* __restrict__ tile_base, const int* __restrict__ tile_base_s,
                            const int* __restrict__ nkb, const int* __restrict__ swap_row) {
  T* buf = static_cast<T*>(bufv);
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
      VRefF rf;
      for (int JT = Jmin; JT <= Jmax; JT += 2) {
        if (!d_vref_f(D, h, a, p, b, JT, rf)) continue;
        const float v = f64_to_f32(op[rf.idx]) * rf.scale(herm);
        sm += ((JT & 2) ? -1.0f : 1.0f) * (float)(JT + 1) * d_sixjf(D, jp, jh, JC, ja, jb, JT) * v;
      }
      val = sm * (((jh + jb + JC) & 2) ? -1.0f : 1.0f) * sqrtf((float)(JC + 1));
    }
    const int rs = swap_row[D.cc_row_off[q] + r];
    const int64_t dst = split_offset<T>(tile_base[q], nkb[q], r, nbx);
    const int64_t dsts = split_offset<T>(tile_base_s[q], nkb[q], rs, nbx);
    const bool flip = ((ja + jb) & 2) != 0;  // phi(r) = -1
    float rem = val;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const T hv = SplitElem<T>::take(rem);
      buf[s * slice_elems + dst] = flip ? SplitElem<T>::neg(hv) : hv;
      buf[s * slice_elems + dsts] = hv;
    }
  }
}
void launch_pandya_tc(int S, int kind, int grid, cudaStream_t stream, const DevLayout& D, const double* op, int herm,
                      void* buf, int64_t slice_elems, const int* tile_base, const int* tile_base_s, const int* nkb,
                      const int* swap_row) {
  if (kind == 1)
    k_pandya_tc<2, float><<<grid, 256, 0, stream>>>(D, op, herm, buf, slice_elems, tile_base, tile_base_s, nkb,
                                                     swap_row);
  else if (S == 2)
    k_pandya_tc<2, __nv_bfloat16><<<grid, 256, 0, stream>>>(D, op, herm, buf, slice_elems, tile_base, tile_base_s,
                                                             nkb, swap_row);
  else
    k_pandya_tc<3, __nv_bfloat16><<<grid, 256, 0, stream>>>(D, op, herm, buf, slice_elems, tile_base, tile_base_s,
                                                             nkb, swap_row);
}

// commutator_221 (src/commutators.f90:435-578) with FP32 arithmetic: one warp per
// one-body output, ACCUMULATES into RES (FP64)
__global__ void k_comm221f(DevLayout D, int pm, double* __restrict__ RES, int hRES, const double* __restrict__ w1,
                           const double* __restrict__ w2) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= D.n_ob) return;
  const int kind = D.ob_kind[warp], p = D.ob_p[warp], q = D.ob_q[warp], ik = D.ob_pk[warp], jk = D.ob_qk[warp];
  const int ji = D.jj[ik];
  float sm = 0.0f;
  VRefF r;
  for (int ck = lane; ck < D.N; ck += 32) {
    const double* w = D.con[ck] ? w1 : w2;
    const int jc = D.jj[ck];
    for (int JT = abs(jc - ji); JT <= jc + ji; JT += 2) {
      float v = d_vref_f(D, ck, ik, ck, jk, JT, r) ? f64_to_f32(w[r.idx]) * r.pre : 0.0f;
      if (kind < 2 && d_vref_f(D, ck, jk, ck, ik, JT, r)) v -= (float)pm * f64_to_f32(w[r.idx]) * r.pre;
      sm += v * (float)(JT + 1);
    }
  }
  for (int o = 16; o > 0; o >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, o);
  if (lane == 0) {
    double* f = (kind == 0) ? RES + D.off_fhh + p + (int64_t)q * D.A
                            : (kind == 1 ? RES + D.off_fpp + p + (int64_t)q * D.P : RES + D.off_fph + p + (int64_t)q * D.P);
    const double v = *f + (double)(sm / (float)(ji + 1));
    *f = v;
    if (kind < 2) {
      double* g = (kind == 0) ? RES + D.off_fhh + q + (int64_t)p * D.A : RES + D.off_fpp + q + (int64_t)p * D.P;
      *g = v * hRES;
    }
  }
}

// 222_pp_hh accumulation for the mixed path: FP32 arithmetic, upper triangles of the
// square arrays only (a final mirror pass restores the lower triangles).
__global__ void __launch_bounds__(256) k_pphh_update_f(DevLayout D, const int4* __restrict__ tiles,
                                                       double* __restrict__ RES, const double* __restrict__ w1,
                                                       const double* __restrict__ w2, float pm) {
  __shared__ float Xa[32][33];
  __shared__ float Xb[32][33];
  const int4 t = tiles[blockIdx.x];
  const int k = t.x, i0 = t.y, j0 = t.z;
  const int64_t base = D.goff[k];
  const int n1 = D.gn1[k], n2 = D.gn2[k];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  if (!t.w) {
    for (int r = ty; r < 32; r += 8) {
      const int i = i0 + tx, j = j0 + r;
      if (i < n1 && j < n2) {
        const int64_t e = base + i + (int64_t)j * n1;
        RES[e] += f32_to_f64(f64_to_f32(w1[e]) - f64_to_f32(w2[e]));
      }
    }
    return;
  }
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, j = j0 + r;
    Xa[r][tx] = (i < n1 && j < n1) ? f64_to_f32(w1[base + i + (int64_t)j * n1]) - f64_to_f32(w2[base + i + (int64_t)j * n1])
                                   : 0.0f;
    const int ib = j0 + tx, jb = i0 + r;
    Xb[r][tx] = (ib < n1 && jb < n1) ? f64_to_f32(w1[base + ib + (int64_t)jb * n1]) -
                                           f64_to_f32(w2[base + ib + (int64_t)jb * n1])
                                     : 0.0f;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, j = j0 + r;
    if (i < n1 && j < n1 && i <= j) {
      const int64_t e = base + i + (int64_t)j * n1;
      RES[e] += f32_to_f64(Xa[r][tx] - Xb[tx][r] * pm);
    }
  }
}

// lower triangle of every square array (pppp, phph, hhhh) = herm * upper triangle
__global__ void __launch_bounds__(256) k_mirror_square(DevLayout D, const int4* __restrict__ tiles,
                                                       double* __restrict__ RES, int herm) {
  __shared__ double T[32][33];
  const int4 t = tiles[blockIdx.x];
  if (!t.w) return;
  const int k = t.x, i0 = t.y, j0 = t.z;  // i0 <= j0: source tile (upper), destination (j0, i0)
  const int64_t base = D.goff[k];
  const int n1 = D.gn1[k];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const unsigned long long flip = herm < 0 ? (1ull << 63) : 0ull;
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, j = j0 + r;
    T[r][tx] = (i < n1 && j < n1) ? RES[base + i + (int64_t)j * n1] : 0.0;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    // destination element (j0 + tx, i0 + r) = herm * source (i0 + r, j0 + tx) = T[tx][r]
    const int i = j0 + tx, j = i0 + r;
    if (i < n1 && j < n1 && i > j) {
      const double v = T[tx][r];
      RES[base + i + (int64_t)j * n1] = __longlong_as_double(__double_as_longlong(v) ^ (long long)flip);
    }
  }
}

}  // namespace imsrg
