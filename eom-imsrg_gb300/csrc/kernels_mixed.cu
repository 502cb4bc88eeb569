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
// cross-coupled GEMM: element (r, ph) of channel q,
//   X(ab, ph) = (-1)^((jh+jb+JC)/2) sqrt(JC+1) sum_JT (-1)^(JT/2) (JT+1) {jp jh JC; ja jb JT} V(ha, pb; JT).
// Each CTA takes one chunk of a channel's elements (pandya_chunks: no search over channels),
// threads run along ph so the writes into each 128-byte tile row are contiguous.  Both
// operators (L and R) share every index of an element, so one thread forms both sums: what
// does not depend on JT is set up once per element (the 6j row, the pair classes and array,
// the stored order of (h, a) and (p, b) and their sqrt 2 factors), and per JT the loop loads
// the two pair positions (adjacent in JT), the array offset, the 6j value and the element
// of each operator.
// The recoupling input X (gemm_tc.cu) is one product A B^T over a K of four segments of seg
// columns, A = [phiL | phiR | Ls | Rs], B = [phiR | phiL | Rs | Ls]: phiO is O with row r
// times phi(r(a,b)) = (-1)^((ja+jb)/2), Os is O with row r(b,a) at row s(r) = r(a,b).  So
// each element of L goes to A and B signed at row r (segments 0 and 1) and unsigned at row
// s(r) (segments 2 and 3); R's to segments 1, 0 and 3, 2.
template <int S, typename T>
__global__ void __launch_bounds__(256) k_pandya_tc(DevLayout D, const PandyaChunk* __restrict__ chunks,
                                                   PandyaOps ops, void* __restrict__ bufv, int64_t slice_elems,
                                                   const int* __restrict__ swap_row) {
  T* buf = static_cast<T*>(bufv);
  const double* __restrict__ opR = ops.op[0];
  const double* __restrict__ opL = ops.op[1];
  const int hR = ops.herm[0], hL = ops.herm[1];
  const PandyaChunk c = chunks[blockIdx.x];
  const int q = c.q, nph = D.cc_nph[q], JC = D.cc_J[q];
  const int col0 = D.cc_col_off[q], row0 = D.cc_row_off[q];
  const int ta = ops.tile_a[q], tbb = ops.tile_b[q], nk = ops.nkb[q], seg = ops.seg[q];
  const int N = D.N, NJ = D.NJ, nh = D.sj_nh;
  for (int x = threadIdx.x; x < c.n; x += blockDim.x) {
    const int loc = c.e0 + x;
    const int r = (int)__umulhi((unsigned)loc, c.mnph), nbx = loc - r * nph;
    const int p = D.cc_cp[col0 + nbx], h = D.cc_ch[col0 + nbx];
    const int a = D.cc_ra[row0 + r], b = D.cc_rb[row0 + r];
    const int jp = D.jj[p], jh = D.jj[h], ja = D.jj[a], jb = D.jj[b];
    float valL = 0.0f, valR = 0.0f;
    if (((D.ll[a] + D.ll[h]) & 1) == ((D.ll[b] + D.ll[p]) & 1) && D.tz[a] + D.tz[h] == D.tz[b] + D.tz[p]) {
      const int Jmin = max(abs(jp - jb), abs(ja - jh)), Jmax = min(jp + jb, ja + jh);
      // 6j {jp jh JC; ja jb JT} as srow[JT / 2] (zero unless both JC triads hold)
      const int ks = (((jp >> 1) * nh + (jh >> 1)) * nh + (ja >> 1)) * nh + (jb >> 1);
      const bool ok6 = d_tri(jp, jh, JC) && d_tri(ja, jb, JC);
      const float* srow = D.sj_valf + D.sj_off[ks] + ((JC - D.sj_j3min[ks]) >> 1) * D.sj_n6[ks] - (D.sj_j6min[ks] >> 1);
      // V(ha, pb; JT): stored order, classes and array of both pairs
      const bool s1 = h > a, s2 = p > b;
      const int* pp1 = D.pairpos + ((s1 ? a : h) * N + (s1 ? h : a)) * NJ;
      const int* pp2 = D.pairpos + ((s2 ? b : p) * N + (s2 ? p : b)) * NJ;
      const int nsq = (!s1 && h == a) + (!s2 && p == b);
      const float m = nsq == 0 ? 1.0f : (nsq == 1 ? 1.41421356f : 2.0f);
      const int C1 = D.con[h] + D.con[a], C2 = D.con[p] + D.con[b];
      const int lo = min(C1, C2), hi = max(C1, C2);
      const int g = (lo == 0) ? hi : (lo == 1 ? (hi == 1 ? 3 : 5) : 4);
      const bool tr = C1 > C2;
      // the transposed block is herm times the stored one
      const float mL = (tr && hL < 0) ? -m : m, mR = (tr && hR < 0) ? -m : m;
      const int qb = (D.tz[h] + D.tz[a] + 2) + ((D.ll[h] + D.ll[a]) & 1);  // channel of JT: 3 JT + qb
      float smL = 0.0f, smR = 0.0f;
      for (int JT = Jmin; JT <= Jmax; JT += 2) {
        int neg = 0;
        if (s1) neg ^= (1 + ((jh + ja - JT) >> 1)) & 1;
        if (s2) neg ^= (1 + ((jp + jb - JT) >> 1)) & 1;
        const int i1 = __ldg(pp1 + (JT >> 1)), i2 = __ldg(pp2 + (JT >> 1));
        const int k = (3 * JT + qb) * 6 + g;
        const int n1 = __ldg(D.gn1 + k);
        const int64_t idx = __ldg(D.goff + k) + (tr ? i2 + (int64_t)i1 * n1 : i1 + (int64_t)i2 * n1);
        const float vl = f64_to_f32(__ldg(opL + idx)), vr = f64_to_f32(__ldg(opR + idx));
        const float sj = ok6 ? __ldg(srow + (JT >> 1)) : 0.0f;
        const float cf = (((JT & 2) ^ (neg << 1)) ? -1.0f : 1.0f) * (float)(JT + 1) * sj;
        smL += cf * (vl * mL);
        smR += cf * (vr * mR);
      }
      const float f = (((jh + jb + JC) & 2) ? -1.0f : 1.0f) * sqrtf((float)(JC + 1));
      valL = smL * f;
      valR = smR * f;
    }
    const int rs = swap_row[row0 + r];
    // L: A(r, nbx), B(r, seg + nbx), A(s(r), 2 seg + nbx), B(s(r), 3 seg + nbx); R: A(r, seg + nbx),
    // B(r, nbx), A(s(r), 3 seg + nbx), B(s(r), 2 seg + nbx)
    const int64_t a0 = split_offset<T>(ta, nk, r, nbx), a1 = split_offset<T>(ta, nk, r, seg + nbx);
    const int64_t b0 = split_offset<T>(tbb, nk, r, nbx), b1 = split_offset<T>(tbb, nk, r, seg + nbx);
    const int64_t sa2 = split_offset<T>(ta, nk, rs, 2 * seg + nbx), sa3 = split_offset<T>(ta, nk, rs, 3 * seg + nbx);
    const int64_t sb2 = split_offset<T>(tbb, nk, rs, 2 * seg + nbx), sb3 = split_offset<T>(tbb, nk, rs, 3 * seg + nbx);
    const bool flip = ((ja + jb) & 2) != 0;  // phi(r) = -1
    float remL = valL, remR = valR;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const T hl = SplitElem<T>::take(remL), hr = SplitElem<T>::take(remR);
      const T sl = flip ? SplitElem<T>::neg(hl) : hl, sr = flip ? SplitElem<T>::neg(hr) : hr;
      T* o = buf + s * slice_elems;
      o[a0] = sl;
      o[b1] = sl;
      o[sa2] = hl;
      o[sb3] = hl;
      o[a1] = sr;
      o[b0] = sr;
      o[sa3] = hr;
      o[sb2] = hr;
    }
  }
}
void launch_pandya_tc(int S, int kind, int nchunks, cudaStream_t stream, const DevLayout& D, const PandyaChunk* chunks,
                      const PandyaOps& ops, void* buf, int64_t slice_elems, const int* swap_row) {
  if (kind == 1)
    k_pandya_tc<2, float><<<nchunks, 256, 0, stream>>>(D, chunks, ops, buf, slice_elems, swap_row);
  else if (S == 2)
    k_pandya_tc<2, __nv_bfloat16><<<nchunks, 256, 0, stream>>>(D, chunks, ops, buf, slice_elems, swap_row);
  else
    k_pandya_tc<3, __nv_bfloat16><<<nchunks, 256, 0, stream>>>(D, chunks, ops, buf, slice_elems, swap_row);
}

// commutator_221 (src/commutators.f90:435-578) with FP32 arithmetic, ACCUMULATES into RES
// (FP64).  About a thousand one-body outputs at eMax=10, so one 256-thread CTA per output: the
// threads take the (orbit c, JT) terms of its sum, (2JT+1) w(c p, c q; JT) with w = W1 for a
// hole c and W2 for a particle, all independent, and a block reduction adds them up.
__global__ void __launch_bounds__(256) k_comm221f(DevLayout D, int pm, double* __restrict__ RES, int hRES,
                                                  const float* __restrict__ w1, const float* __restrict__ w2) {
  __shared__ float red[8];
  const int o = blockIdx.x;
  if (o >= D.n_ob) return;
  const int kind = D.ob_kind[o], p = D.ob_p[o], q = D.ob_q[o], ik = D.ob_pk[o], jk = D.ob_qk[o];
  const int ji = D.jj[ik];
  float sm = 0.0f;
  VRefF r;
  for (int t = threadIdx.x; t < D.N * D.NJ; t += blockDim.x) {
    const int ck = t % D.N, m = t / D.N;
    const int jc = D.jj[ck];
    const int JT = abs(jc - ji) + 2 * m;
    if (JT > jc + ji) continue;
    const float* w = D.con[ck] ? w1 : w2;
    float v = d_vref_f(D, ck, ik, ck, jk, JT, r) ? __ldg(w + r.idx) * r.pre : 0.0f;
    if (kind < 2 && d_vref_f(D, ck, jk, ck, ik, JT, r)) v -= (float)pm * __ldg(w + r.idx) * r.pre;
    sm += v * (float)(JT + 1);
  }
  for (int s = 16; s > 0; s >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sm;
  __syncthreads();
  if (threadIdx.x == 0) {
    float tot = 0.0f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) tot += red[k];
    double* f = (kind == 0) ? RES + D.off_fhh + p + (int64_t)q * D.A
                            : (kind == 1 ? RES + D.off_fpp + p + (int64_t)q * D.P : RES + D.off_fph + p + (int64_t)q * D.P);
    const double v = *f + (double)(tot / (float)(ji + 1));
    *f = v;
    if (kind < 2) {
      double* g = (kind == 0) ? RES + D.off_fhh + q + (int64_t)p * D.A : RES + D.off_fpp + q + (int64_t)p * D.P;
      *g = v * hRES;
    }
  }
}

// commutator_111 (src/commutators.f90:36-80) of the mixed path, FP64, ASSIGNS the one-body part:
// one thread per element of fhh, fph and fpp.  One-body operators only couple orbits of one
// (l, j, tz) block, so (L R - R L)(a, b) sums over the at most six orbits of that block and is
// zero between blocks.
__global__ void k_comm111f(DevLayout D, const double* __restrict__ L, int hL, const double* __restrict__ R, int hR,
                           double* __restrict__ RES) {
  const int A = D.A, P = D.P;
  const int total = A * A + P * A + P * P;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    int a, b;
    int64_t off;
    if (t < A * A) {
      a = D.holes[t % A]; b = D.holes[t / A]; off = D.off_fhh + t;
    } else if (t < A * A + P * A) {
      const int s = t - A * A;
      a = D.parts[s % P]; b = D.holes[s / P]; off = D.off_fph + s;
    } else {
      const int s = t - A * A - P * A;
      a = D.parts[s % P]; b = D.parts[s / P]; off = D.off_fpp + s;
    }
    double v = 0.0;
    if (D.jj[a] == D.jj[b] && D.ll[a] == D.ll[b] && D.tz[a] == D.tz[b]) {
      const int* blk = D.same_list + D.same_start[a];
      for (int x = 0; x < D.same_count[a]; ++x) {
        const int k = blk[x];
        v += d_f_elem(D, L, hL, a, k) * d_f_elem(D, R, hR, k, b) - d_f_elem(D, R, hR, a, k) * d_f_elem(D, L, hL, k, b);
      }
    }
    RES[off] = v;
  }
}


// lower triangle of every square array (pppp, phph, hhhh) = herm * upper triangle
// The ladder update and the mirror pass in one: RES += W1 - W2 on the rectangular arrays and,
// on the square arrays, RES(i, j) += W(i, j) - pm W(j, i) for i <= j (W = W1 - W2, FP32) with
// the lower triangle then written from the updated upper one, RES(j, i) = herm RES(i, j).  It
// runs after every other contribution to RES's two-body part (122 assigns it, the recoupling
// adds to the upper triangles; additions commute), so RES's upper triangles are read once.
__global__ void __launch_bounds__(256) k_pphh_update_mirror_f(DevLayout D, const int4* __restrict__ tiles,
                                                              double* __restrict__ RES, const float* __restrict__ w1,
                                                              const float* __restrict__ w2, float pm, int herm) {
  __shared__ float Xa[32][33];
  __shared__ float Xb[32][33];
  __shared__ double V[32][33];
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
        RES[e] += f32_to_f64(w1[e] - w2[e]);
      }
    }
    return;
  }
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, j = j0 + r;
    Xa[r][tx] = (i < n1 && j < n1) ? w1[base + i + (int64_t)j * n1] - w2[base + i + (int64_t)j * n1] : 0.0f;
    const int ib = j0 + tx, jb = i0 + r;
    Xb[r][tx] = (ib < n1 && jb < n1) ? w1[base + ib + (int64_t)jb * n1] - w2[base + ib + (int64_t)jb * n1] : 0.0f;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, j = j0 + r;
    if (i < n1 && j < n1 && i <= j) {
      const int64_t e = base + i + (int64_t)j * n1;
      const double v = RES[e] + f32_to_f64(Xa[r][tx] - Xb[tx][r] * pm);
      RES[e] = v;
      V[r][tx] = v;
    }
  }
  __syncthreads();
  const unsigned long long flip = herm < 0 ? (1ull << 63) : 0ull;
  for (int r = ty; r < 32; r += 8) {
    // destination (j0 + tx, i0 + r) = herm * source (i0 + r, j0 + tx) = V[tx][r]
    const int i = j0 + tx, j = i0 + r;
    if (i < n1 && j < n1 && i > j)
      RES[base + i + (int64_t)j * n1] = __longlong_as_double(__double_as_longlong(V[tx][r]) ^ (long long)flip);
  }
}


}  // namespace imsrg
