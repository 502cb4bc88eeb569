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
    VRefF r;
    const int who[4] = {a, b, c, d};
#pragma unroll
    for (int slot = 0; slot < 4; ++slot) {
      const int x = who[slot];
      const int s0 = D.same_start[x], n = D.same_count[x];
      for (int t = 0; t < n; ++t) {
        const int i = D.same_list[s0 + t];
        bool ok;
        if (slot == 0) ok = d_vref_f(D, i, b, c, d, JT, r);
        else if (slot == 1) ok = d_vref_f(D, a, i, c, d, JT, r);
        else if (slot == 2) ok = d_vref_f(D, a, b, i, d, JT, r);
        else ok = d_vref_f(D, a, b, c, i, JT, r);
        if (!ok) continue;
        const float vR = f64_to_f32(R[r.idx]) * r.scale(hR);
        const float vL = f64_to_f32(L[r.idx]) * r.scale(hL);
        if (slot < 2) {
          sm += d_f_elem_f(D, L, hL, x, i) * vR - d_f_elem_f(D, R, hR, x, i) * vL;
        } else {
          sm += -d_f_elem_f(D, L, hL, i, x) * vR + d_f_elem_f(D, R, hR, i, x) * vL;
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

// ---------------------------------------------------------------- commutator_122 by pair groups
// commutator_122 (src/commutators.f90:283-396) of one group-pair sub-block (G1 <= G2) of
// channel q, FP32.  In the ordered-pair form X_A(ab,cd) (what v_elem returns) the one-body
// factors act on one index at a time:
//   OUT[a,b,c,d] = sum_a' fL(a,a') R_A[a',b,c,d] - fR(a,a') L_A[a',b,c,d]   (and b)
//                - sum_c' fL(c',c) R_A[a,b,c',d] - fR(c',c) L_A[a,b,c',d]   (and d)
// with a' etc. running over the orbits of the same (l, j, tz) block.  Each element of L and
// R is gathered once per sub-block (the neighbour-list form gathers every neighbour of
// every output), the result is written to the stored pairs with the exchange phase and
// 1/sqrt(2) for identical orbits, and for G1 != G2 also mirrored with hRES.  ASSIGNS.
namespace {
// floor(e / n) for 0 <= e, e (n - 1) < 2^32, with m = ceil(2^32 / n)
__device__ __forceinline__ int g122_div(int e, unsigned long long m) {
  return (int)(((unsigned long long)e * m) >> 32);
}
__device__ __forceinline__ unsigned long long g122_magic(int n) {
  return ((1ull << 32) + (unsigned long long)n - 1) / (unsigned long long)n;
}

// Shared-memory slice of one task: XL / XR, the ordered four-index sub-blocks of L and R
// (element x0 + n0 (x1 + n1 (x2 + n2 x3))); PB / PK, the stored position of every bra pair
// (x0, x1) and ket pair (x2, x3): (index in its class list << 2 | class), with FBp / FKp the
// factor pre of V_A = pre x stored (sqrt 2 for identical orbits, the exchange phase when the
// stored order is swapped).
struct G122Smem {
  float *XL, *XR;
  int *PB, *PK;
  float *FBp, *FKp;
};

// kLanes lanes of a warp per task (mask: those lanes), or the whole CTA (kLanes == 0).
// FB: f(x, y) of L (first nblk2 entries) and of R for the orbits x, y of every block,
// FB[blk_off[B] + x*n + y].
template <int kLanes>
__device__ __forceinline__ void g122_task(const DevLayout& D, const PairGroupsDev& G, int4 t,
                                          const double* __restrict__ L, int hL, const double* __restrict__ R, int hR,
                                          double* __restrict__ RES, int hRES, const float* __restrict__ FB, int nblk2,
                                          const G122Smem& S, int tid, int nth, unsigned mask) {
  const int q = t.x, G1 = t.y, G2 = t.z;
  const int b0 = G.grp_b1[G1], b1 = G.grp_b2[G1], b2 = G.grp_b1[G2], b3 = G.grp_b2[G2];
  const int n0 = G.spb_n[b0], n1 = G.spb_n[b1], n2 = G.spb_n[b2], n3 = G.spb_n[b3];
  const int* o0 = G.spb_orb + G.spb_start[b0];
  const int* o1 = G.spb_orb + G.spb_start[b1];
  const int* o2 = G.spb_orb + G.spb_start[b2];
  const int* o3 = G.spb_orb + G.spb_start[b3];
  const int J = D.lamJ[q];
  const int nb = n0 * n1, nk = n2 * n3, ntot = nb * nk;
  const unsigned long long m0 = g122_magic(n0), m2 = g122_magic(n2), mb = g122_magic(nb);
  const int NJ = D.NJ, N = D.N, Jh = J >> 1;
  for (int x = tid; x < nb + nk; x += nth) {  // stored positions of the bra and ket pairs
    const bool bra = x < nb;
    const int y = bra ? x : x - nb;
    const int na = bra ? n0 : n2;
    const int xa = y % na, xb = y / na;
    const int oa = bra ? o0[xa] : o2[xa], ob = bra ? o1[xb] : o3[xb];
    const int lo = min(oa, ob), hi = max(oa, ob);
    float pre = 1.0f;
    if (oa == ob) pre = 1.41421356f;
    else if (oa > ob && ((1 + ((D.jj[oa] + D.jj[ob] - J) >> 1)) & 1)) pre = -1.0f;
    const int code = (D.pairpos[(lo * N + hi) * NJ + Jh] << 2) | (D.con[lo] + D.con[hi]);
    if (bra) { S.PB[y] = code; S.FBp[y] = pre; } else { S.PK[y] = code; S.FKp[y] = pre; }
  }
  if (kLanes) __syncwarp(mask); else __syncthreads();
  const int64_t* go = D.goff + q * 6;
  const int* gn = D.gn1 + q * 6;
  for (int e = tid; e < ntot; e += nth) {  // gather V_A of L and R
    const int ek = g122_div(e, mb), eb = e - ek * nb;
    const int cb = S.PB[eb], ck = S.PK[ek];
    const int C1 = cb & 3, C2 = ck & 3;
    const int lo = min(C1, C2), hi = max(C1, C2);
    const int g = (lo == 0) ? hi : (lo == 1 ? (hi == 1 ? 3 : 5) : 4);
    const int64_t idx = C1 <= C2 ? go[g] + (cb >> 2) + (int64_t)(ck >> 2) * gn[g]
                                 : go[g] + (ck >> 2) + (int64_t)(cb >> 2) * gn[g];
    const float pre = S.FBp[eb] * S.FKp[ek];
    const float sl = (C1 > C2 && hL < 0) ? -pre : pre, sr = (C1 > C2 && hR < 0) ? -pre : pre;
    S.XL[e] = f64_to_f32(L[idx]) * sl;
    S.XR[e] = f64_to_f32(R[idx]) * sr;
  }
  if (kLanes) __syncwarp(mask); else __syncthreads();
  const int s1 = n0, s2 = nb, s3 = nb * n2;
  const float* XL = S.XL;
  const float* XR = S.XR;
  const float* FL0 = FB + G.blk_off[b0];
  const float* FL1 = FB + G.blk_off[b1];
  const float* FL2 = FB + G.blk_off[b2];
  const float* FL3 = FB + G.blk_off[b3];
  for (int e = tid; e < ntot; e += nth) {
    const int ek = g122_div(e, mb), eb = e - ek * nb;
    const int x1 = g122_div(eb, m0), x0 = eb - x1 * n0;
    const int x3 = g122_div(ek, m2), x2 = ek - x3 * n2;
    if ((b0 == b1 && x0 > x1) || (b2 == b3 && x2 > x3)) continue;  // the other order is stored
    float out = 0.0f;
    {  // sum_a' f(a, a') X[a', ...]
      const float* fL = FL0 + x0 * n0;
      const int base = e - x0;
      for (int a = 0; a < n0; ++a) out += __ldg(fL + a) * XR[base + a] - __ldg(fL + nblk2 + a) * XL[base + a];
    }
    {
      const float* fL = FL1 + x1 * n1;
      const int base = e - x1 * s1;
      for (int a = 0; a < n1; ++a)
        out += __ldg(fL + a) * XR[base + a * s1] - __ldg(fL + nblk2 + a) * XL[base + a * s1];
    }
    {  // - sum_c' f(c', c) X[..., c', ...]
      const float* fL = FL2 + x2;
      const int base = e - x2 * s2;
      for (int a = 0; a < n2; ++a)
        out -= __ldg(fL + a * n2) * XR[base + a * s2] - __ldg(fL + nblk2 + a * n2) * XL[base + a * s2];
    }
    {
      const float* fL = FL3 + x3;
      const int base = e - x3 * s3;
      for (int a = 0; a < n3; ++a)
        out -= __ldg(fL + a * n3) * XR[base + a * s3] - __ldg(fL + nblk2 + a * n3) * XL[base + a * s3];
    }
    const int cb = S.PB[eb], ck = S.PK[ek];
    const int C1 = cb & 3, C2 = ck & 3;
    const float w = out / (S.FBp[eb] * S.FKp[ek]);  // stored = V_A / pre
    const int lo = min(C1, C2), hi = max(C1, C2);
    const int g = (lo == 0) ? hi : (lo == 1 ? (hi == 1 ? 3 : 5) : 4);
    if (C1 <= C2) RES[go[g] + (cb >> 2) + (int64_t)(ck >> 2) * gn[g]] = f32_to_f64(w);
    if (G1 != G2 && C2 <= C1) RES[go[g] + (ck >> 2) + (int64_t)(cb >> 2) * gn[g]] = f32_to_f64(hRES < 0 ? -w : w);
  }
  if (kLanes) __syncwarp(mask); else __syncthreads();
}

__device__ __forceinline__ void g122_slice(float* base, int cap, int nmax2, G122Smem& S) {
  S.XL = base;
  S.XR = base + cap;
  S.PB = reinterpret_cast<int*>(base + 2 * cap);
  S.PK = S.PB + nmax2;
  S.FBp = reinterpret_cast<float*>(S.PK + nmax2);
  S.FKp = S.FBp + nmax2;
}
}  // namespace

// FB: f(x, y) of L (first nblk2 entries) and of R for the orbits x, y of every block
__global__ void k_comm122_fblocks(DevLayout D, PairGroupsDev G, int nspb, int nblk2, const double* __restrict__ L,
                                  int hL, const double* __restrict__ R, int hR, float* __restrict__ FB) {
  const int B = blockIdx.x;
  if (B >= nspb) return;
  const int n = G.spb_n[B];
  const int* o = G.spb_orb + G.spb_start[B];
  for (int r = threadIdx.x; r < n * n; r += blockDim.x) {
    const int x = r / n, y = r - (r / n) * n;
    FB[G.blk_off[B] + r] = d_f_elem_f(D, L, hL, o[x], o[y]);
    FB[nblk2 + G.blk_off[B] + r] = d_f_elem_f(D, R, hR, o[x], o[y]);
  }
}

// kLanes-lane groups inside the warps of a 256-thread CTA, each group with its own
// shared-memory slice [XL cap | XR cap | PB, PK, FBp, FKp nmax2 each]; tasks of at most cap
// elements (the host split guarantees it)
template <int kLanes>
__global__ void __launch_bounds__(256) k_comm122_groups_lanes(DevLayout D, PairGroupsDev G, int ntasks, int cap,
                                                              int nmax2, const double* __restrict__ L, int hL,
                                                              const double* __restrict__ R, int hR,
                                                              double* __restrict__ RES, int hRES,
                                                              const float* __restrict__ FB, int nblk2) {
  extern __shared__ float g122_sm[];
  constexpr int kGroups = 256 / kLanes;
  const int grp = threadIdx.x / kLanes, lane = threadIdx.x % kLanes;
  const unsigned mask =
      (kLanes == 32) ? 0xffffffffu : (((1u << kLanes) - 1u) << (((threadIdx.x & 31) / kLanes) * kLanes));
  G122Smem S;
  g122_slice(g122_sm + (size_t)grp * (2 * cap + 4 * nmax2), cap, nmax2, S);
  for (int t = blockIdx.x * kGroups + grp; t < ntasks; t += gridDim.x * kGroups)
    g122_task<kLanes>(D, G, G.tasks[t], L, hL, R, hR, RES, hRES, FB, nblk2, S, lane, kLanes, mask);
}
void launch_comm122_lanes(int lanes, int grid, size_t smem, cudaStream_t st, const DevLayout& D,
                          const PairGroupsDev& G, int ntasks, int cap, int nmax2, const double* L, int hL,
                          const double* R, int hR, double* RES, int hRES, const float* FB, int nblk2) {
  if (lanes == 8)
    k_comm122_groups_lanes<8><<<grid, 256, smem, st>>>(D, G, ntasks, cap, nmax2, L, hL, R, hR, RES, hRES, FB, nblk2);
  else
    k_comm122_groups_lanes<32><<<grid, 256, smem, st>>>(D, G, ntasks, cap, nmax2, L, hL, R, hR, RES, hRES, FB, nblk2);
}

// one CTA per task (the larger sub-blocks): [XL nmax4 | XR nmax4 | PB, PK, FBp, FKp]
__global__ void __launch_bounds__(256) k_comm122_groups_cta(DevLayout D, PairGroupsDev G, int nmax4, int nmax2,
                                                            const double* __restrict__ L, int hL,
                                                            const double* __restrict__ R, int hR,
                                                            double* __restrict__ RES, int hRES,
                                                            const float* __restrict__ FB, int nblk2) {
  extern __shared__ float g122_sm[];
  G122Smem S;
  g122_slice(g122_sm, nmax4, nmax2, S);
  g122_task<0>(D, G, G.tasks[blockIdx.x], L, hL, R, hR, RES, hRES, FB, nblk2, S, threadIdx.x, blockDim.x, 0u);
}

}  // namespace imsrg
