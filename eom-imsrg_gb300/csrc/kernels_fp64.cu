// FP64 kernels of the IMSRG(2) commutator engine (everything except the channel GEMMs).
// Each kernel restates one routine of the reference and keeps its assign / accumulate
// semantics; the memory-bound ones are gathers over the device tables of dev.cuh.
#include "dev.cuh"
#include "kernels.h"

namespace imsrg {

// ---------------------------------------------------------------- Pandya transform
// calculate_cross_coupled (src/cross_coupled.f90:1190-1300): one thread per CCX element,
// CCX(q) column-major (rlen x nph), threads consecutive in the row index.
__global__ void k_pandya(DevLayout D, const double* __restrict__ op, int herm, double* __restrict__ cc) {
  const int64_t total = D.cc_size;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = D.ncc;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (D.cc_off[mid] <= e) lo = mid; else hi = mid;
    }
    while (D.cc_off[lo + 1] <= e) ++lo;
    const int q = lo;
    const int rlen = D.cc_rlen[q];
    const int64_t loc = e - D.cc_off[q];
    const int nbx = (int)(loc / rlen);
    const int r = (int)(loc - (int64_t)nbx * rlen);
    const int JC = D.cc_J[q];
    const int p = D.cc_cp[D.cc_col_off[q] + nbx], h = D.cc_ch[D.cc_col_off[q] + nbx];
    const int a = D.cc_ra[D.cc_row_off[q] + r], b = D.cc_rb[D.cc_row_off[q] + r];
    const int jp = D.jj[p], jh = D.jj[h], ja = D.jj[a], jb = D.jj[b];
    double val = 0.0;
    if (((D.ll[a] + D.ll[h]) & 1) == ((D.ll[b] + D.ll[p]) & 1) && D.tz[a] + D.tz[h] == D.tz[b] + D.tz[p]) {
      const int Jmin = max(abs(jp - jb), abs(ja - jh)), Jmax = min(jp + jb, ja + jh);
      double sm = 0.0;
      for (int JT = Jmin; JT <= Jmax; JT += 2)
        sm += d_sgn(JT >> 1) * (JT + 1) * d_sixj(D, jp, jh, JC, ja, jb, JT) * d_v_elem(D, op, herm, h, a, p, b, JT);
      val = sm * d_sgn((jh + jb + JC) >> 1) * sqrt(JC + 1.0);
    }
    cc[e] = val;
  }
}

// ---------------------------------------------------------------- commutator_122
// src/commutators.f90:283-396 -- ASSIGNS every 2b element of RES.
__global__ void k_comm122(DevLayout D, const double* __restrict__ L, int hL, const double* __restrict__ R, int hR,
                          double* __restrict__ RES, int hRES) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < D.n_unique; u += (int64_t)gridDim.x * blockDim.x) {
    int q, g, IX, JX;
    d_unique_decode(D, u, q, g, IX, JX);
    const int c1 = (g < 3) ? 0 : (g == 4 ? 2 : 1);
    const int c2 = (g == 0) ? 0 : ((g == 1 || g == 3) ? 1 : 2);
    const int o1 = D.pair_off[q * 3 + c1] + IX, o2 = D.pair_off[q * 3 + c2] + JX;
    const int a = D.pair_a[o1], b = D.pair_b[o1], c = D.pair_a[o2], d = D.pair_b[o2];
    const int JT = D.lamJ[q];
    double sm = 0.0;
    VRef r;
    {
      const int s0 = D.same_start[a], n = D.same_count[a];
      for (int t = 0; t < n; ++t) {
        const int i = D.same_list[s0 + t];
        if (d_vref(D, i, b, c, d, JT, r)) {
          const double vR = R[r.idx] * (r.herm ? hR * r.pre : r.pre), vL = L[r.idx] * (r.herm ? hL * r.pre : r.pre);
          sm += d_f_elem(D, L, hL, a, i) * vR - d_f_elem(D, R, hR, a, i) * vL;
        }
      }
    }
    {
      const int s0 = D.same_start[b], n = D.same_count[b];
      for (int t = 0; t < n; ++t) {
        const int i = D.same_list[s0 + t];
        if (d_vref(D, a, i, c, d, JT, r)) {
          const double vR = R[r.idx] * (r.herm ? hR * r.pre : r.pre), vL = L[r.idx] * (r.herm ? hL * r.pre : r.pre);
          sm += d_f_elem(D, L, hL, b, i) * vR - d_f_elem(D, R, hR, b, i) * vL;
        }
      }
    }
    {
      const int s0 = D.same_start[c], n = D.same_count[c];
      for (int t = 0; t < n; ++t) {
        const int i = D.same_list[s0 + t];
        if (d_vref(D, a, b, i, d, JT, r)) {
          const double vR = R[r.idx] * (r.herm ? hR * r.pre : r.pre), vL = L[r.idx] * (r.herm ? hL * r.pre : r.pre);
          sm += -d_f_elem(D, L, hL, i, c) * vR + d_f_elem(D, R, hR, i, c) * vL;
        }
      }
    }
    {
      const int s0 = D.same_start[d], n = D.same_count[d];
      for (int t = 0; t < n; ++t) {
        const int i = D.same_list[s0 + t];
        if (d_vref(D, a, b, c, i, JT, r)) {
          const double vR = R[r.idx] * (r.herm ? hR * r.pre : r.pre), vL = L[r.idx] * (r.herm ? hL * r.pre : r.pre);
          sm += -d_f_elem(D, L, hL, i, d) * vR + d_f_elem(D, R, hR, i, d) * vL;
        }
      }
    }
    sm = sm / sqrt(1.0 + (a == b ? 1.0 : 0.0)) / sqrt(1.0 + (c == d ? 1.0 : 0.0));
    const int k = q * 6 + g;
    double* X = RES + D.goff[k];
    const int n1 = D.gn1[k];
    X[IX + (int64_t)JX * n1] = sm;
    if (g == 0 || g == 3 || g == 4) X[JX + (int64_t)IX * n1] = sm * hRES;
  }
}

// ---------------------------------------------------------------- 222_pp_hh accumulation
// RES += W1 - W2 - pm (W1 - W2)^T for pppp/phph/hhhh, RES += W1 - W2 for the rest
// (src/commutators.f90:700-764), over every stored 2b element.
__global__ void k_pphh_update(DevLayout D, double* __restrict__ RES, const double* __restrict__ w1,
                              const double* __restrict__ w2, double pm) {
  const int64_t base = D.goff[0];
  const int64_t total = D.slab - base;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = base + t;
    int lo = 0, hi = D.nblocks * 6;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (D.goff[mid] <= e) lo = mid; else hi = mid;
    }
    while (lo + 1 < D.nblocks * 6 && D.goff[lo + 1] <= e) ++lo;
    const int g = lo % 6;
    double v = RES[e] + w1[e] - w2[e];
    if (g == 0 || g == 3 || g == 4) {
      const int n = D.gn1[lo];
      const int64_t loc = e - D.goff[lo];
      const int j = (int)(loc / n), i = (int)(loc - (int64_t)j * n);
      const int64_t et = D.goff[lo] + j + (int64_t)i * n;
      v = RES[e] + w1[e] - w2[e] - (w1[et] - w2[et]) * pm;
    }
    RES[e] = v;
  }
}

// Tiled form of k_pphh_update: a block owns a 32x32 tile of one array (and, for square
// arrays, its mirror tile), so both the direct and the transposed W reads are coalesced
// through shared memory.  Same arithmetic per element as k_pphh_update.
__global__ void __launch_bounds__(256) k_pphh_update_tiled(DevLayout D, const int4* __restrict__ tiles,
                                                           double* __restrict__ RES, const double* __restrict__ w1,
                                                           const double* __restrict__ w2, double pm) {
  __shared__ double Xa[32][33];
  __shared__ double Xb[32][33];
  const int4 t = tiles[blockIdx.x];  // (array k, row0, col0, square flag)
  const int k = t.x, i0 = t.y, j0 = t.z;
  const int64_t base = D.goff[k];
  const int n1 = D.gn1[k], n2 = D.gn2[k];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  if (!t.w) {
    for (int r = ty; r < 32; r += 8) {
      const int i = i0 + tx, j = j0 + r;
      if (i < n1 && j < n2) {
        const int64_t e = base + i + (int64_t)j * n1;
        RES[e] = RES[e] + w1[e] - w2[e];
      }
    }
    return;
  }
  // square: tiles A = (i0, j0) and B = (j0, i0) (the same tile on the diagonal)
  for (int r = ty; r < 32; r += 8) {
    const int i = i0 + tx, j = j0 + r;
    Xa[r][tx] = (i < n1 && j < n1) ? w1[base + i + (int64_t)j * n1] - w2[base + i + (int64_t)j * n1] : 0.0;
    const int ib = j0 + tx, jb = i0 + r;
    Xb[r][tx] = (ib < n1 && jb < n1) ? w1[base + ib + (int64_t)jb * n1] - w2[base + ib + (int64_t)jb * n1] : 0.0;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    {  // element (i0+tx, j0+r): its transpose is (j0+r, i0+tx) = Xb[tx][r]
      const int i = i0 + tx, j = j0 + r;
      if (i < n1 && j < n1) {
        const int64_t e = base + i + (int64_t)j * n1;
        RES[e] = RES[e] + Xa[r][tx] - Xb[tx][r] * pm;
      }
    }
    if (i0 != j0) {  // element (j0+tx, i0+r): transpose (i0+r, j0+tx) = Xa[tx][r]
      const int i = j0 + tx, j = i0 + r;
      if (i < n1 && j < n1) {
        const int64_t e = base + i + (int64_t)j * n1;
        RES[e] = RES[e] + Xb[r][tx] - Xa[tx][r] * pm;
      }
    }
  }
}

// ---------------------------------------------------------------- 222_ph recoupling
// src/commutators.f90:804-921: for each unique 2b element, sum over the cross-coupled J'
// of 6j-weighted WCC gathers (direct and exchange terms); ACCUMULATES into RES.
__global__ void k_comm222ph(DevLayout D, const double* __restrict__ WCC, int hL, int hR, double* __restrict__ RES,
                            int hRES) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < D.n_unique; u += (int64_t)gridDim.x * blockDim.x) {
    int q, g, IX, JX;
    d_unique_decode(D, u, q, g, IX, JX);
    const int c1 = (g < 3) ? 0 : (g == 4 ? 2 : 1);
    const int c2 = (g == 0) ? 0 : ((g == 1 || g == 3) ? 1 : 2);
    const int o1 = D.pair_off[q * 3 + c1] + IX, o2 = D.pair_off[q * 3 + c2] + JX;
    const int i = D.pair_a[o1], j = D.pair_b[o1], k = D.pair_a[o2], l = D.pair_b[o2];
    const double pre = (i == j) ? .70710678118 : 1.0;   // literal of src/commutators.f90:834
    const double pre2 = (k == l) ? .70710678118 : 1.0;
    const int ji = D.jj[i], jj = D.jj[j], jk = D.jj[k], jl = D.jj[l];
    const int Jtot = D.lamJ[q];
    const int N = D.N, NJ = D.NJ;
    const double phase = d_sgn((ji + jj + jk + jl) >> 1);
    double sm = 0.0;
    {
      const int Tz = abs(D.tz[i] - D.tz[k]) >> 1;
      const int PAR = (D.ll[i] + D.ll[k]) & 1;
      const int jmin = max(abs(jj - jl), abs(ji - jk)), jmax = min(jj + jl, ji + jk);
      const double s0 = d_sgn((jl + jk + Jtot) >> 1);
      for (int JP = jmin; JP <= jmax; JP += 2) {
        const int qx = (JP >> 1) + Tz * (D.JM + 1) + PAR * 2 * (D.JM + 1);
        const double* W = WCC + D.wcc_off[qx];
        const int64_t rl = D.cc_rlen[qx];
        const int h = JP >> 1;
        const int64_t rjl = D.ccr[(j * N + l) * NJ + h], rik = D.ccr[(i * N + k) * NJ + h];
        const int64_t gjl = D.ccr[(l * N + j) * NJ + h], gik = D.ccr[(k * N + i) * NJ + h];
        if ((rjl | rik | gjl | gik) < 0) continue;  // cannot happen for channel-conserving pairs
        sm -= s0 * ((W[gik + rjl * rl] + phase * W[gjl + rik * rl]) * hL -
                    (phase * W[rik + gjl * rl] + W[rjl + gik * rl]) * hR) *
              d_sixj(D, ji, jj, Jtot, jl, jk, JP);
      }
    }
    {
      const int Tz = abs(D.tz[i] - D.tz[l]) >> 1;
      const int PAR = (D.ll[i] + D.ll[l]) & 1;
      const int jmin = max(abs(ji - jl), abs(jj - jk)), jmax = min(ji + jl, jj + jk);
      for (int JP = jmin; JP <= jmax; JP += 2) {
        const int qx = (JP >> 1) + Tz * (D.JM + 1) + PAR * 2 * (D.JM + 1);
        const double* W = WCC + D.wcc_off[qx];
        const int64_t rl = D.cc_rlen[qx];
        const int h = JP >> 1;
        const int64_t ril = D.ccr[(i * N + l) * NJ + h], rjk = D.ccr[(j * N + k) * NJ + h];
        const int64_t gil = D.ccr[(l * N + i) * NJ + h], gjk = D.ccr[(k * N + j) * NJ + h];
        if ((ril | rjk | gil | gjk) < 0) continue;
        sm += ((W[gil + rjk * rl] + phase * W[gjk + ril * rl]) * hL -
               (phase * W[ril + gjk * rl] + W[rjk + gil * rl]) * hR) *
              d_sixj(D, ji, jj, Jtot, jk, jl, JP);
      }
    }
    const int kk = q * 6 + g;
    double* X = RES + D.goff[kk];
    const int n1 = D.gn1[kk];
    const double v = X[IX + (int64_t)JX * n1] + sm * pre * pre2;
    X[IX + (int64_t)JX * n1] = v;
    if (g == 0 || g == 3 || g == 4) X[JX + (int64_t)IX * n1] = v * hRES;
  }
}

// ---------------------------------------------------------------- one-body pieces
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// commutator_111 (src/commutators.f90:36-80): one warp per output of fhh, fph, fpp
// (lanes split the contractions), ASSIGNS the one-body part
__global__ void k_comm111(DevLayout D, const double* __restrict__ L, int hL, const double* __restrict__ R, int hR,
                          double* __restrict__ RES) {
  const int A = D.A, P = D.P;
  const int total = A * A + P * A + P * P;
  const int lane = threadIdx.x & 31;
  const double *Lhh = L + D.off_fhh, *Rhh = R + D.off_fhh, *Lph = L + D.off_fph, *Rph = R + D.off_fph;
  const double *Lpp = L + D.off_fpp, *Rpp = R + D.off_fpp;
  for (int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < total; t += (gridDim.x * blockDim.x) >> 5) {
    if (t < A * A) {
      const int i = t % A, j = t / A;
      double th1 = 0, th2 = 0, th1t = 0, th2t = 0;
      for (int k = lane; k < A; k += 32) {
        th1 += Lhh[i + k * A] * Rhh[k + j * A];
        th1t += Lhh[j + k * A] * Rhh[k + i * A];
      }
      for (int p = lane; p < P; p += 32) {
        th2 += Lph[p + i * P] * Rph[p + j * P];
        th2t += Lph[p + j * P] * Rph[p + i * P];
      }
      th1 = warp_sum(th1); th2 = warp_sum(th2); th1t = warp_sum(th1t); th2t = warp_sum(th2t);
      if (lane == 0) RES[D.off_fhh + t] = th1 + th2 * hL - (th1t * hL + th2t) * hR;
    } else if (t < A * A + P * A) {
      const int s = t - A * A;
      const int p = s % P, i = s / P;
      double a1 = 0, a2 = 0, b1 = 0, b2 = 0;
      for (int k = lane; k < A; k += 32) {
        a1 += Lph[p + k * P] * Rhh[k + i * A];
        b1 += Rph[p + k * P] * Lhh[k + i * A];
      }
      for (int r = lane; r < P; r += 32) {
        a2 += Lpp[p + (int64_t)r * P] * Rph[r + i * P];
        b2 += Rpp[p + (int64_t)r * P] * Lph[r + i * P];
      }
      a1 = warp_sum(a1); a2 = warp_sum(a2); b1 = warp_sum(b1); b2 = warp_sum(b2);
      if (lane == 0) RES[D.off_fph + s] = (a1 + a2) - b1 - b2;
    } else {
      const int s = t - A * A - P * A;
      const int p = s % P, r = s / P;
      double tp1 = 0, tp2 = 0, tp1t = 0, tp2t = 0;
      for (int k = lane; k < A; k += 32) {
        tp1 += Lph[p + k * P] * Rph[r + k * P];
        tp1t += Lph[r + k * P] * Rph[p + k * P];
      }
      for (int m = lane; m < P; m += 32) {
        tp2 += Lpp[p + (int64_t)m * P] * Rpp[m + (int64_t)r * P];
        tp2t += Lpp[r + (int64_t)m * P] * Rpp[m + (int64_t)p * P];
      }
      tp1 = warp_sum(tp1); tp2 = warp_sum(tp2); tp1t = warp_sum(tp1t); tp2t = warp_sum(tp2t);
      if (lane == 0) RES[D.off_fpp + s] = tp1 * hR + tp2 - (tp1t + tp2t * hR) * hL;
    }
  }
}

__device__ __forceinline__ double* ob_ptr(const DevLayout& D, double* op, int kind, int p, int q) {
  if (kind == 0) return op + D.off_fhh + p + (int64_t)q * D.A;
  if (kind == 1) return op + D.off_fpp + p + (int64_t)q * D.P;
  return op + D.off_fph + p + (int64_t)q * D.P;
}

// commutator_121 (src/commutators.f90:83-280): one warp per one-body output (ACCUMULATE)
__global__ void k_comm121(DevLayout D, const double* __restrict__ L, int hL, const double* __restrict__ R, int hR,
                          double* __restrict__ RES, int hRES) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= D.n_ob) return;
  const int kind = D.ob_kind[warp], p = D.ob_p[warp], q = D.ob_q[warp], pk = D.ob_pk[warp], qk = D.ob_qk[warp];
  const int jq = D.jj[qk];
  double sm = 0.0;
  for (int t = lane; t < D.n_ai; t += 32) {
    const int a = D.ai_a[t], i = D.ai_i[t];
    const int ak = D.parts[a], ik = D.holes[i];
    const int ji = D.jj[ik];
    double smx = 0, smy = 0, smx2 = 0, smy2 = 0;
    VRef r;
    for (int JT = abs(ji - jq); JT <= ji + jq; JT += 2) {
      if (d_vref(D, ak, pk, ik, qk, JT, r)) {
        smx += R[r.idx] * (r.herm ? hR * r.pre : r.pre) * (JT + 1);
        smx2 += L[r.idx] * (r.herm ? hL * r.pre : r.pre) * (JT + 1);
      }
      if (d_vref(D, ik, pk, ak, qk, JT, r)) {
        smy += R[r.idx] * (r.herm ? hR * r.pre : r.pre) * (JT + 1);
        smy2 += L[r.idx] * (r.herm ? hL * r.pre : r.pre) * (JT + 1);
      }
    }
    const double lph = L[D.off_fph + a + (int64_t)i * D.P], rph = R[D.off_fph + a + (int64_t)i * D.P];
    sm += lph * (hL * smx - smy) - rph * (hR * smx2 - smy2);
  }
  sm = warp_sum(sm);
  if (lane == 0) {
    double* f = ob_ptr(D, RES, kind, p, q);
    const double v = *f + sm / (D.jj[pk] + 1.0);
    *f = v;
    if (kind < 2) *ob_ptr(D, RES, kind, q, p) = v * hRES;
  }
}

// commutator_221 (src/commutators.f90:435-578): one warp per one-body output (ACCUMULATE);
// w1, w2 are the hermitian intermediates of 222_pp_hh.
__global__ void k_comm221(DevLayout D, int pm, double* __restrict__ RES, int hRES, const double* __restrict__ w1,
                          const double* __restrict__ w2) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= D.n_ob) return;
  const int kind = D.ob_kind[warp], p = D.ob_p[warp], q = D.ob_q[warp], ik = D.ob_pk[warp], jk = D.ob_qk[warp];
  const int ji = D.jj[ik];
  double sm = 0.0;
  for (int ck = lane; ck < D.N; ck += 32) {
    const double* w = D.con[ck] ? w1 : w2;
    const int jc = D.jj[ck];
    for (int JT = abs(jc - ji); JT <= jc + ji; JT += 2) {
      double v = d_v_elem(D, w, 1, ck, ik, ck, jk, JT);
      if (kind < 2) v -= pm * d_v_elem(D, w, 1, ck, jk, ck, ik, JT);
      sm += v * (JT + 1);
    }
  }
  sm = warp_sum(sm);
  if (lane == 0) {
    double* f = ob_ptr(D, RES, kind, p, q);
    const double v = *f + sm / (ji + 1.0);
    *f = v;
    if (kind < 2) *ob_ptr(D, RES, kind, q, p) = v * hRES;
  }
}

// commutator_110 + commutator_220 (src/commutators.f90:10-33, 399-432), stage 1: block q
// sums the 220 contribution of channel q, block nblocks the 110 sum (fixed order).
__global__ void k_e0_partial(DevLayout D, const double* __restrict__ L, int hL, const double* __restrict__ R, int hR,
                             double* __restrict__ partial) {
  __shared__ double red[256];
  const int q = blockIdx.x;
  double acc = 0.0;
  if (q == D.nblocks) {
    const int A = D.A, P = D.P;
    for (int t = threadIdx.x; t < A * P; t += blockDim.x) {
      const int i = t / P;
      const double lv = L[D.off_fph + t], rv = R[D.off_fph + t];
      acc += (lv * rv * hL - rv * lv * hR) * (D.jj[D.holes[i]] + 1);
    }
  } else if (hR * hL == -1) {
    const int np = D.ncls[q * 3], nh = D.ncls[q * 3 + 2];
    const int64_t n = (int64_t)np * nh;
    const double* XL = L + D.goff[q * 6 + 2];
    const double* XR = R + D.goff[q * 6 + 2];
    for (int64_t t = threadIdx.x; t < n; t += blockDim.x) acc -= XL[t] * XR[t] * hR;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[q] = (q == D.nblocks) ? red[0] : red[0] * (D.lamJ[q] + 1);
}

// stage 2: out[0] = 110, out[1] = 220 and, when RES is given, RES%E0 = 110 + 220 (ASSIGN)
__global__ void k_e0_final(DevLayout D, const double* __restrict__ partial, double* __restrict__ RES,
                           double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s220 = 0.0;
  for (int q = 0; q < D.nblocks; ++q) s220 += partial[q];
  const double e110 = partial[D.nblocks], e220 = s220 * 2.0;
  if (out) { out[0] = e110; out[1] = e220; }
  if (RES) RES[0] = e110 + e220;
}

}  // namespace imsrg
