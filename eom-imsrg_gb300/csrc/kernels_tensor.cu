// FP64 kernels of the scalar-tensor commutator [L (scalar), R (rank lambda)] of BCH_TENSOR
// (src/TS_commutators.f90).  Each kernel restates one TS_commutator routine over the device
// tables of dev.cuh / tensor.h and keeps its assign / accumulate semantics.
#include "dev.cuh"
#include "kernels.h"
#include "tensor.h"

namespace imsrg {

namespace {

__device__ __forceinline__ double wsum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// {J1 J2 rank; j4 j5 j6} (j4 up to jmax + rank)
__device__ __forceinline__ double d_six_t(const DevTLayout& T, int J1, int J2, int j4, int j5, int j6) {
  const int a = J1 >> 1, b = J2 >> 1, x = (j4 - 1) >> 1, y = (j5 - 1) >> 1, z = (j6 - 1) >> 1;
  if (a < 0 || b < 0 || a >= T.six_nJ || b >= T.six_nJ || x < 0 || x >= T.six_nhx || y < 0 || y >= T.six_nh ||
      z < 0 || z >= T.six_nh)
    return 0.0;
  const int nh = T.six_nh;
  return __ldg(T.six + (((size_t)a * T.six_nJ + b) * T.six_nhx + x) * nh * nh + (size_t)y * nh + z);
}

// {c d J2; b x J4} (x up to jmax + rank)
__device__ __forceinline__ double d_six_m(const DevTLayout& T, int c, int d, int J2, int b, int x, int J4) {
  const int nh = T.six_nh, nJ = T.six_nJ;
  const int ic = (c - 1) >> 1, id = (d - 1) >> 1, ib = (b - 1) >> 1, ix = (x - 1) >> 1, a2 = J2 >> 1, a4 = J4 >> 1;
  if (ic < 0 || ic >= nh || id < 0 || id >= nh || ib < 0 || ib >= nh || ix < 0 || ix >= T.six_nhx || a2 < 0 ||
      a2 >= nJ || a4 < 0 || a4 >= nJ)
    return 0.0;
  return __ldg(T.six_m + ((((size_t)ic * nh + id) * nh + ib) * T.six_nhx + ix) * nJ * nJ + (size_t)a2 * nJ + a4);
}

// 9j {a b J1; c d J2; J3 J4 rank} by the sum of ninej (src/basic_IMSRG.f90:4425-4444)
__device__ double d_nine(const DevTLayout& T, int a, int b, int J1, int c, int d, int J2, int J3, int J4) {
  const int rank = T.rank;
  const int xmin = max(max(abs(J2 - b), abs(a - rank)), abs(J4 - c));
  const int xmax = min(min(J2 + b, a + rank), J4 + c);
  double sm = 0.0;
  for (int x = xmin; x <= xmax; x += 2)
    sm -= (x + 1.0) * d_six_t(T, J1, J2, x, a, b) * d_six_m(T, c, d, J2, b, x, J4) * d_six_t(T, J3, J4, x, a, c);
  return sm;
}

__device__ __forceinline__ int d_tg(int c1, int c2) {
  // (bra class, ket class) -> tgam index: pp-pp 0 pp-ph 1 pp-hh 2 ph-ph 3 hh-hh 4 ph-hh 5 hh-pp 6 ph-pp 7 hh-ph 8
  return c1 == 0 ? c2 : (c1 == 1 ? (c2 == 0 ? 7 : (c2 == 1 ? 3 : 5)) : (c2 == 0 ? 6 : (c2 == 1 ? 8 : 4)));
}

__device__ __forceinline__ int d_tblock(const DevLayout& D, const DevTLayout& T, int J1, int J2, int tz, int p) {
  if (J2 < J1 || J2 - J1 > T.rank || J1 > 2 * D.JM) return -1;
  return T.lut[(((J1 >> 1) * (T.rank / 2 + 1) + ((J2 - J1) >> 1)) * 3 + (tz + 1)) * 2 + p];
}

struct TRef {
  int64_t idx;
  double f;
};

// position and factor of tensor_elem(a,b,c,d,J1,J2) (src/basic_IMSRG.f90:1548-1684)
__device__ bool d_tref(const DevLayout& D, const DevTLayout& T, int herm, int ax, int bx, int cx, int dx, int J1x,
                       int J2x, TRef& r) {
  int a = ax, b = bx, c = cx, d = dx, J1 = J1x, J2 = J2x;
  double phase = 1.0;
  if (J1x > J2x) {
    a = cx; b = dx; c = ax; d = bx;
    J1 = J2x; J2 = J1x;
    phase = d_sgn((J1 - J2) >> 1) * herm;
  }
  if (!d_tri(J1, J2, T.rank)) return false;
  const int ja = D.jj[a], jb = D.jj[b], jc = D.jj[c], jd = D.jj[d];
  if (!(d_tri(ja, jb, J1) && d_tri(jc, jd, J2))) return false;
  const int P = (D.ll[a] + D.ll[b]) & 1;
  const int Pk = (T.dpar >> 1) & 1 ? 1 - P : P;
  if (((D.ll[c] + D.ll[d]) & 1) != Pk) return false;
  const int tab = D.tz[a] + D.tz[b];
  if (D.tz[c] + D.tz[d] != tab) return false;
  const int q = d_tblock(D, T, J1, J2, tab >> 1, P);
  if (q < 0 || T.q1[q] < 0) return false;
  const int g = d_tg(D.con[a] + D.con[b], D.con[c] + D.con[d]);
  const int N = D.N, NJ = D.NJ;
  double pre = 1.0;
  int i1, i2;
  if (a > b) {
    i1 = D.pairpos[(b * N + a) * NJ + (J1 >> 1)];
    pre = d_sgn(1 + ((ja + jb - J1) >> 1));
  } else {
    if (a == b) pre = 1.4142135623730951;
    i1 = D.pairpos[(a * N + b) * NJ + (J1 >> 1)];
  }
  if (c > d) {
    i2 = D.pairpos[(d * N + c) * NJ + (J2 >> 1)];
    pre *= d_sgn(1 + ((jc + jd - J2) >> 1));
  } else {
    if (c == d) pre *= 1.4142135623730951;
    i2 = D.pairpos[(c * N + d) * NJ + (J2 >> 1)];
  }
  const int k = q * 9 + g;
  r.idx = T.goff[k] + i1 + (int64_t)i2 * T.n1[k];
  r.f = pre * phase;
  return true;
}

__device__ __forceinline__ double d_telem(const DevLayout& D, const DevTLayout& T, const double* op, int herm, int a,
                                          int b, int c, int d, int J1, int J2) {
  TRef r;
  return d_tref(D, T, herm, a, b, c, d, J1, J2, r) ? op[r.idx] * r.f : 0.0;
}

// f_tensor_elem (src/basic_IMSRG.f90:1261-1290)
__device__ __forceinline__ double d_ftelem(const DevLayout& D, const DevTLayout& T, const double* op, int herm, int a,
                                           int b) {
  const int c1 = D.con[a], c2 = D.con[b];
  if (c1 + c2 == 0) return op[T.off_fpp + D.loc[a] + (int64_t)D.loc[b] * D.P];
  if (c1 + c2 == 2) return op[T.off_fhh + D.loc[a] + (int64_t)D.loc[b] * D.A];
  if (c1 > c2) return op[T.off_fph + D.loc[b] + (int64_t)D.loc[a] * D.P] * herm * d_sgn((D.jj[a] - D.jj[b]) >> 1);
  return op[T.off_fph + D.loc[a] + (int64_t)D.loc[b] * D.P];
}

__device__ __forceinline__ double* tob_at(const DevLayout& D, const DevTLayout& T, double* op, int kind, int p, int q) {
  if (kind == 0) return op + T.off_fhh + p + (int64_t)q * D.A;
  if (kind == 1) return op + T.off_fpp + p + (int64_t)q * D.P;
  return op + T.off_fph + p + (int64_t)q * D.P;
}

// RES(p,q) += sm and the mirror RES(q,p) = RES(p,q) herm (-1)^((jp-jq)/2) (src/TS_commutators.f90:143-144)
__device__ __forceinline__ void tob_acc(const DevLayout& D, const DevTLayout& T, double* RES, int hRES, int kind, int p,
                                        int q, int pk, int qk, double sm) {
  double* f = tob_at(D, T, RES, kind, p, q);
  const double v = *f + sm;
  *f = v;
  if (kind < 2) *tob_at(D, T, RES, kind, q, p) = v * hRES * d_sgn((D.jj[pk] - D.jj[qk]) >> 1);
}

// (q, g, IX, JX, a, b, c, d) of tensor two-body element e (0 <= e < n2b)
__device__ __forceinline__ void d_tdecode(const DevLayout& D, const DevTLayout& T, int64_t e, int& q, int& g, int& a,
                                          int& b, int& c, int& d) {
  const int64_t x = T.goff[0] + e;
  int lo = 0, hi = T.nblocks * 9;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (T.goff[mid] <= x) lo = mid; else hi = mid;
  }
  while (lo + 1 < T.nblocks * 9 && T.goff[lo + 1] <= x) ++lo;
  q = lo / 9;
  g = lo - q * 9;
  const int n1 = T.n1[lo];
  const int64_t loc = x - T.goff[lo];
  const int JX = (int)(loc / n1), IX = (int)(loc - (int64_t)JX * n1);
  const int c1 = (g < 3) ? 0 : ((g == 4 || g == 6 || g == 8) ? 2 : 1);
  const int c2 = (g == 0 || g == 6 || g == 7) ? 0 : ((g == 1 || g == 3 || g == 8) ? 1 : 2);
  const int o1 = D.pair_off[T.q1[q] * 3 + c1] + IX, o2 = D.pair_off[T.q2[q] * 3 + c2] + JX;
  a = D.pair_a[o1]; b = D.pair_b[o1]; c = D.pair_a[o2]; d = D.pair_b[o2];
}

}  // namespace

// ---------------------------------------------------------------- TS_commutator_111
// src/TS_commutators.f90:10-55: one warp per one-body element, ASSIGNS
__global__ void k_ts111(DevLayout D, DevTLayout T, const double* __restrict__ L, int hL, const double* __restrict__ R,
                        int hR, double* __restrict__ RES) {
  const int A = D.A, P = D.P;
  const int total = A * A + P * A + P * P;
  const int lane = threadIdx.x & 31;
  const double *Lhh = L + D.off_fhh, *Lph = L + D.off_fph, *Lpp = L + D.off_fpp;
  const double *Rhh = R + T.off_fhh, *Rph = R + T.off_fph, *Rpp = R + T.off_fpp;
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
      th1 = wsum(th1); th2 = wsum(th2); th1t = wsum(th1t); th2t = wsum(th2t);
      const double ph = d_sgn((D.jj[D.holes[i]] - D.jj[D.holes[j]]) >> 1);
      if (lane == 0) RES[T.off_fhh + t] = th1 + th2 * hL - (th1t * hL + th2t) * hR * ph;
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
      a1 = wsum(a1); a2 = wsum(a2); b1 = wsum(b1); b2 = wsum(b2);
      if (lane == 0) RES[T.off_fph + s] = (a1 + a2) - b1 - b2;
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
      tp1 = wsum(tp1); tp2 = wsum(tp2); tp1t = wsum(tp1t); tp2t = wsum(tp2t);
      const double ph = d_sgn((D.jj[D.parts[p]] - D.jj[D.parts[r]]) >> 1);
      if (lane == 0) RES[T.off_fpp + s] = tp1 * hR * ph + tp2 - (tp1t + tp2t * hR * ph) * hL;
    }
  }
}

// ---------------------------------------------------------------- TS_commutator_121
// src/TS_commutators.f90:58-303: one warp per tensor one-body output, lanes over (a, i)
__global__ void k_ts121(DevLayout D, DevTLayout T, const double* __restrict__ L, int hL, const double* __restrict__ R,
                        int hR, double* __restrict__ RES, int hRES) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= T.n_ob) return;
  const int kind = T.ob_kind[w], p = T.ob_p[w], q = T.ob_q[w], pk = T.ob_pk[w], qk = T.ob_qk[w];
  const int jp = D.jj[pk], jq = D.jj[qk], rank = T.rank;
  double sm = 0.0;
  for (int t = lane; t < D.n_ai; t += 32) {
    const int a = D.ai_a[t], i = D.ai_i[t];
    const int ak = D.parts[a], ik = D.holes[i];
    const int ja = D.jj[ak], ji = D.jj[ik];
    double smx = 0.0, smy = 0.0;
    for (int J2 = abs(ji - jq); J2 <= ji + jq; J2 += 2)
      for (int J1 = abs(ja - jp); J1 <= ja + jp; J1 += 2)
        smx += d_telem(D, T, R, hR, ak, pk, ik, qk, J1, J2) * sqrt((J1 + 1.0) * (J2 + 1.0)) * d_sgn(J1 >> 1) *
               d_six_t(T, J1, J2, jq, jp, ji);
    for (int J1 = abs(ji - jp); J1 <= ji + jp; J1 += 2)
      for (int J2 = abs(ja - jq); J2 <= ja + jq; J2 += 2)
        smy += d_telem(D, T, R, hR, ik, pk, ak, qk, J1, J2) * sqrt((J1 + 1.0) * (J2 + 1.0)) * d_sgn(J1 >> 1) *
               d_six_t(T, J1, J2, jq, jp, ji);
    sm += L[D.off_fph + a + (int64_t)i * D.P] * (hL * smx - smy) * d_sgn((rank + jq + ji) >> 1);
  }
  sm = wsum(sm);
  if (lane == 0) tob_acc(D, T, RES, hRES, kind, p, q, pk, qk, sm);
}

// ---------------------------------------------------------------- TS_commutator_211
// src/TS_commutators.f90:307-552: -[R1, L2] through the cross-coupled scalar L (channel JC = rank)
__global__ void k_ts211(DevLayout D, DevTLayout T, const double* __restrict__ LCC, int hL,
                        const double* __restrict__ R, int hR, double* __restrict__ RES, int hRES) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= T.n_ob) return;
  const int kind = T.ob_kind[w], p = T.ob_p[w], q = T.ob_q[w], pk = T.ob_pk[w], qk = T.ob_qk[w];
  const int jp = D.jj[pk], jq = D.jj[qk], rank = T.rank, dp = T.dpar >> 1;
  const int N = D.N, NJ = D.NJ;
  double sm = 0.0;
  for (int t = lane; t < D.P * D.A; t += 32) {
    const int a = t % D.P, i = t / D.P;
    const int ak = D.parts[a], ik = D.holes[i];
    const int ja = D.jj[ak], ji = D.jj[ik];
    if ((D.ll[ik] & 1) != ((D.ll[ak] + dp) & 1)) continue;
    if (D.tz[ik] != D.tz[ak]) continue;
    if (!d_tri(ja, ji, rank)) continue;
    const int Tz = abs(D.tz[ak] - D.tz[ik]) >> 1;
    if (abs(D.tz[pk] - D.tz[qk]) != Tz * 2) continue;
    const int PAR = (D.ll[ak] + D.ll[ik]) & 1;
    if (((D.ll[pk] + D.ll[qk]) & 1) != PAR) continue;
    const int qx = (rank >> 1) + Tz * (D.JM + 1) + PAR * 2 * (D.JM + 1);
    const int rai = T.ccnb[(ak * N + ik) * NJ + (rank >> 1)];
    const int rpq = D.ccr[(pk * N + qk) * NJ + (rank >> 1)];
    const int rqp = D.ccr[(qk * N + pk) * NJ + (rank >> 1)];
    if (rai < 0 || rpq < 0 || rqp < 0) continue;
    const double* X = LCC + D.cc_off[qx];
    const int64_t rl = D.cc_rlen[qx];
    sm += R[T.off_fph + a + (int64_t)i * D.P] *
          (d_sgn((jp - jq + rank) >> 1) * X[rpq + rai * rl] - hR * hL * d_sgn(rank >> 1) * X[rqp + rai * rl]) /
          sqrt(rank + 1.0);
  }
  sm = wsum(sm);
  if (lane == 0) tob_acc(D, T, RES, hRES, kind, p, q, pk, qk, sm);
}

// ---------------------------------------------------------------- TS_commutator_221
// src/TS_commutators.f90:809-1067: one-body traces of the tensor intermediates w1 (hole c), w2 (particle c)
__global__ void k_ts221(DevLayout D, DevTLayout T, const double* __restrict__ w1, const double* __restrict__ w2,
                        int pm, double* __restrict__ RES, int hRES) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= T.n_ob) return;
  const int kind = T.ob_kind[w], p = T.ob_p[w], q = T.ob_q[w], ik = T.ob_pk[w], jk = T.ob_qk[w];
  const int ji = D.jj[ik], jj = D.jj[jk], rank = T.rank;
  double sm = 0.0;
  for (int c = lane; c < D.N; c += 32) {
    const double* wx = D.con[c] ? w1 : w2;
    const int jc = D.jj[c];
    double s = 0.0;
    for (int J1 = abs(jc - ji); J1 <= jc + ji; J1 += 2) {
      for (int J2 = abs(jc - jj); J2 <= min(J1 - 2, jc + jj); J2 += 2)
        s -= sqrt((J1 + 1.0) * (J2 + 1.0)) * d_six_t(T, J1, J2, jj, ji, jc) *
             d_telem(D, T, wx, 1, c, jk, c, ik, J2, J1) * d_sgn(J2 >> 1) * pm;
      for (int J2 = max(J1, abs(jc - jj)); J2 <= jc + jj; J2 += 2)
        s += sqrt((J1 + 1.0) * (J2 + 1.0)) * d_six_t(T, J1, J2, jj, ji, jc) *
             d_telem(D, T, wx, 1, c, ik, c, jk, J1, J2) * d_sgn(J1 >> 1);
    }
    sm += s * d_sgn((jc + jj) >> 1);
  }
  sm = wsum(sm);
  if (lane == 0) tob_acc(D, T, RES, hRES, kind, p, q, ik, jk, sm * d_sgn(rank >> 1));
}

// ---------------------------------------------------------------- TS_commutator_122 / 212
// src/TS_commutators.f90:555-663 (ASSIGNS) and :666-806 (ACCUMULATES): one thread per two-body element
// element x of a segment list (binary search over the prefix counts); x itself without one
__device__ __forceinline__ int64_t d_seg_elem(const ElemSegs& sg, int64_t x) {
  if (!sg.n) return x;
  int lo = 0, hi = sg.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (sg.pre[mid] <= x) lo = mid;
    else hi = mid - 1;
  }
  return sg.off[lo] + (x - sg.pre[lo]);
}

__global__ void k_ts122(DevLayout D, DevTLayout T, const double* __restrict__ L, int hL, const double* __restrict__ R,
                        int hR, double* __restrict__ RES, ElemSegs sg) {
  const int64_t ntot = sg.n ? sg.pre[sg.n] : T.n2b;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < ntot; x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = d_seg_elem(sg, x);
    int q, g, a, b, c, d;
    d_tdecode(D, T, e, q, g, a, b, c, d);
    const int J1 = T.J1[q], J2 = T.J2[q];
    double sm = 0.0;
    for (int t = 0, s0 = D.same_start[a], n = D.same_count[a]; t < n; ++t) {
      const int i = D.same_list[s0 + t];
      sm += d_f_elem(D, L, hL, a, i) * d_telem(D, T, R, hR, i, b, c, d, J1, J2);
    }
    for (int t = 0, s0 = D.same_start[b], n = D.same_count[b]; t < n; ++t) {
      const int i = D.same_list[s0 + t];
      sm += d_f_elem(D, L, hL, b, i) * d_telem(D, T, R, hR, a, i, c, d, J1, J2);
    }
    for (int t = 0, s0 = D.same_start[c], n = D.same_count[c]; t < n; ++t) {
      const int i = D.same_list[s0 + t];
      sm -= d_f_elem(D, L, hL, i, c) * d_telem(D, T, R, hR, a, b, i, d, J1, J2);
    }
    for (int t = 0, s0 = D.same_start[d], n = D.same_count[d]; t < n; ++t) {
      const int i = D.same_list[s0 + t];
      sm -= d_f_elem(D, L, hL, i, d) * d_telem(D, T, R, hR, a, b, c, i, J1, J2);
    }
    RES[T.goff[0] + e] = sm / sqrt(1.0 + (a == b ? 1.0 : 0.0)) / sqrt(1.0 + (c == d ? 1.0 : 0.0));
  }
}

__global__ void k_ts212(DevLayout D, DevTLayout T, const double* __restrict__ L, int hL, const double* __restrict__ R,
                        int hR, double* __restrict__ RES, ElemSegs sg) {
  const int rank = T.rank;
  const int64_t ntot = sg.n ? sg.pre[sg.n] : T.n2b;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < ntot; x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = d_seg_elem(sg, x);
    int q, g, a, b, c, d;
    d_tdecode(D, T, e, q, g, a, b, c, d);
    const int J1 = T.J1[q], J2 = T.J2[q];
    const int ja = D.jj[a], jb = D.jj[b], jc = D.jj[c], jd = D.jj[d];
    // each sum runs over the orbits the tensor one-body element can couple (tz, parity, rank)
    double s1 = 0.0, s2 = 0.0, s3 = 0.0, s4 = 0.0;
    for (int t = 0, s0 = T.tnb_start[a], n = T.tnb_count[a]; t < n; ++t) {
      const int i = T.tnb_list[s0 + t];
      s1 -= d_six_t(T, J1, J2, D.jj[i], ja, jb) * d_ftelem(D, T, R, hR, a, i) * d_v_elem(D, L, hL, i, b, c, d, J2);
    }
    for (int t = 0, s0 = T.tnb_start[b], n = T.tnb_count[b]; t < n; ++t) {
      const int i = T.tnb_list[s0 + t];
      s2 += d_six_t(T, J1, J2, D.jj[i], jb, ja) * d_ftelem(D, T, R, hR, b, i) * d_v_elem(D, L, hL, i, a, c, d, J2);
    }
    for (int t = 0, s0 = T.tnb_start[d], n = T.tnb_count[d]; t < n; ++t) {
      const int i = T.tnb_list[s0 + t];
      s3 += d_six_t(T, J1, J2, jd, D.jj[i], jc) * d_ftelem(D, T, R, hR, i, d) * d_v_elem(D, L, hL, a, b, c, i, J1);
    }
    for (int t = 0, s0 = T.tnb_start[c], n = T.tnb_count[c]; t < n; ++t) {
      const int i = T.tnb_list[s0 + t];
      s4 -= d_six_t(T, J1, J2, jc, D.jj[i], jd) * d_ftelem(D, T, R, hR, i, c) * d_v_elem(D, L, hL, a, b, d, i, J1);
    }
    const double sm = s1 * d_sgn((ja + jb - J2) >> 1) + s2 * d_sgn((J1 + J2) >> 1) + s3 * d_sgn((jc + jd - J1) >> 1) +
                      s4 * d_sgn((J2 + J1) >> 1);
    RES[T.goff[0] + e] += sm * sqrt((J1 + 1.0) * (J2 + 1.0) / (1.0 + (a == b ? 1.0 : 0.0)) /
                                    (1.0 + (c == d ? 1.0 : 0.0))) * d_sgn(rank >> 1);
  }
}

// RES(2b) += W1 - W2 (src/TS_commutators.f90:1107-1453)
__global__ void k_ts_pphh_update(int64_t n, int64_t off, double* __restrict__ RES, const double* __restrict__ w1,
                                 const double* __restrict__ w2) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    RES[off + e] = RES[off + e] + w1[off + e] - w2[off + e];
}

// ---------------------------------------------------------------- calculate_single_pandya
// src/cross_coupled.f90:1416-1634 for the cross-coupled tensor block (J3, J4, Tz, PAR):
// term 1 fills CCX (r1 x nb2: rows (a,b) of channel qa, ph columns (p,h) of channel qb),
// term 2 fills CCR (nb1 x r2: ph columns (p,h) of qa, rows (b,a) of qb); out is scaled by `scale`.
namespace {
// one element of the tensor Pandya transform (rows (a, b) / ph columns (p, h) as k_tpandya
// reads them); exc: zero unless the tensor element read is (pp,hh) or (hh,pp)
__device__ __forceinline__ double tpandya_at(const DevLayout& D, const DevTLayout& T, const double* __restrict__ R,
                                             int hR, int J3, int J4, int term, int a, int b, int p, int h, double norm,
                                             int exc) {
  const int dp = T.dpar >> 1;
  // an excitation operator has only (pp,hh) and (hh,pp) elements: the pairs (a,h) and (p,b) read
  // below must be of opposite classes
  const int ca = D.con[a] + D.con[h], cb = D.con[p] + D.con[b];
  const bool live = !exc || (ca == 0 && cb == 2) || (ca == 2 && cb == 0);
  if (!(live && ((D.ll[a] + D.ll[h]) & 1) == ((D.ll[b] + D.ll[p] + dp) & 1) && D.tz[a] + D.tz[h] == D.tz[b] + D.tz[p]))
    return 0.0;
  const int ja = D.jj[a], jb = D.jj[b], jp = D.jj[p], jh = D.jj[h];
  double sm = 0.0;
  for (int Ja = abs(ja - jh); Ja <= ja + jh; Ja += 2)
    for (int Jb = abs(jp - jb); Jb <= jp + jb; Jb += 2) {
      const double t = term == 1 ? d_telem(D, T, R, hR, a, h, p, b, Ja, Jb) : d_telem(D, T, R, hR, h, a, b, p, Ja, Jb);
      if (t == 0.0) continue;
      const double nj = term == 1 ? d_nine(T, ja, jb, J3, jh, jp, J4, Ja, Jb) : d_nine(T, jh, jp, J3, ja, jb, J4, Ja, Jb);
      sm -= d_sgn(Jb >> 1) * sqrt((Ja + 1.0) * (Jb + 1.0)) * nj * t;
    }
  return term == 1 ? sm * d_sgn((jh + jb + J4) >> 1) * norm : sm * d_sgn((jp + ja + J4) >> 1) * norm * d_sgn((jp + jh) >> 1);
}

// the block of a flattened element index (prefix counts pre[0..n], pre[0] = 0)
__device__ __forceinline__ int d_block_of(const int64_t* __restrict__ pre, int n, int64_t e) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= e) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
}  // namespace

__global__ void k_tpandya(DevLayout D, DevTLayout T, const double* __restrict__ R, int hR, int J3, int J4, int qa,
                          int qb, int term, double scale, double* __restrict__ out) {
  const int r1 = D.cc_rlen[qa], r2 = D.cc_rlen[qb];
  const int nb1 = D.cc_nph[qa], nb2 = D.cc_nph[qb];
  const int64_t n = term == 1 ? (int64_t)r1 * nb2 : (int64_t)nb1 * r2;
  const double norm = sqrt((J3 + 1.0) * (J4 + 1.0)) * scale;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    int a, b, p, h;
    if (term == 1) {
      const int col = (int)(e / r1), row = (int)(e - (int64_t)col * r1);
      a = D.cc_ra[D.cc_row_off[qa] + row]; b = D.cc_rb[D.cc_row_off[qa] + row];
      p = D.cc_cp[D.cc_col_off[qb] + col]; h = D.cc_ch[D.cc_col_off[qb] + col];
    } else {
      const int col = (int)(e / nb1), row = (int)(e - (int64_t)col * nb1);
      p = D.cc_cp[D.cc_col_off[qa] + row]; h = D.cc_ch[D.cc_col_off[qa] + row];
      b = D.cc_ra[D.cc_row_off[qb] + col]; a = D.cc_rb[D.cc_row_off[qb] + col];
    }
    out[e] = tpandya_at(D, T, R, hR, J3, J4, term, a, b, p, h, norm, 0);
  }
}

// Excitation mode, all cross-coupled tensor blocks in one launch: per block, the packed CCR
// (nb1 x nx, columns pe of qb, scale 1/sqrt(J3+1)) and then the packed CCX (ny x nb2, rows hp of
// qa, scale 1/sqrt(J4+1)); pre: prefix counts of nb1 nx + ny nb2 over the blocks
__global__ void k_tpandya_exc(DevLayout D, DevTLayout T, const double* __restrict__ R, int hR,
                              const ExcBlock* __restrict__ blk, const int64_t* __restrict__ pre, int nblk,
                              const int* __restrict__ pe, const int* __restrict__ hp, double* __restrict__ ccr,
                              double* __restrict__ ccx) {
  const int64_t n = pre[nblk];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int ib = d_block_of(pre, nblk, e);
    const ExcBlock B = blk[ib];
    const int64_t f = e - pre[ib];
    const int qa = B.qa, qb = B.qb, nb1 = D.cc_nph[qa];
    const double n34 = sqrt((B.J3 + 1.0) * (B.J4 + 1.0));
    if (f < (int64_t)nb1 * B.nx) {  // CCR
      const int c = (int)(f / nb1), row = (int)(f - (int64_t)c * nb1);
      const int col = pe[B.xs + c];
      const int p = D.cc_cp[D.cc_col_off[qa] + row], h = D.cc_ch[D.cc_col_off[qa] + row];
      const int b = D.cc_ra[D.cc_row_off[qb] + col], a = D.cc_rb[D.cc_row_off[qb] + col];
      ccr[B.ccr + f] = tpandya_at(D, T, R, hR, B.J3, B.J4, 2, a, b, p, h, n34 / sqrt(B.J3 + 1.0), 1);
    } else {  // CCX
      const int64_t g = f - (int64_t)nb1 * B.nx;
      const int col = (int)(g / B.ny), r = (int)(g - (int64_t)col * B.ny);
      const int row = hp[B.ys + r];
      const int a = D.cc_ra[D.cc_row_off[qa] + row], b = D.cc_rb[D.cc_row_off[qa] + row];
      const int p = D.cc_cp[D.cc_col_off[qb] + col], h = D.cc_ch[D.cc_col_off[qb] + col];
      ccx[B.ccx + g] = tpandya_at(D, T, R, hR, B.J3, B.J4, 1, a, b, p, h, n34 / sqrt(B.J4 + 1.0), 1);
    }
  }
}

namespace {
// add_elem_to_tensor (src/basic_IMSRG.f90:1687-1772): a <= b, c <= d, J1 <= J2
__device__ __forceinline__ void d_tadd(const DevLayout& D, const DevTLayout& T, double* RES, double V, int a, int b,
                                       int c, int d, int J1, int J2) {
  const int P = (D.ll[a] + D.ll[b]) & 1;
  const int q = d_tblock(D, T, J1, J2, (D.tz[a] + D.tz[b]) >> 1, P);
  if (q < 0) return;
  const int g = d_tg(D.con[a] + D.con[b], D.con[c] + D.con[d]);
  const int N = D.N, NJ = D.NJ;
  const int i1 = D.pairpos[(a * N + b) * NJ + (J1 >> 1)], i2 = D.pairpos[(c * N + d) * NJ + (J2 >> 1)];
  if (i1 < 0 || i2 < 0) return;
  double pre = 1.0;
  if (a == b) pre *= 1.4142135623730951;
  if (c == d) pre *= 1.4142135623730951;
  const int k = q * 9 + g;
  atomicAdd(RES + T.goff[k] + i1 + (int64_t)i2 * T.n1[k], V * pre);
}

__device__ __forceinline__ bool d_odd(int J) { return ((J >> 1) & 1) == 1; }

// one recoupling loop of TS_commutator_222_ph: J1 over [o1, o2], J2 over
// [max(J1, i1, |J1 - rank|), min(i2, J1 + rank)], 9j {n1 n2 J3; n3 n4 J4; J1 J2 rank}
template <class C>
__device__ __forceinline__ void recouple_loop(const DevLayout& D, const DevTLayout& T, double* RES, int J3, int J4,
                                              int o1, int o2, int i1, int i2, bool skip_o, bool skip_i, int n1, int n2,
                                              int n3, int n4, double p34, C coef, int a, int b, int c, int d,
                                              int exc) {
  if (exc) {  // only the (pp,hh) and (hh,pp) outputs are wanted
    const int g = d_tg(D.con[a] + D.con[b], D.con[c] + D.con[d]);
    if (g != 2 && g != 6) return;
  }
  for (int J1 = o1; J1 <= o2; J1 += 2) {
    if (skip_o && d_odd(J1)) continue;
    const double p134 = p34 * sqrt(J1 + 1.0);
    for (int J2 = max(max(J1, i1), abs(J1 - T.rank)); J2 <= min(i2, J1 + T.rank); J2 += 2) {
      if (skip_i && d_odd(J2)) continue;
      const double V = p134 * sqrt(J2 + 1.0) * d_nine(T, n1, n2, J3, n3, n4, J4, J1, J2) * coef(J1, J2);
      d_tadd(D, T, RES, V, a, b, c, d, J1, J2);
    }
  }
}
}  // namespace

// ---------------------------------------------------------------- TS_commutator_222_ph
// src/TS_commutators.f90:1529-1843 for one cross-coupled tensor block: every element of
// Wx (and Wy) above thresh in size recouples into the two-body tensor elements it feeds (ACCUMULATES);
// TS_commutator_222_ph uses thresh = 1e-6 (src/TS_commutators.f90:1562, 1714), the EOM product 0
namespace {
// the recouplings of one (Wx, Wy) element pair, rows (d, a) of qa and (c, b) of qb
__device__ __forceinline__ void ph_scatter_elem(const DevLayout& D, const DevTLayout& T, double* RES, int J3, int J4,
                                                int qa, int qb, int IX, int JX, double X, double Y, int hL, int hR,
                                                double thresh, int exc) {
  const int rank = T.rank;
  const double p34 = sqrt((J3 + 1.0) * (J4 + 1.0));
  const double ph34 = d_sgn((J3 + J4) >> 1);
  const int d = D.cc_ra[D.cc_row_off[qa] + IX], a = D.cc_rb[D.cc_row_off[qa] + IX];
  const int c = D.cc_ra[D.cc_row_off[qb] + JX], b = D.cc_rb[D.cc_row_off[qb] + JX];
  const int ja = D.jj[a], jb = D.jj[b], jc = D.jj[c], jd = D.jj[d];
  const double pabcd = d_sgn((ja + jb + jc + jd) >> 1);
  if (fabs(X) > thresh) {
    const int J1min = abs(ja - jb), J1max = ja + jb, J2min = abs(jc - jd), J2max = jc + jd;
    if (b >= a) {
      if (d >= c) {
        recouple_loop(D, T, RES, J3, J4, J1min, J1max, J2min, J2max, a == b, c == d, ja, jd, jb, jc, p34,
                      [&](int, int J2) { return d_sgn((jb + jd + J2) >> 1) * ph34 * hL * X; }, a, b, c, d, exc);
        recouple_loop(D, T, RES, J3, J4, J2min, J2max, J1min, J1max, c == d, a == b, jd, ja, jc, jb, p34,
                      [&](int J1, int) { return -d_sgn((jc + ja + J1 + rank) >> 1) * hR * X; }, c, d, a, b, exc);
      } else {
        recouple_loop(D, T, RES, J3, J4, J1min, J1max, J2min, J2max, a == b, false, ja, jd, jb, jc, p34,
                      [&](int, int) { return d_sgn((jb + jc) >> 1) * ph34 * hL * X; }, a, b, d, c, exc);
        recouple_loop(D, T, RES, J3, J4, J2min, J2max, J1min, J1max, false, a == b, jd, ja, jc, jb, p34,
                      [&](int, int) { return d_sgn((ja - jd + rank) >> 1) * hR * X; }, d, c, a, b, exc);
      }
    } else {
      if (d >= c) {
        recouple_loop(D, T, RES, J3, J4, J1min, J1max, J2min, J2max, false, c == d, ja, jd, jb, jc, p34,
                      [&](int J1, int J2) { return d_sgn((ja + jd + J1 + J2) >> 1) * ph34 * hL * X; }, b, a, c, d, exc);
        recouple_loop(D, T, RES, J3, J4, J2min, J2max, J1min, J1max, c == d, false, jd, ja, jc, jb, p34,
                      [&](int J1, int J2) { return d_sgn((jc - jb + J1 + J2 + rank) >> 1) * hR * X; }, c, d, b, a, exc);
      } else {
        recouple_loop(D, T, RES, J3, J4, J1min, J1max, J2min, J2max, false, false, ja, jd, jb, jc, p34,
                      [&](int J1, int) { return d_sgn((ja + jc + J1) >> 1) * ph34 * hL * X; }, b, a, d, c, exc);
        recouple_loop(D, T, RES, J3, J4, J2min, J2max, J1min, J1max, false, false, jd, ja, jc, jb, p34,
                      [&](int, int J2) { return d_sgn((jb - jd + J2 + rank) >> 1) * hR * X; }, d, c, b, a, exc);
      }
    }
  }
  if (fabs(Y) > thresh) {
    const int J1min = abs(jd - jb), J1max = jd + jb, J2min = abs(jc - ja), J2max = jc + ja;
    if (b >= d) {
      if (a >= c) {
        recouple_loop(D, T, RES, J3, J4, J1min, J1max, J2min, J2max, d == b, c == a, jd, ja, jb, jc, p34,
                      [&](int, int J2) { return d_sgn((jc + ja + J2) >> 1) * hL * Y; }, d, b, c, a, exc);
        recouple_loop(D, T, RES, J3, J4, J2min, J2max, J1min, J1max, c == a, b == d, ja, jd, jc, jb, p34,
                      [&](int J1, int) { return d_sgn((jd - jb + J1 + rank) >> 1) * ph34 * hR * Y; }, c, a, d, b, exc);
      } else {
        recouple_loop(D, T, RES, J3, J4, J1min, J1max, J2min, J2max, d == b, c == a, jd, ja, jb, jc, p34,
                      [&](int, int) { return -hL * Y; }, d, b, a, c, exc);
        recouple_loop(D, T, RES, J3, J4, J2min, J2max, J1min, J1max, a == c, b == d, ja, jd, jc, jb, p34,
                      [&](int, int) { return pabcd * ph34 * d_sgn(rank >> 1) * hR * Y; }, a, c, d, b, exc);
      }
    } else {
      if (a >= c) {
        recouple_loop(D, T, RES, J3, J4, J1min, J1max, J2min, J2max, b == d, a == c, jd, ja, jb, jc, p34,
                      [&](int J1, int J2) { return -pabcd * d_sgn((J1 + J2) >> 1) * hL * Y; }, b, d, c, a, exc);
        recouple_loop(D, T, RES, J3, J4, J2min, J2max, J1min, J1max, c == a, b == d, ja, jd, jc, jb, p34,
                      [&](int J1, int J2) { return d_sgn((J1 + J2 + rank) >> 1) * ph34 * hR * Y; }, c, a, b, d, exc);
      } else {
        recouple_loop(D, T, RES, J3, J4, J1min, J1max, J2min, J2max, b == d, a == c, jd, ja, jb, jc, p34,
                      [&](int J1, int) { return d_sgn((jb + jd + J1) >> 1) * hL * Y; }, b, d, a, c, exc);
        recouple_loop(D, T, RES, J3, J4, J2min, J2max, J1min, J1max, a == c, d == b, ja, jd, jc, jb, p34,
                      [&](int, int J2) { return d_sgn((ja - jc + J2 + rank) >> 1) * ph34 * hR * Y; }, a, c, b, d, exc);
      }
    }
  }
}
}  // namespace

__global__ void k_ts222ph_scatter(DevLayout D, DevTLayout T, const double* __restrict__ Wx,
                                  const double* __restrict__ Wy, int J3, int J4, int qa, int qb, int hL, int hR,
                                  double thresh, int exc, double* __restrict__ RES) {
  const int r1 = D.cc_rlen[qa], r2 = D.cc_rlen[qb];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)r1 * r2;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int JX = (int)(e / r1), IX = (int)(e - (int64_t)JX * r1);
    const double X = Wx[e], Y = Wy ? Wy[e] : 0.0;
    if (fabs(X) <= thresh && fabs(Y) <= thresh) continue;
    ph_scatter_elem(D, T, RES, J3, J4, qa, qb, IX, JX, X, Y, hL, hR, thresh, exc);
  }
}

// Excitation mode, all cross-coupled tensor blocks in one launch: per block, the elements of the
// packed Wx (r1 x nx, columns pe of qb) and then of Wy (ny x r2, rows hp of qa) recouple, into
// (pp,hh) and (hh,pp) outputs only; pre: prefix counts of r1 nx + ny r2 over the blocks
__global__ void k_ts222ph_scatter_exc(DevLayout D, DevTLayout T, const ExcBlock* __restrict__ blk,
                                      const int64_t* __restrict__ pre, int nblk, const int* __restrict__ pe,
                                      const int* __restrict__ hp, const double* __restrict__ Wx,
                                      const double* __restrict__ Wy, int hL, int hR, double* __restrict__ RES) {
  const int64_t n = pre[nblk];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int ib = d_block_of(pre, nblk, e);
    const ExcBlock B = blk[ib];
    const int64_t f = e - pre[ib];
    const int r1 = D.cc_rlen[B.qa];
    int IX, JX;
    double X = 0.0, Y = 0.0;
    if (f < (int64_t)r1 * B.nx) {
      const int c = (int)(f / r1);
      IX = (int)(f - (int64_t)c * r1);
      JX = pe[B.xs + c];
      X = Wx[B.wx + f];
    } else {
      const int64_t g = f - (int64_t)r1 * B.nx;
      JX = (int)(g / B.ny);
      const int r = (int)(g - (int64_t)JX * B.ny);
      IX = hp[B.ys + r];
      Y = Wy[B.wy + g];
    }
    if (X == 0.0 && Y == 0.0) continue;
    ph_scatter_elem(D, T, RES, B.J3, B.J4, B.qa, B.qb, IX, JX, X, Y, hL, hR, 0.0, 1);
  }
}


// ---------------------------------------------------------------- FP32 forms for the mixed modes
// The same sums as k_ts122 / k_ts212 in FP32 (FP64 elements converted with integer
// instructions, products and sums in FP32, the result added to the FP64 slab).
namespace {
__device__ __forceinline__ float d_six_tf(const DevTLayout& T, int J1, int J2, int j4, int j5, int j6) {
  const int a = J1 >> 1, b = J2 >> 1, x = (j4 - 1) >> 1, y = (j5 - 1) >> 1, z = (j6 - 1) >> 1;
  if (a < 0 || b < 0 || a >= T.six_nJ || b >= T.six_nJ || x < 0 || x >= T.six_nhx || y < 0 || y >= T.six_nh ||
      z < 0 || z >= T.six_nh)
    return 0.0f;
  const int nh = T.six_nh;
  return __ldg(T.six_f + (((size_t)a * T.six_nJ + b) * T.six_nhx + x) * nh * nh + (size_t)y * nh + z);
}

__device__ __forceinline__ float d_ftelem_f(const DevLayout& D, const DevTLayout& T, const double* op, int herm, int a,
                                            int b) {
  const int c1 = D.con[a], c2 = D.con[b];
  if (c1 + c2 == 0) return f64_to_f32(op[T.off_fpp + D.loc[a] + (int64_t)D.loc[b] * D.P]);
  if (c1 + c2 == 2) return f64_to_f32(op[T.off_fhh + D.loc[a] + (int64_t)D.loc[b] * D.A]);
  if (c1 > c2) {
    const float v = f64_to_f32(op[T.off_fph + D.loc[b] + (int64_t)D.loc[a] * D.P]);
    const bool neg = (herm < 0) != ((((D.jj[a] - D.jj[b]) >> 1) & 1) != 0);
    return neg ? -v : v;
  }
  return f64_to_f32(op[T.off_fph + D.loc[a] + (int64_t)D.loc[b] * D.P]);
}

__device__ __forceinline__ float d_velem_f(const DevLayout& D, const double* op, int herm, int a, int b, int c, int d,
                                           int J) {
  VRefF r;
  return d_vref_f(D, a, b, c, d, J, r) ? f64_to_f32(op[r.idx]) * r.scale(herm) : 0.0f;
}

// tensor_elem in FP32: the position from d_tref, its factor (+-1, +-sqrt 2, +-2) in FP32
__device__ __forceinline__ float d_telem_f(const DevLayout& D, const DevTLayout& T, const double* op, int herm, int a,
                                           int b, int c, int d, int J1, int J2) {
  TRef r;
  if (!d_tref(D, T, herm, a, b, c, d, J1, J2, r)) return 0.0f;
  const unsigned long long bits = (unsigned long long)__double_as_longlong(r.f);
  const bool neg = (bits >> 63) != 0;
  // |f| is 1, sqrt 2 or 2 (sqrt 2 squared, possibly an ulp above 2)
  const int e = (int)((bits >> 52) & 0x7FF) - 1023;
  const float m = e >= 1 ? 2.0f : ((bits & 0xFFFFFFFFFFFFFull) ? 1.41421356f : 1.0f);
  const float v = f64_to_f32(op[r.idx]) * m;
  return neg ? -v : v;
}
}  // namespace

__global__ void k_ts122f(DevLayout D, DevTLayout T, const double* __restrict__ L, int hL, const double* __restrict__ R,
                         int hR, double* __restrict__ RES, ElemSegs sg) {
  const int64_t ntot = sg.n ? sg.pre[sg.n] : T.n2b;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < ntot; x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = d_seg_elem(sg, x);
    int q, g, a, b, c, d;
    d_tdecode(D, T, e, q, g, a, b, c, d);
    const int J1 = T.J1[q], J2 = T.J2[q];
    float sm = 0.0f;
    for (int t = 0, s0 = D.same_start[a], n = D.same_count[a]; t < n; ++t) {
      const int i = D.same_list[s0 + t];
      sm += d_f_elem_f(D, L, hL, a, i) * d_telem_f(D, T, R, hR, i, b, c, d, J1, J2);
    }
    for (int t = 0, s0 = D.same_start[b], n = D.same_count[b]; t < n; ++t) {
      const int i = D.same_list[s0 + t];
      sm += d_f_elem_f(D, L, hL, b, i) * d_telem_f(D, T, R, hR, a, i, c, d, J1, J2);
    }
    for (int t = 0, s0 = D.same_start[c], n = D.same_count[c]; t < n; ++t) {
      const int i = D.same_list[s0 + t];
      sm -= d_f_elem_f(D, L, hL, i, c) * d_telem_f(D, T, R, hR, a, b, i, d, J1, J2);
    }
    for (int t = 0, s0 = D.same_start[d], n = D.same_count[d]; t < n; ++t) {
      const int i = D.same_list[s0 + t];
      sm -= d_f_elem_f(D, L, hL, i, d) * d_telem_f(D, T, R, hR, a, b, c, i, J1, J2);
    }
    const float nrm = ((a == b) ? 0.70710678f : 1.0f) * ((c == d) ? 0.70710678f : 1.0f);
    RES[T.goff[0] + e] = f32_to_f64(sm * nrm);
  }
}

__global__ void k_ts212f(DevLayout D, DevTLayout T, const double* __restrict__ L, int hL, const double* __restrict__ R,
                         int hR, double* __restrict__ RES, ElemSegs sg) {
  const int rank = T.rank;
  const int64_t ntot = sg.n ? sg.pre[sg.n] : T.n2b;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < ntot; x += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = d_seg_elem(sg, x);
    int q, g, a, b, c, d;
    d_tdecode(D, T, e, q, g, a, b, c, d);
    const int J1 = T.J1[q], J2 = T.J2[q];
    const int ja = D.jj[a], jb = D.jj[b], jc = D.jj[c], jd = D.jj[d];
    float s1 = 0.0f, s2 = 0.0f, s3 = 0.0f, s4 = 0.0f;
    for (int t = 0, s0 = T.tnb_start[a], n = T.tnb_count[a]; t < n; ++t) {
      const int i = T.tnb_list[s0 + t];
      s1 -= d_six_tf(T, J1, J2, D.jj[i], ja, jb) * d_ftelem_f(D, T, R, hR, a, i) * d_velem_f(D, L, hL, i, b, c, d, J2);
    }
    for (int t = 0, s0 = T.tnb_start[b], n = T.tnb_count[b]; t < n; ++t) {
      const int i = T.tnb_list[s0 + t];
      s2 += d_six_tf(T, J1, J2, D.jj[i], jb, ja) * d_ftelem_f(D, T, R, hR, b, i) * d_velem_f(D, L, hL, i, a, c, d, J2);
    }
    for (int t = 0, s0 = T.tnb_start[d], n = T.tnb_count[d]; t < n; ++t) {
      const int i = T.tnb_list[s0 + t];
      s3 += d_six_tf(T, J1, J2, jd, D.jj[i], jc) * d_ftelem_f(D, T, R, hR, i, d) * d_velem_f(D, L, hL, a, b, c, i, J1);
    }
    for (int t = 0, s0 = T.tnb_start[c], n = T.tnb_count[c]; t < n; ++t) {
      const int i = T.tnb_list[s0 + t];
      s4 -= d_six_tf(T, J1, J2, jc, D.jj[i], jd) * d_ftelem_f(D, T, R, hR, i, c) * d_velem_f(D, L, hL, a, b, d, i, J1);
    }
    auto sg = [](int n) { return (n & 1) ? -1.0f : 1.0f; };
    const float sm = s1 * sg((ja + jb - J2) >> 1) + s2 * sg((J1 + J2) >> 1) + s3 * sg((jc + jd - J1) >> 1) +
                     s4 * sg((J2 + J1) >> 1);
    // sqrt((J1+1)(J2+1)) / sqrt((1+d_ab)(1+d_cd)) (-1)^(rank/2), in FP32
    const float f = sqrtf((float)((J1 + 1) * (J2 + 1))) * ((a == b) ? 0.70710678f : 1.0f) *
                    ((c == d) ? 0.70710678f : 1.0f) * sg(rank >> 1);
    double* X = RES + T.goff[0] + e;
    *X += f32_to_f64(sm * f);
  }
}

}  // namespace imsrg
