// Reverse-mode (vector-Jacobian product) kernels of the FP64 commutator, the White
// generator and the slab inner product, for the adjoint dE0/dtheta of a Magnus flow.
//
// The reference has no derivative code.  Each kernel is the transpose of one forward
// kernel of kernels_fp64.cu / kernels_ops.cu: it walks the same index space (the same
// unique-element / one-body-output / CCX-element enumerations) and, where the forward
// gathers sum += X[x] * Y[y], it scatters Xbar[x] += g * Y[y] and Ybar[y] += g * X[x]
// with FP64 atomics.  The forward's write pattern is reversed exactly: an element written
// as X(i,j) (+)= s followed by the mirror X(j,i) = X(i,j) * herm passes the cotangent
// cb(i,j) + herm * cb(j,i) (herm * cb(i,i) on the diagonal) to s.
#include "dev.cuh"
#include "kernels.h"

namespace imsrg {

namespace {

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double vfac(const VRef& r, int herm) { return r.herm ? herm * r.pre : r.pre; }

__device__ __forceinline__ void d_vadd(const DevLayout& D, double* bar, int herm, int a, int b, int c, int d, int J,
                                       double g) {
  VRef r;
  if (d_vref(D, a, b, c, d, J, r)) atomicAdd(bar + r.idx, g * vfac(r, herm));
}

// slab position f_elem(a,b) reads, and whether the operator's herm multiplies it
struct FRef {
  int64_t idx;
  bool herm;
};
__device__ __forceinline__ FRef d_fref(const DevLayout& D, int a, int b) {
  const int c1 = D.con[a], c2 = D.con[b];
  if (c1 + c2 == 0) return {D.off_fpp + D.loc[a] + (int64_t)D.loc[b] * D.P, false};
  if (c1 + c2 == 2) return {D.off_fhh + D.loc[a] + (int64_t)D.loc[b] * D.A, false};
  if (c1 > c2) return {D.off_fph + D.loc[b] + (int64_t)D.loc[a] * D.P, true};
  return {D.off_fph + D.loc[a] + (int64_t)D.loc[b] * D.P, false};
}
__device__ __forceinline__ double fval(const double* op, const FRef& f, int herm) {
  return f.herm ? op[f.idx] * herm : op[f.idx];
}

// reverse of "X(ij) (+)= s; X(ji) = X(ij) * h": cotangent of s; the old X(ij) keeps it
// when accumulating, the overwritten entries lose theirs
__device__ __forceinline__ double d_fold(double* cb, int64_t ij, int64_t ji, bool diag, int h, bool accumulate) {
  const double g = diag ? h * cb[ij] : cb[ij] + h * cb[ji];
  cb[ij] = accumulate ? g : 0.0;
  if (!diag) cb[ji] = 0.0;
  return g;
}

__device__ __forceinline__ double* ob_at(const DevLayout& D, double* op, int kind, int p, int q) {
  if (kind == 0) return op + D.off_fhh + p + (int64_t)q * D.A;
  if (kind == 1) return op + D.off_fpp + p + (int64_t)q * D.P;
  return op + D.off_fph + p + (int64_t)q * D.P;
}

// lane 0 folds the one-body output of this warp, every lane gets the cotangent
__device__ __forceinline__ double ob_fold(const DevLayout& D, double* cb, int kind, int p, int q, int hRES, int lane) {
  double g = 0.0;
  if (lane == 0) {
    double* f = ob_at(D, cb, kind, p, q);
    if (kind < 2) {
      double* ft = ob_at(D, cb, kind, q, p);
      const bool diag = p == q;
      g = diag ? hRES * *f : *f + hRES * *ft;
      *f = g;
      if (!diag) *ft = 0.0;
    } else {
      g = *f;
    }
  }
  return __shfl_sync(0xffffffffu, g, 0);
}

__device__ __forceinline__ void decode_pairs(const DevLayout& D, int64_t u, int& q, int& g, int& IX, int& JX, int& a,
                                             int& b, int& c, int& d) {
  d_unique_decode(D, u, q, g, IX, JX);
  const int c1 = (g < 3) ? 0 : (g == 4 ? 2 : 1);
  const int c2 = (g == 0) ? 0 : ((g == 1 || g == 3) ? 1 : 2);
  const int o1 = D.pair_off[q * 3 + c1] + IX, o2 = D.pair_off[q * 3 + c2] + JX;
  a = D.pair_a[o1];
  b = D.pair_b[o1];
  c = D.pair_a[o2];
  d = D.pair_b[o2];
}

}  // namespace

// ---------------------------------------------------------------- 222_ph recoupling
// transpose of k_comm222ph: cotangent of RES (cb, folded in place) -> cotangent of WCC
__global__ void k_vjp_222ph(DevLayout D, double* __restrict__ cb, int hL, int hR, int hRES, double* __restrict__ Wb) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < D.n_unique; u += (int64_t)gridDim.x * blockDim.x) {
    int q, g, IX, JX, i, j, k, l;
    decode_pairs(D, u, q, g, IX, JX, i, j, k, l);
    const int kk = q * 6 + g;
    const int n1 = D.gn1[kk];
    const int64_t ij = D.goff[kk] + IX + (int64_t)JX * n1, ji = D.goff[kk] + JX + (int64_t)IX * n1;
    const bool sq = (g == 0 || g == 3 || g == 4);
    const double pre = (i == j) ? .70710678118 : 1.0;
    const double pre2 = (k == l) ? .70710678118 : 1.0;
    const double s = (sq ? d_fold(cb, ij, ji, IX == JX, hRES, true) : cb[ij]) * pre * pre2;
    if (s == 0.0) continue;
    const int jI = D.jj[i], jJ = D.jj[j], jK = D.jj[k], jL = D.jj[l];
    const int Jtot = D.lamJ[q];
    const int N = D.N, NJ = D.NJ;
    const double phase = d_sgn((jI + jJ + jK + jL) >> 1);
    {
      const int Tz = abs(D.tz[i] - D.tz[k]) >> 1;
      const int PAR = (D.ll[i] + D.ll[k]) & 1;
      const int jmin = max(abs(jJ - jL), abs(jI - jK)), jmax = min(jJ + jL, jI + jK);
      const double s0 = d_sgn((jL + jK + Jtot) >> 1);
      for (int JP = jmin; JP <= jmax; JP += 2) {
        const int qx = (JP >> 1) + Tz * (D.JM + 1) + PAR * 2 * (D.JM + 1);
        double* W = Wb + D.wcc_off[qx];
        const int64_t rl = D.cc_rlen[qx];
        const int h = JP >> 1;
        const int64_t rjl = D.ccr[(j * N + l) * NJ + h], rik = D.ccr[(i * N + k) * NJ + h];
        const int64_t gjl = D.ccr[(l * N + j) * NJ + h], gik = D.ccr[(k * N + i) * NJ + h];
        if ((rjl | rik | gjl | gik) < 0) continue;
        const double c = -s0 * d_sixj(D, jI, jJ, Jtot, jL, jK, JP) * s;
        atomicAdd(W + gik + rjl * rl, c * hL);
        atomicAdd(W + gjl + rik * rl, c * phase * hL);
        atomicAdd(W + rik + gjl * rl, -c * phase * hR);
        atomicAdd(W + rjl + gik * rl, -c * hR);
      }
    }
    {
      const int Tz = abs(D.tz[i] - D.tz[l]) >> 1;
      const int PAR = (D.ll[i] + D.ll[l]) & 1;
      const int jmin = max(abs(jI - jL), abs(jJ - jK)), jmax = min(jI + jL, jJ + jK);
      for (int JP = jmin; JP <= jmax; JP += 2) {
        const int qx = (JP >> 1) + Tz * (D.JM + 1) + PAR * 2 * (D.JM + 1);
        double* W = Wb + D.wcc_off[qx];
        const int64_t rl = D.cc_rlen[qx];
        const int h = JP >> 1;
        const int64_t ril = D.ccr[(i * N + l) * NJ + h], rjk = D.ccr[(j * N + k) * NJ + h];
        const int64_t gil = D.ccr[(l * N + i) * NJ + h], gjk = D.ccr[(k * N + j) * NJ + h];
        if ((ril | rjk | gil | gjk) < 0) continue;
        const double c = d_sixj(D, jI, jJ, Jtot, jK, jL, JP) * s;
        atomicAdd(W + gil + rjk * rl, c * hL);
        atomicAdd(W + gjk + ril * rl, c * phase * hL);
        atomicAdd(W + ril + gjk * rl, -c * phase * hR);
        atomicAdd(W + rjk + gil * rl, -c * hR);
      }
    }
  }
}

// ---------------------------------------------------------------- 221
// transpose of k_comm221: one warp per one-body output; cotangents of the w1 / w2 traces
__global__ void k_vjp_221(DevLayout D, int pm, double* __restrict__ cb, int hRES, double* __restrict__ w1b,
                          double* __restrict__ w2b) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= D.n_ob) return;
  const int kind = D.ob_kind[warp], p = D.ob_p[warp], q = D.ob_q[warp], ik = D.ob_pk[warp], jk = D.ob_qk[warp];
  const double g = ob_fold(D, cb, kind, p, q, hRES, lane);
  if (g == 0.0) return;
  const int ji = D.jj[ik];
  const double tb = g / (ji + 1.0);
  for (int ck = lane; ck < D.N; ck += 32) {
    double* w = D.con[ck] ? w1b : w2b;
    const int jc = D.jj[ck];
    for (int JT = abs(jc - ji); JT <= jc + ji; JT += 2) {
      d_vadd(D, w, 1, ck, ik, ck, jk, JT, tb * (JT + 1));
      if (kind < 2) d_vadd(D, w, 1, ck, jk, ck, ik, JT, -pm * tb * (JT + 1));
    }
  }
}

// ---------------------------------------------------------------- 222_pp_hh accumulation
// transpose of k_pphh_update: w1b += cb - pm cb^T (squares) or cb, w2b -= the same
__global__ void k_vjp_pphh_wbar(DevLayout D, const double* __restrict__ cb, double* __restrict__ w1b,
                                double* __restrict__ w2b, double pm) {
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
    double v = cb[e];
    if (g == 0 || g == 3 || g == 4) {
      const int n = D.gn1[lo];
      const int64_t loc = e - D.goff[lo];
      const int j = (int)(loc / n), i = (int)(loc - (int64_t)j * n);
      v = cb[e] - pm * cb[D.goff[lo] + j + (int64_t)i * n];
    }
    w1b[e] += v;
    w2b[e] -= v;
  }
}

// ---------------------------------------------------------------- 122
// transpose of k_comm122 (which assigns every 2b element)
__global__ void k_vjp_122(DevLayout D, const double* __restrict__ L, int hL, const double* __restrict__ R, int hR,
                          double* __restrict__ cb, int hRES, double* __restrict__ Lb, double* __restrict__ Rb) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < D.n_unique; u += (int64_t)gridDim.x * blockDim.x) {
    int q, g, IX, JX, a, b, c, d;
    decode_pairs(D, u, q, g, IX, JX, a, b, c, d);
    const int kk = q * 6 + g;
    const int n1 = D.gn1[kk];
    const int64_t ij = D.goff[kk] + IX + (int64_t)JX * n1, ji = D.goff[kk] + JX + (int64_t)IX * n1;
    double s;
    if (g == 0 || g == 3 || g == 4) {
      s = d_fold(cb, ij, ji, IX == JX, hRES, false);
    } else {
      s = cb[ij];
      cb[ij] = 0.0;
    }
    s = s / sqrt(1.0 + (a == b ? 1.0 : 0.0)) / sqrt(1.0 + (c == d ? 1.0 : 0.0));
    if (s == 0.0) continue;
    const int JT = D.lamJ[q];
    // term sign * (f(L; x, y) v(R; ...) - f(R; x, y) v(L; ...))
    auto term = [&](int fx, int fy, int va, int vb, int vc, int vd, double sign) {
      VRef r;
      if (!d_vref(D, va, vb, vc, vd, JT, r)) return;
      const FRef f = d_fref(D, fx, fy);
      const double vR = R[r.idx] * vfac(r, hR), vL = L[r.idx] * vfac(r, hL);
      const double fL = fval(L, f, hL), fR = fval(R, f, hR);
      const double ss = sign * s;
      atomicAdd(Lb + f.idx, ss * vR * (f.herm ? hL : 1));
      atomicAdd(Rb + r.idx, ss * fL * vfac(r, hR));
      atomicAdd(Rb + f.idx, -ss * vL * (f.herm ? hR : 1));
      atomicAdd(Lb + r.idx, -ss * fR * vfac(r, hL));
    };
    for (int t = 0, s0 = D.same_start[a], n = D.same_count[a]; t < n; ++t) {
      const int i = D.same_list[s0 + t];
      term(a, i, i, b, c, d, 1.0);
    }
    for (int t = 0, s0 = D.same_start[b], n = D.same_count[b]; t < n; ++t) {
      const int i = D.same_list[s0 + t];
      term(b, i, a, i, c, d, 1.0);
    }
    for (int t = 0, s0 = D.same_start[c], n = D.same_count[c]; t < n; ++t) {
      const int i = D.same_list[s0 + t];
      term(i, c, a, b, i, d, -1.0);
    }
    for (int t = 0, s0 = D.same_start[d], n = D.same_count[d]; t < n; ++t) {
      const int i = D.same_list[s0 + t];
      term(i, d, a, b, c, i, -1.0);
    }
  }
}

// ---------------------------------------------------------------- 121
// transpose of k_comm121: one warp per one-body output
__global__ void k_vjp_121(DevLayout D, const double* __restrict__ L, int hL, const double* __restrict__ R, int hR,
                          double* __restrict__ cb, int hRES, double* __restrict__ Lb, double* __restrict__ Rb) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= D.n_ob) return;
  const int kind = D.ob_kind[warp], p = D.ob_p[warp], q = D.ob_q[warp], pk = D.ob_pk[warp], qk = D.ob_qk[warp];
  const double g = ob_fold(D, cb, kind, p, q, hRES, lane);
  if (g == 0.0) return;
  const double sb = g / (D.jj[pk] + 1.0);
  const int jq = D.jj[qk];
  for (int t = lane; t < D.n_ai; t += 32) {
    const int a = D.ai_a[t], i = D.ai_i[t];
    const int ak = D.parts[a], ik = D.holes[i];
    const int ji = D.jj[ik];
    const int64_t ph = D.off_fph + a + (int64_t)i * D.P;
    const double lph = L[ph], rph = R[ph];
    double smx = 0, smy = 0, smx2 = 0, smy2 = 0;
    VRef r;
    for (int JT = abs(ji - jq); JT <= ji + jq; JT += 2) {
      if (d_vref(D, ak, pk, ik, qk, JT, r)) {
        smx += R[r.idx] * vfac(r, hR) * (JT + 1);
        smx2 += L[r.idx] * vfac(r, hL) * (JT + 1);
        atomicAdd(Rb + r.idx, sb * lph * hL * (JT + 1) * vfac(r, hR));
        atomicAdd(Lb + r.idx, -sb * rph * hR * (JT + 1) * vfac(r, hL));
      }
      if (d_vref(D, ik, pk, ak, qk, JT, r)) {
        smy += R[r.idx] * vfac(r, hR) * (JT + 1);
        smy2 += L[r.idx] * vfac(r, hL) * (JT + 1);
        atomicAdd(Rb + r.idx, -sb * lph * (JT + 1) * vfac(r, hR));
        atomicAdd(Lb + r.idx, sb * rph * (JT + 1) * vfac(r, hL));
      }
    }
    atomicAdd(Lb + ph, sb * (hL * smx - smy));
    atomicAdd(Rb + ph, -sb * (hR * smx2 - smy2));
  }
}

// ---------------------------------------------------------------- 111
// transpose of k_comm111 (which assigns the one-body part): one warp per one-body element
// of Lb (first half of the index space) or Rb (second half), accumulated
__global__ void k_vjp_111(DevLayout D, const double* __restrict__ L, int hL, const double* __restrict__ R, int hR,
                          const double* __restrict__ cb, double* __restrict__ Lb, double* __restrict__ Rb) {
  const int A = D.A, P = D.P;
  const int n1 = A * A + P * A + P * P;
  const int lane = threadIdx.x & 31;
  const double *Lhh = L + D.off_fhh, *Rhh = R + D.off_fhh, *Lph = L + D.off_fph, *Rph = R + D.off_fph;
  const double *Lpp = L + D.off_fpp, *Rpp = R + D.off_fpp;
  const double *Chh = cb + D.off_fhh, *Cph = cb + D.off_fph, *Cpp = cb + D.off_fpp;
  const double hh = (double)hL * hR;
  auto t1 = [&](int i, int k) { return Chh[i + k * A] - hh * Chh[k + i * A]; };
  auto t2 = [&](int i, int k) { return hL * Chh[i + k * A] - hR * Chh[k + i * A]; };
  auto u1 = [&](int p, int m) { return hR * Cpp[p + (int64_t)m * P] - hL * Cpp[m + (int64_t)p * P]; };
  auto u2 = [&](int p, int m) { return Cpp[p + (int64_t)m * P] - hh * Cpp[m + (int64_t)p * P]; };
  for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < 2 * n1; w += (gridDim.x * blockDim.x) >> 5) {
    const bool isR = w >= n1;
    const int t = isR ? w - n1 : w;
    double acc = 0.0;
    if (t < A * A) {
      const int i = t % A, j = t / A;
      if (!isR) {  // Lhhb = t1 Rhh^T - Rph^T Cph
        for (int k = lane; k < A; k += 32) acc += t1(i, k) * Rhh[j + k * A];
        for (int p = lane; p < P; p += 32) acc -= Rph[p + i * P] * Cph[p + j * P];
      } else {     // Rhhb = Lhh^T t1 + Lph^T Cph
        for (int k = lane; k < A; k += 32) acc += Lhh[k + i * A] * t1(k, j);
        for (int p = lane; p < P; p += 32) acc += Lph[p + i * P] * Cph[p + j * P];
      }
      acc = warp_sum(acc);
      if (lane == 0) (isR ? Rb : Lb)[D.off_fhh + t] += acc;
    } else if (t < A * A + P * A) {
      const int s = t - A * A;
      const int p = s % P, i = s / P;
      if (!isR) {  // Lphb = Rph t2^T + Cph Rhh^T - Rpp^T Cph + u1 Rph
        for (int k = lane; k < A; k += 32) acc += Rph[p + k * P] * t2(i, k) + Cph[p + k * P] * Rhh[i + k * A];
        for (int m = lane; m < P; m += 32) acc += -Rpp[m + (int64_t)p * P] * Cph[m + i * P] + u1(p, m) * Rph[m + i * P];
      } else {     // Rphb = Lph t2 + Lpp^T Cph - Cph Lhh^T + u1^T Lph
        for (int k = lane; k < A; k += 32) acc += Lph[p + k * P] * t2(k, i) - Cph[p + k * P] * Lhh[i + k * A];
        for (int m = lane; m < P; m += 32) acc += Lpp[m + (int64_t)p * P] * Cph[m + i * P] + u1(m, p) * Lph[m + i * P];
      }
      acc = warp_sum(acc);
      if (lane == 0) (isR ? Rb : Lb)[D.off_fph + s] += acc;
    } else {
      const int s = t - A * A - P * A;
      const int p = s % P, r = s / P;
      if (!isR) {  // Lppb = Cph Rph^T + u2 Rpp^T
        for (int k = lane; k < A; k += 32) acc += Cph[p + k * P] * Rph[r + k * P];
        for (int m = lane; m < P; m += 32) acc += u2(p, m) * Rpp[r + (int64_t)m * P];
      } else {     // Rppb = -Cph Lph^T + Lpp^T u2
        for (int k = lane; k < A; k += 32) acc -= Cph[p + k * P] * Lph[r + k * P];
        for (int m = lane; m < P; m += 32) acc += Lpp[m + (int64_t)p * P] * u2(m, r);
      }
      acc = warp_sum(acc);
      if (lane == 0) (isR ? Rb : Lb)[D.off_fpp + s] += acc;
    }
  }
}

// ---------------------------------------------------------------- E0 = 110 + 220
// blockIdx.y < nblocks: the pphh block of channel y (220, when hL hR = -1); y = nblocks: fph (110)
__global__ void k_vjp_e0(DevLayout D, const double* __restrict__ L, int hL, const double* __restrict__ R, int hR,
                         const double* __restrict__ cb, double* __restrict__ Lb, double* __restrict__ Rb) {
  const double eb = cb[0];
  if (eb == 0.0) return;
  const int q = blockIdx.y;
  if (q == D.nblocks) {
    const int A = D.A, P = D.P;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < A * P; t += gridDim.x * blockDim.x) {
      const int i = t / P;
      const double w = eb * (hL - hR) * (D.jj[D.holes[i]] + 1);
      const int64_t k = D.off_fph + t;
      Lb[k] += w * R[k];
      Rb[k] += w * L[k];
    }
    return;
  }
  if (hR * hL != -1) return;
  const int64_t n = (int64_t)D.ncls[q * 3] * D.ncls[q * 3 + 2];
  const int64_t o = D.goff[q * 6 + 2];
  const double w = -2.0 * hR * (D.lamJ[q] + 1) * eb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    Lb[o + t] += w * R[o + t];
    Rb[o + t] += w * L[o + t];
  }
}

// ---------------------------------------------------------------- Pandya transform
// transpose of k_pandya: CCX cotangent -> operator cotangent
__global__ void k_pandya_vjp(DevLayout D, int herm, const double* __restrict__ ccb, double* __restrict__ opb) {
  const int64_t total = D.cc_size;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const double cv = ccb[e];
    if (cv == 0.0) continue;
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
    if (!(((D.ll[a] + D.ll[h]) & 1) == ((D.ll[b] + D.ll[p]) & 1) && D.tz[a] + D.tz[h] == D.tz[b] + D.tz[p])) continue;
    const int jp = D.jj[p], jh = D.jj[h], ja = D.jj[a], jb = D.jj[b];
    const double g = cv * d_sgn((jh + jb + JC) >> 1) * sqrt(JC + 1.0);
    const int Jmin = max(abs(jp - jb), abs(ja - jh)), Jmax = min(jp + jb, ja + jh);
    for (int JT = Jmin; JT <= Jmax; JT += 2)
      d_vadd(D, opb, herm, h, a, p, b, JT, g * d_sgn(JT >> 1) * (JT + 1) * d_sixj(D, jp, jh, JC, ja, jb, JT));
  }
}

// ---------------------------------------------------------------- White generator
// transpose of k_white_1b (numerator and denominator of eta_ai)
__global__ void k_white_vjp_1b(DevLayout D, const double* __restrict__ H, int hH, const double* __restrict__ ETAb,
                               double* __restrict__ Hb) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= D.n_ai) return;
  const int a = D.ai_a[w], i = D.ai_i[w];
  const int64_t ph = D.off_fph + a + (int64_t)i * D.P;
  const double eb = ETAb[ph];
  if (eb == 0.0) return;
  const int ak = D.parts[a], ik = D.holes[i];
  const int ji = D.jj[ik];
  double Eden = 0.0;
  for (int JT = 0; JT <= 2 * ji; JT += 2) Eden = Eden - (JT + 1) * d_v_elem(D, H, hH, ak, ik, ak, ik, JT);
  Eden = Eden / (ji + 1.0) / (ji + 1.0);
  Eden = Eden + H[D.off_fpp + a + (int64_t)a * D.P] - H[D.off_fhh + i + (int64_t)i * D.A];
  atomicAdd(Hb + ph, eb / Eden);
  const double db = -eb * H[ph] / (Eden * Eden);
  atomicAdd(Hb + D.off_fpp + a + (int64_t)a * D.P, db);
  atomicAdd(Hb + D.off_fhh + i + (int64_t)i * D.A, -db);
  for (int JT = 0; JT <= 2 * ji; JT += 2)
    d_vadd(D, Hb, hH, ak, ik, ak, ik, JT, -db * (JT + 1) / (ji + 1.0) / (ji + 1.0));
}

// transpose of k_white_2b: numerator into Hb, denominator into the one-body diagonal of Hb
// and into monob (cotangents of the monopoles, expanded by k_monopole_vjp)
__global__ void k_white_vjp_2b(DevLayout D, const double* __restrict__ H, int hH, const double* __restrict__ mono,
                               const double* __restrict__ ETAb, double* __restrict__ Hb, double* __restrict__ monob) {
  const int q = blockIdx.y;
  const int np = D.ncls[q * 3], nh = D.ncls[q * 3 + 2];
  const int64_t n = (int64_t)np * nh;
  const int64_t off = D.goff[q * 6 + 2];
  const int N = D.N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const double eb = ETAb[off + t];
    if (eb == 0.0) continue;
    const int JX = (int)(t / np), IX = (int)(t - (int64_t)JX * np);
    const int o1 = D.pair_off[q * 3] + IX, o2 = D.pair_off[q * 3 + 2] + JX;
    const int a = D.pair_a[o1], b = D.pair_b[o1], i = D.pair_a[o2], j = D.pair_b[o2];
    double Eden = 0.0;
    Eden = Eden + mono[a * N + b];
    Eden = Eden + mono[i * N + j];
    Eden = Eden - mono[a * N + i];
    Eden = Eden - mono[a * N + j];
    Eden = Eden - mono[i * N + b];
    Eden = Eden - mono[j * N + b];
    Eden = Eden + d_f_elem(D, H, hH, a, a) + d_f_elem(D, H, hH, b, b) - d_f_elem(D, H, hH, i, i) -
           d_f_elem(D, H, hH, j, j);
    atomicAdd(Hb + off + t, eb / Eden);
    const double db = -eb * H[off + t] / (Eden * Eden);
    atomicAdd(monob + a * N + b, db);
    atomicAdd(monob + i * N + j, db);
    atomicAdd(monob + a * N + i, -db);
    atomicAdd(monob + a * N + j, -db);
    atomicAdd(monob + i * N + b, -db);
    atomicAdd(monob + j * N + b, -db);
    const int xs[4] = {a, b, i, j};
    for (int m = 0; m < 4; ++m) {
      const FRef f = d_fref(D, xs[m], xs[m]);
      atomicAdd(Hb + f.idx, (m < 2 ? db : -db) * (f.herm ? hH : 1));
    }
  }
}

// transpose of k_monopole
__global__ void k_monopole_vjp(DevLayout D, int hH, const double* __restrict__ monob, double* __restrict__ Hb) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= D.N * D.N) return;
  const double g = monob[t];
  if (g == 0.0) return;
  const int a = t / D.N, b = t % D.N;
  const int ja = D.jj[a], jb = D.jj[b];
  for (int JT = abs(ja - jb); JT <= ja + jb; JT += 2)
    d_vadd(D, Hb, hH, a, b, a, b, JT, g * (JT + 1) / (ja + 1.0) / (jb + 1.0));
}

// ---------------------------------------------------------------- slab inner product
__global__ void k_dot_partial(const double* __restrict__ x, const double* __restrict__ y, int64_t n,
                              double* __restrict__ partial) {
  __shared__ double red[256];
  double acc = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    acc += x[e] * y[e];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

}  // namespace imsrg
