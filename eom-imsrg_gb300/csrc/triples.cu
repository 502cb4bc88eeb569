// The perturbative triples correction after the Magnus flow on the device: restore_triples
// (src/IMSRG_MAGNUS.f90:767-902) with the three-body element commutator_223_single
// (src/commutators.f90:928-1325) over the three-body basis of enumerate_three_body
// (src/basic_IMSRG.f90:4215-4420).
//
//   E3 = sum over channels (Jtot, Tz, parity), ppp triples a <= b <= c, hhh triples i <= j <= k
//        and the pair couplings Jab, Jij of W^2 / D (Jtot + 1),
//   W  = <(ab)Jab c; Jtot| [Omega, H] |(ij)Jij k; Jtot>  (the three-body part of the commutator
//        of the two-body parts, nine J-coupled terms, each a sum over one orbit and up to two
//        intermediate couplings with 6j symbols),
//   D  = -(e_a + e_b + e_c - e_i - e_j - e_k + the 15 two-body monopoles) times the
//        multiplicity factors (6 for three equal orbits, 2 for two) of both triples.
//
// One thread per (channel, ppp, hhh) item (the kernel can split the orbit sums of the nine terms
// over a lane group, which measured slower) evaluates the denominator once and W for every
// allowed (Jab, Jij).  Every 6j symbol of the nine terms has three single-particle j, one
// three-body total (up to 3 jmax) and two pair couplings, so one table {j1 j2 x; J j3 y}, filled
// on the device by Racah's single-sum formula over a log-factorial table (165 MB at eMax=10),
// serves them all through the column symmetry of the 6j symbol.  Each block reduces its items and adds
// one partial into the result.  The reference's cuts are kept: the terms with a single
// two-body factor outside the J sums skip orbits where both factors are below 1e-8.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "engine.h"

using namespace imsrg;

namespace {

#define CKR(expr)                  \
  do {                             \
    imsrg_status _s = (expr);      \
    if (_s != IMSRG_OK) return _s; \
  } while (0)

constexpr int kLogFact = 256;

struct TriChan {
  int J, nppp, nhhh, ppp0, hhh0;
  int64_t item0;  // first item of the channel
};

struct DevTriples {
  const TriChan* chan;
  int nchan;
  int64_t nitems;
  const int16_t* ppp;  // 3 orbits per triple
  const int16_t* hhh;
  const double* lf;    // log(n!), n < kLogFact
  const double* mono;  // twobody_monopole(a, b) of H, N x N
  const double* fdiag; // f(a, a) of H
  // 6j {j1 j2 x; J j3 y}: j1, j2, j3 single-particle (h = (j-1)/2 < nh), J a three-body total
  // (hJ < nJ), x, y pair couplings (x/2, y/2 < nx)
  const double* six;
  int nh, nJ, nx;
};

__device__ __forceinline__ double dsgn(int n) { return (n & 1) ? -1.0 : 1.0; }
__device__ __forceinline__ bool dtri(int a, int b, int c) { return c <= a + b && c >= abs(a - b); }

// Wigner 6j {j1 j2 j3; j4 j5 j6} of doubled arguments, Racah's formula
__device__ double d_sixj(const double* __restrict__ lf, int j1, int j2, int j3, int j4, int j5, int j6) {
  auto ok = [](int a, int b, int c) { return dtri(a, b, c) && !((a + b + c) & 1); };
  if (!(ok(j1, j2, j3) && ok(j1, j5, j6) && ok(j4, j2, j6) && ok(j4, j5, j3))) return 0.0;
  auto ldelta = [&](int a, int b, int c) {
    return 0.5 * (lf[(a + b - c) / 2] + lf[(a - b + c) / 2] + lf[(-a + b + c) / 2] - lf[(a + b + c) / 2 + 1]);
  };
  const double ld = ldelta(j1, j2, j3) + ldelta(j1, j5, j6) + ldelta(j4, j2, j6) + ldelta(j4, j5, j3);
  const int a1 = (j1 + j2 + j3) / 2, a2 = (j1 + j5 + j6) / 2, a3 = (j4 + j2 + j6) / 2, a4 = (j4 + j5 + j3) / 2;
  const int b1 = (j1 + j2 + j4 + j5) / 2, b2 = (j2 + j3 + j5 + j6) / 2, b3 = (j3 + j1 + j6 + j4) / 2;
  const int zmin = max(max(a1, a2), max(a3, a4)), zmax = min(b1, min(b2, b3));
  double s = 0.0;
  for (int z = zmin; z <= zmax; ++z)
    s += dsgn(z) * exp(ld + lf[z + 1] - lf[z - a1] - lf[z - a2] - lf[z - a3] - lf[z - a4] - lf[b1 - z] - lf[b2 - z] -
                       lf[b3 - z]);
  return s;
}

__global__ void k_six_table(const double* __restrict__ lf, int nh, int nJ, int nx, double* __restrict__ out) {
  const int64_t n = (int64_t)nh * nh * nh * nJ * nx * nx;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t r = e;
    const int y = (int)(r % nx); r /= nx;
    const int x = (int)(r % nx); r /= nx;
    const int hJ = (int)(r % nJ); r /= nJ;
    const int h3 = (int)(r % nh); r /= nh;
    const int h2 = (int)(r % nh);
    const int h1 = (int)(r / nh);
    out[e] = d_sixj(lf, 2 * h1 + 1, 2 * h2 + 1, 2 * x, 2 * hJ + 1, 2 * h3 + 1, 2 * y);
  }
}

// commutator_223_single (src/commutators.f90:928-1325): <(pq)jpq r; J| [L, R] |(st)jst u; J>
__device__ double d_comm223(const DevLayout& D, const DevTriples& T, const double* __restrict__ L, int hL,
                            const double* __restrict__ R, int hR, int ip, int iq, int ir, int is, int it, int iu,
                            int J, int jpq, int jst, int lane, int nlanes) {
  // this lane's share: the orbits a = lane, lane + nlanes, ... of every term's sum
  const int jp = D.jj[ip], jq = D.jj[iq], jr = D.jj[ir], js = D.jj[is], jt = D.jj[it], ju = D.jj[iu];
  const int tp = D.tz[ip], tq = D.tz[iq], tr = D.tz[ir], ts = D.tz[is], tt = D.tz[it], tu = D.tz[iu];
  const int lp = D.ll[ip], lq = D.ll[iq], lr = D.ll[ir], ls = D.ll[is], lt = D.ll[it], lu = D.ll[iu];
  const int N = D.N;
  auto vL = [&](int a, int b, int c, int d, int Jx) { return d_v_elem(D, L, hL, a, b, c, d, Jx); };
  auto vR = [&](int a, int b, int c, int d, int Jx) { return d_v_elem(D, R, hR, a, b, c, d, Jx); };
  // 6j symbols from the table: {a b c; J e f} directly, {a b c; d J f} = {b a c; J d f}
  auto six4 = [&](int a, int b, int c, int Jx, int e, int f) {
    return T.six[(((((int64_t)(a >> 1) * T.nh + (b >> 1)) * T.nh + (e >> 1)) * T.nJ + (Jx >> 1)) * T.nx + (c >> 1)) *
                     T.nx + (f >> 1)];
  };
  auto six5 = [&](int a, int b, int c, int d, int Jx, int f) { return six4(b, a, c, Jx, d, f); };
  auto same = [&](int a, int tx, int lx, int t1, int t2, int l1, int l2) {
    return D.tz[a] + tx == t1 + t2 && ((D.ll[a] + lx) & 1) == ((l1 + l2) & 1);
  };
  double tot = 0.0;
  {  // 1
    double sm = 0.0;
    for (int a = lane; a < N; a += nlanes) {
      if (!same(a, tp, lp, ts, tt, ls, lt)) continue;
      const int ja = D.jj[a];
      if (!dtri(jp, ja, jst)) continue;
      const double V1 = vR(ip, a, is, it, jst), V2 = vL(ip, a, is, it, jst);
      if (fabs(V1) < 1e-8 && fabs(V2) < 1e-8) continue;
      const int lo = max(max(abs(jq - jr), abs(ja - ju)), abs(jp - J)), hi = min(min(jq + jr, ja + ju), jp + J);
      for (int J2 = lo; J2 <= hi; J2 += 2)
        sm += dsgn((ja - ju) / 2) * (J2 + 1.0) * six4(jq, jp, jpq, J, jr, J2) * six4(ja, jp, jst, J, ju, J2) *
              (V1 * vL(iq, ir, a, iu, J2) - V2 * vR(iq, ir, a, iu, J2));
    }
    tot += sm * dsgn((jq - jr) / 2);
  }
  {  // 2
    double sm = 0.0;
    for (int a = lane; a < N; a += nlanes) {
      if (!same(a, tp, lp, tu, tt, lu, lt)) continue;
      const int ja = D.jj[a];
      const int lo = max(max(abs(jp - ja), abs(jt - ju)), abs(js - J)), hi = min(min(jp + ja, jt + ju), js + J);
      const int lo2 = max(max(abs(jq - jr), abs(ja - js)), abs(jp - J)), hi2 = min(min(jq + jr, ja + js), jp + J);
      for (int J1 = lo; J1 <= hi; J1 += 2) {
        const double other = (J1 + 1.0) * dsgn(J1 / 2) * six4(jt, js, jst, J, ju, J1);
        if (other == 0.0) continue;
        const double r1 = vR(ip, a, it, iu, J1), l1 = vL(ip, a, it, iu, J1);
        double sub = 0.0;
        for (int J2 = lo2; J2 <= hi2; J2 += 2)
          sub += (J2 + 1.0) * six4(jq, jp, jpq, J, jr, J2) * six5(jp, ja, J1, js, J, J2) *
                 (r1 * vL(iq, ir, a, is, J2) - l1 * vR(iq, ir, a, is, J2));
        sm += sub * dsgn((ja + ju) / 2) * other;
      }
    }
    tot += sm * dsgn((jq + jr + js - jt) / 2);
  }
  {  // 3
    double sm = 0.0;
    for (int a = lane; a < N; a += nlanes) {
      if (!same(a, tp, lp, tu, ts, lu, ls)) continue;
      const int ja = D.jj[a];
      const int lo = max(max(abs(jp - ja), abs(js - ju)), abs(jt - J)), hi = min(min(jp + ja, js + ju), jt + J);
      const int lo2 = max(max(abs(jq - jr), abs(ja - jt)), abs(jp - J)), hi2 = min(min(jq + jr, ja + jt), jp + J);
      for (int J1 = lo; J1 <= hi; J1 += 2) {
        const double other = (J1 + 1.0) * six4(js, jt, jst, J, ju, J1);
        if (other == 0.0) continue;
        const double r1 = vR(ip, a, iu, is, J1), l1 = vL(ip, a, iu, is, J1);
        double sub = 0.0;
        for (int J2 = lo2; J2 <= hi2; J2 += 2)
          sub += (J2 + 1.0) * six4(jq, jp, jpq, J, jr, J2) * six5(jp, ja, J1, jt, J, J2) *
                 (r1 * vL(iq, ir, a, it, J2) - l1 * vR(iq, ir, a, it, J2));
        sm += sub * dsgn((ja + js) / 2) * other;
      }
    }
    tot += sm * dsgn((jq + jr + jst) / 2);
  }
  {  // 4
    double sm = 0.0;
    for (int a = lane; a < N; a += nlanes) {
      if (!same(a, tq, lq, tt, ts, lt, ls)) continue;
      const int ja = D.jj[a];
      if (!dtri(jq, ja, jst)) continue;
      const double V1 = vR(iq, a, is, it, jst), V2 = vL(iq, a, is, it, jst);
      if (fabs(V1) < 1e-8 && fabs(V2) < 1e-8) continue;
      const int lo = max(max(abs(jp - jr), abs(ja - ju)), abs(J - jq)), hi = min(min(jp + jr, ja + ju), J + jq);
      for (int J2 = lo; J2 <= hi; J2 += 2)
        sm += dsgn((ja + ju) / 2) * (J2 + 1.0) * dsgn(J2 / 2) * six4(jp, jq, jpq, J, jr, J2) *
              six4(ja, jq, jst, J, ju, J2) * (V1 * vL(ir, ip, a, iu, J2) - V2 * vR(ir, ip, a, iu, J2));
    }
    tot += sm * dsgn((jpq + jp + jq) / 2);
  }
  {  // 5
    double sm = 0.0;
    for (int a = lane; a < N; a += nlanes) {
      if (!same(a, tq, lq, tt, tu, lt, lu)) continue;
      const int ja = D.jj[a];
      const int lo = max(max(abs(jq - ja), abs(jt - ju)), abs(js - J)), hi = min(min(jq + ja, jt + ju), js + J);
      const int lo2 = max(max(abs(jp - jr), abs(ja - js)), abs(jq - J)), hi2 = min(min(jp + jr, ja + js), jq + J);
      for (int J1 = lo; J1 <= hi; J1 += 2) {
        const double other = (J1 + 1.0) * dsgn(J1 / 2) * six4(jt, js, jst, J, ju, J1);
        if (other == 0.0) continue;
        const double r1 = vR(iq, a, it, iu, J1), l1 = vL(iq, a, it, iu, J1);
        double sub = 0.0;
        for (int J2 = lo2; J2 <= hi2; J2 += 2)
          sub += dsgn(J2 / 2) * (J2 + 1.0) * six4(jp, jq, jpq, J, jr, J2) * six5(jq, ja, J1, js, J, J2) *
                 (r1 * vL(ir, ip, a, is, J2) - l1 * vR(ir, ip, a, is, J2));
        sm += sub * dsgn((ja + ju) / 2) * other;
      }
    }
    tot += sm * dsgn((jpq + js - jt + jp + jq) / 2);
  }
  {  // 6
    double sm = 0.0;
    for (int a = lane; a < N; a += nlanes) {
      if (!same(a, tq, lq, ts, tu, ls, lu)) continue;
      const int ja = D.jj[a];
      const int lo = max(max(abs(jq - ja), abs(js - ju)), abs(jt - J)), hi = min(min(jq + ja, js + ju), jt + J);
      const int lo2 = max(max(abs(jp - jr), abs(ja - jt)), abs(jq - J)), hi2 = min(min(jp + jr, ja + jt), jq + J);
      for (int J1 = lo; J1 <= hi; J1 += 2) {
        const double other = (J1 + 1.0) * six4(js, jt, jst, J, ju, J1);
        if (other == 0.0) continue;
        const double r1 = vR(iq, a, iu, is, J1), l1 = vL(iq, a, iu, is, J1);
        double sub = 0.0;
        for (int J2 = lo2; J2 <= hi2; J2 += 2)
          sub += dsgn(J2 / 2) * (J2 + 1.0) * six4(jp, jq, jpq, J, jr, J2) * six5(jq, ja, J1, jt, J, J2) *
                 (r1 * vL(ir, ip, a, it, J2) - l1 * vR(ir, ip, a, it, J2));
        sm += sub * dsgn((ja - js) / 2) * other;
      }
    }
    tot -= sm * dsgn((jpq + jst + jp + jq) / 2);
  }
  {  // 7
    double sm = 0.0;
    for (int a = lane; a < N; a += nlanes) {
      if (!same(a, tr, lr, ts, tt, ls, lt)) continue;
      const int ja = D.jj[a];
      if (!dtri(ju, ja, jpq) || !dtri(jr, ja, jst)) continue;
      sm += dsgn((ja - ju) / 2) * six5(jr, ja, jst, ju, J, jpq) *
            (vR(ir, a, is, it, jst) * vL(ip, iq, a, iu, jpq) - vL(ir, a, is, it, jst) * vR(ip, iq, a, iu, jpq));
    }
    tot += sm * dsgn(jpq / 2);
  }
  {  // 8
    double sm = 0.0;
    for (int a = lane; a < N; a += nlanes) {
      if (!same(a, tr, lr, tu, tt, lu, lt)) continue;
      const int ja = D.jj[a];
      if (!dtri(js, ja, jpq)) continue;
      const double V1 = vL(ip, iq, a, is, jpq), V2 = vR(ip, iq, a, is, jpq);
      if (fabs(V1) < 1e-8 && fabs(V2) < 1e-8) continue;
      const int lo = max(max(abs(ja - jr), abs(jt - ju)), abs(js - J)), hi = min(min(ja + jr, jt + ju), js + J);
      for (int J1 = lo; J1 <= hi; J1 += 2)
        sm += dsgn((ja + ju) / 2) * dsgn(J1 / 2) * (J1 + 1.0) * six4(jt, js, jst, J, ju, J1) *
              six5(jr, ja, J1, js, J, jpq) * (vR(ir, a, it, iu, J1) * V1 - vL(ir, a, it, iu, J1) * V2);
    }
    tot += sm * dsgn((jpq + js + jt) / 2);
  }
  {  // 9
    double sm = 0.0;
    for (int a = lane; a < N; a += nlanes) {
      if (!same(a, tr, lr, tu, ts, lu, ls)) continue;
      const int ja = D.jj[a];
      if (!dtri(ja, jt, jpq)) continue;
      const double V1 = vL(ip, iq, a, it, jpq), V2 = vR(ip, iq, a, it, jpq);
      if (fabs(V1) < 1e-8 && fabs(V2) < 1e-8) continue;
      const int lo = max(max(abs(ja - jr), abs(js - ju)), abs(jt - J)), hi = min(min(ja + jr, js + ju), jt + J);
      for (int J1 = lo; J1 <= hi; J1 += 2)
        sm += dsgn((ja - js) / 2) * (J1 + 1.0) * six4(js, jt, jst, J, ju, J1) * six5(jr, ja, J1, jt, J, jpq) *
              (vR(ir, a, iu, is, J1) * V1 - vL(ir, a, iu, is, J1) * V2);
    }
    tot += sm * dsgn((jst - jpq) / 2);
  }
  return tot * sqrt((jpq + 1.0) * (jst + 1.0));
}

__device__ __forceinline__ double repeat_factor(int a, int b, int c) {
  if (a == b) return a == c ? 6.0 : 2.0;
  return (a == c || b == c) ? 2.0 : 1.0;
}

// f(a, a) and the monopoles of H
__global__ void k_triples_prep(DevLayout D, const double* __restrict__ H, double* __restrict__ mono,
                               double* __restrict__ fdiag) {
  const int N = D.N;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N * N; e += gridDim.x * blockDim.x) {
    const int a = e / N, b = e - a * N;
    const int ja = D.jj[a], jb = D.jj[b];
    double s = 0.0;
    for (int JT = abs(ja - jb); JT <= ja + jb; JT += 2) s += (JT + 1.0) * d_v_elem(D, H, 1, a, b, a, b, JT);
    mono[e] = s / (ja + 1.0) / (jb + 1.0);
    if (b == 0) fdiag[a] = d_f_elem(D, H, 1, a, a);
  }
}

// kLanes lanes per (channel, ppp, hhh) item, splitting the orbit sums of the nine terms
template <int kLanes>
__global__ void __launch_bounds__(128) k_triples(DevLayout D, DevTriples T, const double* __restrict__ H,
                                                 const double* __restrict__ OM, double* __restrict__ out) {
  __shared__ double red[128];
  const int lane = threadIdx.x & (kLanes - 1);
  constexpr int kPerBlock = 128 / kLanes;
  // the lane groups of a warp run different items (different loop counts): each group
  // shuffles among its own lanes only
  const unsigned gmask = ((1u << kLanes) - 1u) << ((threadIdx.x & 31) & ~(kLanes - 1));
  double acc = 0.0;
  const int N = D.N;
  const int64_t ng = (int64_t)gridDim.x * kPerBlock;
  // the loop bounds are uniform over each lane group, so every shuffle sees the group's lanes
  for (int64_t x = blockIdx.x * (int64_t)kPerBlock + threadIdx.x / kLanes; x < T.nitems; x += ng) {
    int lo = 0, hi = T.nchan - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (T.chan[mid].item0 <= x) lo = mid;
      else hi = mid - 1;
    }
    const TriChan C = T.chan[lo];
    const int64_t f = x - C.item0;
    const int A = (int)(f / C.nhhh), I = (int)(f - (int64_t)A * C.nhhh);
    const int16_t* pa = T.ppp + 3 * (int64_t)(C.ppp0 + A);
    const int16_t* hi3 = T.hhh + 3 * (int64_t)(C.hhh0 + I);
    const int a = pa[0], b = pa[1], c = pa[2], i = hi3[0], j = hi3[1], k = hi3[2];
    const double* M = T.mono;
    const double den = -(T.fdiag[a] + T.fdiag[b] + T.fdiag[c] - T.fdiag[i] - T.fdiag[j] - T.fdiag[k] +
                         M[a * N + b] + M[a * N + c] + M[b * N + c] + M[i * N + j] + M[i * N + k] + M[j * N + k] -
                         M[i * N + a] - M[i * N + b] - M[i * N + c] - M[j * N + a] - M[j * N + b] - M[j * N + c] -
                         M[k * N + a] - M[k * N + b] - M[k * N + c]) *
                       repeat_factor(a, b, c) * repeat_factor(i, j, k);
    const int ja = D.jj[a], jb = D.jj[b], jc = D.jj[c], ji = D.jj[i], jj = D.jj[j], jk = D.jj[k];
    for (int jab = abs(ja - jb); jab <= ja + jb; jab += 2) {
      if (!dtri(C.J, jc, jab) || (a == b && ((jab >> 1) & 1))) continue;
      for (int jij = abs(ji - jj); jij <= ji + jj; jij += 2) {
        if (!dtri(C.J, jk, jij) || (i == j && ((jij >> 1) & 1))) continue;
        double w = d_comm223(D, T, OM, -1, H, 1, a, b, c, i, j, k, C.J, jab, jij, lane, kLanes);
        for (int o = kLanes / 2; o > 0; o >>= 1) w += __shfl_xor_sync(gmask, w, o, kLanes);
        if (lane == 0) acc += w * w / den * (C.J + 1.0);
      }
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 64; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(out, red[0]);
}

}  // namespace

// enumerate_three_body (src/basic_IMSRG.f90:4215-4420): channels Jtot (odd, up to 3 jmax), Tz,
// parity; hhh / ppp triples of non-decreasing index with matching Tz and parity for which some
// integer Jab (the reference steps by 1) closes |jc - Jtot| <= Jab <= jc + Jtot
imsrg_status Ctx::restore_triples(const double* H, const double* OM, double* e3, int64_t* items) {
  const int N = L.N;
  int jmax = 0;
  for (int a = 0; a < N; ++a) jmax = std::max(jmax, L.jj[a]);
  if ((3 * jmax + 6 * jmax) / 2 + 2 >= kLogFact) return fail(IMSRG_ERR_UNSUPPORTED, "restore_triples: j too large");
  std::vector<TriChan> chans;
  std::vector<int16_t> ppp, hhh;
  auto triples = [&](const std::vector<int>& orb, int Jtot, int Tz, int P, std::vector<int16_t>& dst) {
    int cnt = 0;
    const int n = (int)orb.size();
    for (int x = 0; x < n; ++x)
      for (int y = x; y < n; ++y)
        for (int z = y; z < n; ++z) {
          const int a = orb[x], b = orb[y], c = orb[z];
          if (L.tz[a] + L.tz[b] + L.tz[c] != Tz || (L.ll[a] + L.ll[b] + L.ll[c]) % 2 != P) continue;
          bool ok = false;
          for (int Jab = std::abs(L.jj[a] - L.jj[b]); Jab <= L.jj[a] + L.jj[b] && !ok; ++Jab)
            ok = Jab <= L.jj[c] + Jtot && Jab >= std::abs(L.jj[c] - Jtot);
          if (!ok) continue;
          dst.push_back((int16_t)a); dst.push_back((int16_t)b); dst.push_back((int16_t)c);
          ++cnt;
        }
    return cnt;
  };
  int64_t nit = 0;
  for (int Jtot = 1; Jtot <= 3 * jmax; Jtot += 2)
    for (int Tz = -3; Tz <= 3; Tz += 2)
      for (int P = 0; P <= 1; ++P) {
        TriChan c{};
        c.J = Jtot;
        c.ppp0 = (int)(ppp.size() / 3);
        c.hhh0 = (int)(hhh.size() / 3);
        c.nhhh = triples(L.holes, Jtot, Tz, P, hhh);
        c.nppp = triples(L.parts, Jtot, Tz, P, ppp);
        c.item0 = nit;
        if ((int64_t)c.nppp * c.nhhh == 0) continue;
        nit += (int64_t)c.nppp * c.nhhh;
        chans.push_back(c);
      }
  if (items) *items = nit;
  *e3 = 0.0;
  if (!nit) return IMSRG_OK;
  std::vector<double> lf(kLogFact, 0.0);
  for (int n = 2; n < kLogFact; ++n) lf[n] = lf[n - 1] + std::log((double)n);
  // one allocation for the tables and the scratch
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  const int nh = (jmax + 1) / 2, nJ = (3 * jmax + 1) / 2, nx = jmax + 1;
  const int64_t nsix = (int64_t)nh * nh * nh * nJ * nx * nx;
  const size_t bc = al(sizeof(TriChan) * chans.size()), bp = al(sizeof(int16_t) * ppp.size()),
               bh = al(sizeof(int16_t) * hhh.size()), bl = al(sizeof(double) * kLogFact),
               bm = al(sizeof(double) * (size_t)N * N), bf = al(sizeof(double) * N), bo = al(sizeof(double)),
               bs = al(sizeof(double) * (size_t)nsix);
  char* buf = nullptr;
  CKR(cuda(cudaMalloc(&buf, bc + bp + bh + bl + bm + bf + bo + bs), "cudaMalloc(triples)"));
  DevTriples T{};
  T.nh = nh; T.nJ = nJ; T.nx = nx;
  char* o = buf;
  T.chan = reinterpret_cast<const TriChan*>(o);
  imsrg_status st = cuda(cudaMemcpyAsync(o, chans.data(), sizeof(TriChan) * chans.size(), cudaMemcpyHostToDevice, stream),
                         "H2D triples");
  o += bc;
  T.ppp = reinterpret_cast<const int16_t*>(o);
  if (st == IMSRG_OK)
    st = cuda(cudaMemcpyAsync(o, ppp.data(), sizeof(int16_t) * ppp.size(), cudaMemcpyHostToDevice, stream), "H2D triples");
  o += bp;
  T.hhh = reinterpret_cast<const int16_t*>(o);
  if (st == IMSRG_OK)
    st = cuda(cudaMemcpyAsync(o, hhh.data(), sizeof(int16_t) * hhh.size(), cudaMemcpyHostToDevice, stream), "H2D triples");
  o += bh;
  T.lf = reinterpret_cast<const double*>(o);
  if (st == IMSRG_OK)
    st = cuda(cudaMemcpyAsync(o, lf.data(), sizeof(double) * kLogFact, cudaMemcpyHostToDevice, stream), "H2D triples");
  o += bl;
  double* mono = reinterpret_cast<double*>(o);
  T.mono = mono;
  o += bm;
  double* fd = reinterpret_cast<double*>(o);
  T.fdiag = fd;
  o += bf;
  double* d_out = reinterpret_cast<double*>(o);
  o += bo;
  double* six = reinterpret_cast<double*>(o);
  T.six = six;
  T.nchan = (int)chans.size();
  T.nitems = nit;
  if (st == IMSRG_OK) st = cuda(cudaMemsetAsync(d_out, 0, sizeof(double), stream), "memset(triples)");
  if (st == IMSRG_OK) {
    k_six_table<<<(int)std::max<int64_t>(1, std::min<int64_t>((nsix + 255) / 256, 152 * 32)), 256, 0, stream>>>(
        T.lf, nh, nJ, nx, six);
    st = launched("k_six_table");
  }
  if (st == IMSRG_OK) {
    k_triples_prep<<<(N * N + 255) / 256, 256, 0, stream>>>(D, H, mono, fd);
    st = launched("k_triples_prep");
  }
  if (st == IMSRG_OK) {
    constexpr int kLanes = 1;  // measured at eMax=8: 1 lane 1.07 s, 4 lanes 1.40 s, 32 lanes 1.50 s
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((nit + 128 / kLanes - 1) / (128 / kLanes), 152 * 16));
    k_triples<kLanes><<<grid, 128, 0, stream>>>(D, T, H, OM, d_out);
    st = launched("k_triples");
  }
  if (st == IMSRG_OK) st = cuda(cudaMemcpyAsync(e3, d_out, sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H triples");
  if (st == IMSRG_OK) st = cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
  cudaFree(buf);
  return st;
}

#define TRCTX(ptr)                                                                       \
  if (!(ptr)) return IMSRG_ERR_INVALID_ARGUMENT;                                         \
  Ctx* c = reinterpret_cast<Ctx*>(ptr);                                                  \
  if (c->device < 0) return c->fail(IMSRG_ERR_UNSUPPORTED, "host-only context (device < 0)"); \
  {                                                                                      \
    cudaError_t _e = cudaSetDevice(c->device);                                           \
    if (_e != cudaSuccess) return c->cuda(_e, "cudaSetDevice");                          \
  }

extern "C" imsrg_status imsrg_restore_triples(imsrg_ctx* ctx, const imsrg_op* H, const imsrg_op* OM, double* e3,
                                              int64_t* items) {
  TRCTX(ctx);
  if (!H || H->owner != c || !OM || OM->owner != c || !e3)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_restore_triples");
  if (H->herm != 1 || OM->herm != -1)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_restore_triples: H hermitian and Omega anti-hermitian");
  return c->restore_triples(H->d, OM->d, e3, items);
}
