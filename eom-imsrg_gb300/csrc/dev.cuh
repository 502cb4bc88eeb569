// Device view of a Layout (layout.h): raw pointers into one HBM-resident table
// allocation plus scalar sizes, passed by value to every kernel.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace imsrg {

struct DevLayout {
  int N, A, P, JM, NJ, nblocks, ncc, n_ob, sj_nh;
  int64_t off_fhh, off_fpp, off_fph, slab, n_unique, cc_size, wcc_size;
  // per orbit
  const int* jj;
  const int* ll;
  const int* tz;
  const int* con;
  const int* loc;
  const int* holes;
  const int* parts;
  const int* same_start;
  const int* same_count;
  const int* same_list;
  // sq_op channels
  const int* lamJ;
  const int* ncls;      // [q*3+c]
  const int* pair_off;  // [q*3+c]
  const int16_t* pair_a;
  const int16_t* pair_b;
  const int* pairpos;   // [(a*N+b)*NJ+J/2]
  const int64_t* goff;  // [q*6+g]
  const int* gn1;
  const int* gn2;
  const int64_t* uoff;  // [q*6+g], nblocks*6+1 entries
  // cross-coupled
  const int* cc_rlen;
  const int* cc_nph;
  const int* cc_J;
  const int64_t* cc_off;   // ncc+1
  const int64_t* wcc_off;  // ncc+1
  const int* cc_row_off;
  const int* cc_col_off;
  const int16_t* cc_ra;
  const int16_t* cc_rb;
  const int16_t* cc_cp;
  const int16_t* cc_ch;
  const int* ccr;       // [(a*N+b)*NJ+JC/2]
  const int* ccr_t;     // same table, [(a*NJ+JC/2)*N+b]: consecutive b adjacent
  const int* pairpos_t; // pairpos as [(a*NJ+J/2)*N+b]
  // one-body output list
  const int* ob_kind;
  const int* ob_p;
  const int* ob_q;
  const int* ob_pk;
  const int* ob_qk;
  int n_ai;
  const int* ai_a;
  const int* ai_i;
  // 6j
  const int* sj_off;
  const int* sj_j3min;
  const int* sj_j6min;
  const int* sj_n6;
  const double* sj_val;
  const float* sj_valf;
};

#if defined(__CUDACC__)
__device__ __forceinline__ bool d_tri(int a, int b, int J) { return J <= a + b && J >= abs(a - b); }
__device__ __forceinline__ double d_sgn(int n) { return (n & 1) ? -1.0 : 1.0; }

// 6j symbol {j1 j2 j3; j4 j5 j6} (j1,j2,j4,j5 odd, j3,j6 even; doubled units)
__device__ __forceinline__ double d_sixj(const DevLayout& D, int j1, int j2, int j3, int j4, int j5, int j6) {
  if (!(d_tri(j1, j2, j3) && d_tri(j4, j5, j3) && d_tri(j1, j5, j6) && d_tri(j4, j2, j6))) return 0.0;
  const int nh = D.sj_nh;
  const int k = (((j1 >> 1) * nh + (j2 >> 1)) * nh + (j4 >> 1)) * nh + (j5 >> 1);
  return __ldg(D.sj_val + D.sj_off[k] + ((j3 - D.sj_j3min[k]) >> 1) * D.sj_n6[k] + ((j6 - D.sj_j6min[k]) >> 1));
}

// f_elem (src/basic_IMSRG.f90:1191-1221)
__device__ __forceinline__ double d_f_elem(const DevLayout& D, const double* op, int herm, int a, int b) {
  const int c1 = D.con[a], c2 = D.con[b];
  if (c1 + c2 == 0) return op[D.off_fpp + D.loc[a] + (int64_t)D.loc[b] * D.P];
  if (c1 + c2 == 2) return op[D.off_fhh + D.loc[a] + (int64_t)D.loc[b] * D.A];
  if (c1 > c2) return op[D.off_fph + D.loc[b] + (int64_t)D.loc[a] * D.P] * herm;
  return op[D.off_fph + D.loc[a] + (int64_t)D.loc[b] * D.P];
}

// Position of the element v_elem(a,b,c,d,J) would read (src/basic_IMSRG.f90:1314-1429):
// returns false when the element vanishes by symmetry, otherwise the slab index, the
// prefactor (swap phases, sqrt(2) for identical orbits) and whether herm applies.
struct VRef {
  int64_t idx;
  double pre;
  bool herm;
};
__device__ __forceinline__ bool d_vref(const DevLayout& D, int a, int b, int c, int d, int J, VRef& r) {
  const int ja = D.jj[a], jb = D.jj[b], jc = D.jj[c], jd = D.jj[d];
  if (!(d_tri(ja, jb, J) && d_tri(jc, jd, J))) return false;
  const int P = (D.ll[a] + D.ll[b]) & 1;
  if (((D.ll[c] + D.ll[d]) & 1) != P) return false;
  const int tab = D.tz[a] + D.tz[b];
  if (D.tz[c] + D.tz[d] != tab) return false;
  const int q = 3 * J + (tab + 2) + P;  // block_index with 2*(Tz+1) = tab+2
  const int C1 = D.con[a] + D.con[b], C2 = D.con[c] + D.con[d];
  // (C1,C2) -> g : pp,pp 0 | pp,ph 1 | pp,hh 2 | ph,ph 3 | hh,hh 4 | ph,hh 5
  const int lo = C1 < C2 ? C1 : C2, hi = C1 < C2 ? C2 : C1;
  const int g = (lo == 0) ? hi : (lo == 1 ? (hi == 1 ? 3 : 5) : 4);
  const int NJ = D.NJ, N = D.N;
  double pre = 1.0;
  int i1, i2;
  if (a > b) {
    i1 = D.pairpos[(b * N + a) * NJ + (J >> 1)];
    pre = d_sgn(1 + ((ja + jb - J) >> 1));
  } else {
    if (a == b) pre = 1.4142135623730951;
    i1 = D.pairpos[(a * N + b) * NJ + (J >> 1)];
  }
  if (c > d) {
    i2 = D.pairpos[(d * N + c) * NJ + (J >> 1)];
    pre *= d_sgn(1 + ((jc + jd - J) >> 1));
  } else {
    if (c == d) pre *= 1.4142135623730951;
    i2 = D.pairpos[(c * N + d) * NJ + (J >> 1)];
  }
  const int k = q * 6 + g;
  const int n1 = D.gn1[k];
  if (C1 > C2) {
    r.idx = D.goff[k] + i2 + (int64_t)i1 * n1;
    r.herm = true;
  } else {
    r.idx = D.goff[k] + i1 + (int64_t)i2 * n1;
    r.herm = false;
  }
  r.pre = pre;
  return true;
}

// FP32 flavour of d_vref: the same element position with a float prefactor, so the
// FP32 kernels issue no FP64 instruction (GB300 runs FP64 at ~1/64 of the FP32 rate).
struct VRefF {
  int64_t idx;
  float pre;  // swap phases and sqrt(2) factors
  bool tr;    // element read from the transposed storage: multiply by the operator's herm
  __device__ __forceinline__ float scale(int herm) const { return (tr && herm < 0) ? -pre : pre; }
};
__device__ __forceinline__ bool d_vref_f(const DevLayout& D, int a, int b, int c, int d, int J, VRefF& r) {
  const int ja = D.jj[a], jb = D.jj[b], jc = D.jj[c], jd = D.jj[d];
  if (!(d_tri(ja, jb, J) && d_tri(jc, jd, J))) return false;
  const int P = (D.ll[a] + D.ll[b]) & 1;
  if (((D.ll[c] + D.ll[d]) & 1) != P) return false;
  const int tab = D.tz[a] + D.tz[b];
  if (D.tz[c] + D.tz[d] != tab) return false;
  const int q = 3 * J + (tab + 2) + P;
  const int C1 = D.con[a] + D.con[b], C2 = D.con[c] + D.con[d];
  const int lo = C1 < C2 ? C1 : C2, hi = C1 < C2 ? C2 : C1;
  const int g = (lo == 0) ? hi : (lo == 1 ? (hi == 1 ? 3 : 5) : 4);
  const int NJ = D.NJ, N = D.N;
  int neg = 0, nsq = 0;
  int i1, i2;
  if (a > b) {
    i1 = D.pairpos[(b * N + a) * NJ + (J >> 1)];
    neg ^= (1 + ((ja + jb - J) >> 1)) & 1;
  } else {
    nsq += (a == b);
    i1 = D.pairpos[(a * N + b) * NJ + (J >> 1)];
  }
  if (c > d) {
    i2 = D.pairpos[(d * N + c) * NJ + (J >> 1)];
    neg ^= (1 + ((jc + jd - J) >> 1)) & 1;
  } else {
    nsq += (c == d);
    i2 = D.pairpos[(c * N + d) * NJ + (J >> 1)];
  }
  const int k = q * 6 + g;
  const int n1 = D.gn1[k];
  if (C1 > C2) {
    r.idx = D.goff[k] + i2 + (int64_t)i1 * n1;
    r.tr = true;
  } else {
    r.idx = D.goff[k] + i1 + (int64_t)i2 * n1;
    r.tr = false;
  }
  const float m = nsq == 0 ? 1.0f : (nsq == 1 ? 1.41421356f : 2.0f);
  r.pre = neg ? -m : m;
  return true;
}

// FP64 -> FP32 with integer instructions only (GB300's FP64 pipe, which the hardware
// conversion would use, runs at ~1/64 of the FP32 rate).  Rounds to nearest, ties to
// even, as IEEE 754 binary64 -> binary32 conversion does:
//   - NaN stays NaN (quiet, with the top payload bits), +-Inf stays +-Inf;
//   - magnitudes that round above FLT_MAX become +-Inf (the rounding carry runs from the
//     mantissa into the exponent, and exponent field 255 with a zero mantissa is Inf);
//   - magnitudes below FP32's normal range round to FP32 subnormals k * 2^-149, or +-0.
__device__ __forceinline__ float f64_to_f32_any(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned int sign = (unsigned int)(b >> 63) << 31;
  const int e = (int)((b >> 52) & 0x7FF);
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  if (e == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (m ? 0x400000u | (unsigned int)(m >> 29) : 0u));
  if (e >= 1023 - 126) {  // FP32 normal range (or overflow): keep 23 mantissa bits, round off 29
    if (e > 1023 + 127) return __uint_as_float(sign | 0x7F800000u);
    unsigned int v = ((unsigned int)(e - 1023 + 127) << 23) | (unsigned int)(m >> 29);
    const unsigned int rest = (unsigned int)(m & 0x1FFFFFFFu);
    v += (rest > 0x10000000u || (rest == 0x10000000u && (v & 1u))) ? 1u : 0u;
    return __uint_as_float(sign | v);
  }
  // |x| = sig * 2^(e-1075) with sig = 2^52 + m; in units of 2^-149 that is sig >> (926 - e).
  // A shift of 54 or more leaves less than half a unit (sig < 2^53): the result is +-0.
  const int shift = 926 - e;
  if (shift >= 54) return __uint_as_float(sign);
  const unsigned long long sig = m | (1ull << 52);
  unsigned int k = (unsigned int)(sig >> shift);
  const unsigned long long rest = sig & ((1ull << shift) - 1ull), half = 1ull << (shift - 1);
  k += (rest > half || (rest == half && (k & 1u))) ? 1u : 0u;  // k = 2^23 encodes the smallest normal
  return __uint_as_float(sign | k);
}

// The same on FP32's normal range, inline: the FP64 exponent 897..1150 is rebiased, the top
// 23 mantissa bits kept and the 29 below rounded off (round up above half, and at exactly
// half when the kept value is odd: (rest + 2^28 - 1 + odd) >> 29).  Everything else (zeros,
// subnormals, overflow, Inf, NaN) takes f64_to_f32_any.
__device__ __forceinline__ float f64_to_f32(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned ah = hi & 0x7FFFFFFFu;
  if (ah - (897u << 20) < (254u << 20)) {
    unsigned v = ((ah - (896u << 20)) << 3) | (lo >> 29);
    v += ((lo & 0x1FFFFFFFu) + 0x0FFFFFFFu + (v & 1u)) >> 29;
    return __uint_as_float((hi & 0x80000000u) | v);
  }
  return f64_to_f32_any(x);
}

// FP32 -> FP64 (exact) with integer instructions only: zeros keep their sign, subnormals
// are normalised, Inf and NaN (with its payload) carry over.
__device__ __forceinline__ double f32_to_f64_any(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const unsigned int e = (u >> 23) & 0xFF;
  const unsigned int m = u & 0x7FFFFF;
  if (e == 0xFF) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull | ((unsigned long long)m << 29)));
  if (e == 0) {
    if (m == 0) return __longlong_as_double((long long)sign);
    // m * 2^-149 with its leading bit p (0..22) moved into the implicit bit
    const int p = 31 - __clz((int)m);
    const unsigned long long mant = (unsigned long long)(m ^ (1u << p)) << (52 - p);
    return __longlong_as_double((long long)(sign | ((unsigned long long)(p - 149 + 1023) << 52) | mant));
  }
  return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 1023 - 127) << 52) |
                                          ((unsigned long long)m << 29)));
}

// The same for FP32 normal numbers, inline: exponent rebiased by 896, mantissa shifted up 29.
__device__ __forceinline__ double f32_to_f64(float f) {
  const unsigned u = __float_as_uint(f);
  if ((u & 0x7F800000u) - 0x00800000u < 0x7F000000u)
    return __hiloint2double((int)((u & 0x80000000u) | (((u & 0x7FFFFFFFu) >> 3) + (896u << 20))), (int)(u << 29));
  return f32_to_f64_any(f);
}

__device__ __forceinline__ float d_f_elem_f(const DevLayout& D, const double* op, int herm, int a, int b) {
  const int c1 = D.con[a], c2 = D.con[b];
  if (c1 + c2 == 0) return f64_to_f32(op[D.off_fpp + D.loc[a] + (int64_t)D.loc[b] * D.P]);
  if (c1 + c2 == 2) return f64_to_f32(op[D.off_fhh + D.loc[a] + (int64_t)D.loc[b] * D.A]);
  if (c1 > c2) {
    const float v = f64_to_f32(op[D.off_fph + D.loc[b] + (int64_t)D.loc[a] * D.P]);
    return herm < 0 ? -v : v;
  }
  return f64_to_f32(op[D.off_fph + D.loc[a] + (int64_t)D.loc[b] * D.P]);
}

__device__ __forceinline__ double d_v_elem(const DevLayout& D, const double* op, int herm, int a, int b, int c, int d,
                                           int J) {
  VRef r;
  if (!d_vref(D, a, b, c, d, J, r)) return 0.0;
  return op[r.idx] * (r.herm ? herm * r.pre : r.pre);
}

// (q, g, IX, JX) of unique 2b element u (upper triangle incl. diagonal for square arrays,
// column-major order within each array).
__device__ __forceinline__ void d_unique_decode(const DevLayout& D, int64_t u, int& q, int& g, int& IX, int& JX) {
  int lo = 0, hi = D.nblocks * 6;  // find k with uoff[k] <= u < uoff[k+1]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (D.uoff[mid] <= u) lo = mid; else hi = mid;
  }
  // skip empty arrays sharing the same start
  while (D.uoff[lo + 1] <= u) ++lo;
  q = lo / 6;
  g = lo - q * 6;
  const int64_t e = u - D.uoff[lo];
  const int n1 = D.gn1[lo];
  if (g == 0 || g == 3 || g == 4) {
    // column JX holds JX+1 elements (IX = 0..JX)
    int j = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);  // corrected below
    while ((int64_t)(j + 1) * (j + 2) / 2 <= e) ++j;
    while ((int64_t)j * (j + 1) / 2 > e) --j;
    JX = j;
    IX = (int)(e - (int64_t)j * (j + 1) / 2);
  } else {
    JX = (int)(e / n1);
    IX = (int)(e - (int64_t)JX * n1);
  }
}

#endif  // __CUDACC__

}  // namespace imsrg
