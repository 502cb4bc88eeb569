// CPU restatement (FP64, OpenMP) of the EOM-IMSRG IMSRG(2) commutator hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests/, the smoke
// check of __graft_entry__.py and the cpu_baseline leg of bench.py load it as the
// checker or as the timed CPU restatement of the reference algorithm.  The product
// (eom-imsrg_gb300/) never links, loads or calls it.
//
// Every routine restates the reference's algorithm in its own code and cites the
// Fortran it follows (paths relative to the EOM-IMSRG source tree):
//   basis / channel layout ........ src/basic_IMSRG.f90:385-440, 521-685
//   element accessors ............. src/basic_IMSRG.f90:1191-1221, 1314-1429, 2051-2090
//   6j / 9j ....................... src/basic_IMSRG.f90:2227-2332, 2553-2599; src/anglib.f:263-338, 546-567
//   operator algebra, norms ....... src/basic_IMSRG.f90:3005-3032, 3551-3663, 4056-4129, 4165-4199
//   cross-coupled (Pandya) ........ src/cross_coupled.f90:61-177, 1167-1173, 1190-1300, 2196-2210
//   commutators ................... src/commutators.f90:10-925
//   White generator ............... src/generators.f90:4-106
//   Magnus / BCH / Euler .......... src/IMSRG_MAGNUS.f90:149-234, 620-691, 754-764
//   brute-force known answers ..... src/brute_force_testing.f90:15-120, 1765-1823, 1887-1928, 1975-2076
//
// Operators are passed as (slab, herm) pairs.  The slab is the reference's sq_op
// content flattened in a fixed order (all arrays column-major, full storage):
//   [E0][fhh A*A][fpp P*P][fph P*A][ for q=1..nblocks, g=1..6: gam(g) of block q ]
// with gam(1)=pppp(npp,npp) gam(2)=ppph(npp,nph) gam(3)=pphh(npp,nhh)
//      gam(4)=phph(nph,nph) gam(5)=hhhh(nhh,nhh) gam(6)=phhh(nph,nhh).
// Cross-coupled matrices are concatenated CCX(q)(rlen,nph) blocks, WCC(q)(rlen,rlen).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

inline bool tri(int j1, int j2, int J) { return J <= j1 + j2 && J >= std::abs(j1 - j2); }
inline double sgn(int n) { return (n & 1) ? -1.0 : 1.0; }   // (-1)**n, n any integer
inline int kd(int a, int b) { return a == b ? 1 : 0; }

// ---------------------------------------------------------------- dgemm
// column-major, BLAS semantics: C = alpha*op(A)*op(B) + beta*C
typedef void (*blas_dgemm32)(const char*, const char*, const int*, const int*, const int*,
                             const double*, const double*, const int*, const double*, const int*,
                             const double*, double*, const int*);
typedef void (*blas_dgemm64)(const char*, const char*, const int64_t*, const int64_t*, const int64_t*,
                             const double*, const double*, const int64_t*, const double*, const int64_t*,
                             const double*, double*, const int64_t*);
void* g_blas = nullptr;
int g_blas_ilp64 = 0;

void own_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double* A, int lda,
               const double* B, int ldb, double beta, double* C, int ldc) {
  if (m <= 0 || n <= 0) return;
  const long work = (long)m * n * (k > 0 ? k : 1);
  const int KB = 256;
  // scale C first
#pragma omp parallel for schedule(static) if (work > (1L << 16))
  for (int j = 0; j < n; ++j) {
    double* c = C + (size_t)j * ldc;
    if (beta == 0.0) for (int i = 0; i < m; ++i) c[i] = 0.0;
    else if (beta != 1.0) for (int i = 0; i < m; ++i) c[i] *= beta;
  }
  if (k <= 0 || alpha == 0.0) return;
  for (int k0 = 0; k0 < k; k0 += KB) {
    const int k1 = std::min(k, k0 + KB);
#pragma omp parallel for schedule(static) if (work > (1L << 16))
    for (int j = 0; j < n; ++j) {
      double* c = C + (size_t)j * ldc;
      if (ta == 'N') {
        for (int p = k0; p < k1; ++p) {
          const double b = alpha * ((tb == 'N') ? B[p + (size_t)j * ldb] : B[j + (size_t)p * ldb]);
          const double* a = A + (size_t)p * lda;
          for (int i = 0; i < m; ++i) c[i] += a[i] * b;
        }
      } else {
        for (int i = 0; i < m; ++i) {
          const double* a = A + (size_t)i * lda;
          double s = 0.0;
          if (tb == 'N') {
            const double* b = B + (size_t)j * ldb;
            for (int p = k0; p < k1; ++p) s += a[p] * b[p];
          } else {
            for (int p = k0; p < k1; ++p) s += a[p] * B[j + (size_t)p * ldb];
          }
          c[i] += alpha * s;
        }
      }
    }
  }
}

void dgemm(char ta, char tb, int m, int n, int k, double alpha, const double* A, int lda,
           const double* B, int ldb, double beta, double* C, int ldc) {
  if (m <= 0 || n <= 0) return;
  if (g_blas && k > 0) {
    if (g_blas_ilp64) {
      int64_t M = m, N = n, K = k, LA = std::max(lda, 1), LB = std::max(ldb, 1), LC = std::max(ldc, 1);
      ((blas_dgemm64)g_blas)(&ta, &tb, &M, &N, &K, &alpha, A, &LA, B, &LB, &beta, C, &LC);
    } else {
      int M = m, N = n, K = k, LA = std::max(lda, 1), LB = std::max(ldb, 1), LC = std::max(ldc, 1);
      ((blas_dgemm32)g_blas)(&ta, &tb, &M, &N, &K, &alpha, A, &LA, B, &LB, &beta, C, &LC);
    }
    return;
  }
  own_dgemm(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

// ---------------------------------------------------------------- angular momentum
// Racah formula for the 6j symbol with log-factorials (the published formula the
// reference's d6ji evaluates, src/anglib.f:285-338).  Arguments are 2*j.
struct AngMom {
  std::vector<double> lf;  // log(n!)
  AngMom() {
    lf.resize(1001);
    lf[0] = 0.0;
    for (int i = 1; i <= 1000; ++i) lf[i] = lf[i - 1] + std::log((double)i);
  }
  double delta(int a, int b, int c) const {  // log of triangle coefficient (doubled args)
    return 0.5 * (lf[(a + b - c) / 2] + lf[(a - b + c) / 2] + lf[(-a + b + c) / 2] - lf[(a + b + c) / 2 + 1]);
  }
  double sixj(int j1, int j2, int j3, int l1, int l2, int l3) const {
    if (j1 < 0 || j2 < 0 || j3 < 0 || l1 < 0 || l2 < 0 || l3 < 0) return 0.0;
    if (!tri(j1, j2, j3) || !tri(j1, l2, l3) || !tri(l1, j2, l3) || !tri(l1, l2, j3)) return 0.0;
    if (((j1 + j2 + j3) & 1) || ((j1 + l2 + l3) & 1) || ((l1 + j2 + l3) & 1) || ((l1 + l2 + j3) & 1)) return 0.0;
    const double d = delta(j1, j2, j3) + delta(j1, l2, l3) + delta(l1, j2, l3) + delta(l1, l2, j3);
    const int a1 = (j1 + j2 + j3) / 2, a2 = (j1 + l2 + l3) / 2, a3 = (l1 + j2 + l3) / 2, a4 = (l1 + l2 + j3) / 2;
    const int b1 = (j1 + j2 + l1 + l2) / 2, b2 = (j2 + j3 + l2 + l3) / 2, b3 = (j3 + j1 + l3 + l1) / 2;
    const int tmin = std::max(std::max(a1, a2), std::max(a3, a4));
    const int tmax = std::min(b1, std::min(b2, b3));
    double s = 0.0;
    for (int t = tmin; t <= tmax; ++t) {
      const double lt = d + lf[t + 1] - lf[t - a1] - lf[t - a2] - lf[t - a3] - lf[t - a4] - lf[b1 - t] -
                        lf[b2 - t] - lf[b3 - t];
      s += sgn(t) * std::exp(lt);
    }
    return s;
  }
  // 9j as a sum over products of three 6j symbols (Edmonds 6.4.3), rows (j1 j2 j3)(j4 j5 j6)(j7 j8 j9)
  double ninej(int j1, int j2, int j3, int j4, int j5, int j6, int j7, int j8, int j9) const {
    int xmin = std::max(std::abs(j1 - j9), std::max(std::abs(j4 - j8), std::abs(j2 - j6)));
    int xmax = std::min(j1 + j9, std::min(j4 + j8, j2 + j6));
    double s = 0.0;
    for (int x = xmin; x <= xmax; x += 2) {
      s += sgn(x) * (x + 1.0) * sixj(j1, j4, j7, j8, j9, x) * sixj(j2, j5, j8, j4, x, j6) *
           sixj(j3, j6, j9, x, j1, j2);
    }
    return s;
  }
};
const AngMom& angmom() {
  static AngMom a;
  return a;
}

// ---------------------------------------------------------------- basis + layout
struct Basis {
  int N = 0, A = 0, P = 0, JM = 0, lmax = 0, NJ = 0, eMax = 0;
  double hw = 0;
  int Aprot = 0, Aneut = 0;
  std::vector<int> nn, ll, jj, tz, con, holes, parts, loc;  // loc: index within holes / parts (0-based)
  std::vector<std::vector<int>> same;                      // orbits with the same (j,l,tz), ascending
  // sq_op channels (src/basic_IMSRG.f90:521-685): q = 3*J2 + 2*(Tz+1) + Par (0-based)
  int nblocks = 0;
  std::vector<int> lamJ, lamP, lamT;
  std::vector<std::array<int, 3>> ncls;                         // npp, nph, nhh
  std::vector<std::array<std::vector<int>, 3>> qa, qb;          // pair lists (first, second orbit)
  std::vector<int> pairpos;                                     // [(a*N+b)*NJ + J/2] for a<=b
  // slab offsets
  int64_t off_fhh = 1, off_fpp = 0, off_fph = 0, slab = 0;
  std::vector<std::array<int64_t, 6>> goff;
  std::vector<std::array<int, 6>> gn1, gn2;
  // cross-coupled (src/cross_coupled.f90:61-177): q = JC/2 + Tz*(JM+1) + Par*2*(JM+1)
  int ncc = 0;
  std::vector<int> cc_rlen, cc_nph, cc_J;
  std::vector<int64_t> cc_off, wcc_off;
  int64_t cc_size = 0, wcc_size = 0;
  std::vector<int> ccr;   // [(a*N+b)*NJ + JC/2] -> r index in its CC channel (-1 if absent)
  std::vector<int> ccnb;  // same, ph column index (-1 unless a particle, b hole)
  std::vector<std::vector<int>> cc_pa, cc_pb, cc_php, cc_phh;  // rows (a,b) and ph columns (p,h)

  int ccq(int JC, int TZ, int PAR) const { return JC / 2 + TZ * (JM + 1) + PAR * 2 * (JM + 1); }
  int block(int J2, int T, int Par) const { return 3 * J2 + 2 * (T + 1) + Par; }
  double* X(double* op, int q, int g) const { return op + goff[q][g]; }
  const double* X(const double* op, int q, int g) const { return op + goff[q][g]; }
};

Basis* build_basis(int N, const int* nn, const int* ll, const int* jj, const int* tz, const int* con,
                   int eMax, double hw, int Aprot, int Aneut) {
  Basis* b = new Basis();
  b->N = N;
  b->eMax = eMax;
  b->hw = hw;
  b->Aprot = Aprot;
  b->Aneut = Aneut;
  b->nn.assign(nn, nn + N);
  b->ll.assign(ll, ll + N);
  b->jj.assign(jj, jj + N);
  b->tz.assign(tz, tz + N);
  b->con.assign(con, con + N);
  b->loc.resize(N);
  // find_holes (src/basic_IMSRG.f90:385-440): hb4/pb4 counts give the local indices
  for (int i = 0; i < N; ++i) {
    if (con[i]) { b->loc[i] = (int)b->holes.size(); b->holes.push_back(i); }
    else { b->loc[i] = (int)b->parts.size(); b->parts.push_back(i); }
  }
  b->A = (int)b->holes.size();
  b->P = N - b->A;
  b->JM = *std::max_element(jj, jj + N);
  b->lmax = *std::max_element(ll, ll + N);
  b->NJ = b->JM + 1;
  b->same.resize(N);
  for (int i = 0; i < N; ++i)
    for (int k = 0; k < N; ++k)
      if (jj[k] == jj[i] && ll[k] == ll[i] && tz[k] == tz[i]) b->same[i].push_back(k);

  // allocate_blocks
  const int NJ = b->NJ;
  b->nblocks = (b->JM + 1) * 6;
  b->lamJ.resize(b->nblocks); b->lamP.resize(b->nblocks); b->lamT.resize(b->nblocks);
  b->ncls.resize(b->nblocks); b->qa.resize(b->nblocks); b->qb.resize(b->nblocks);
  b->pairpos.assign((size_t)N * N * NJ, -1);
  int q = 0;
  for (int Jt = 0; Jt <= 2 * b->JM; Jt += 2)
    for (int Tz = -1; Tz <= 1; ++Tz)
      for (int Par = 0; Par <= 1; ++Par) {
        b->lamJ[q] = Jt; b->lamP[q] = Par; b->lamT[q] = Tz;
        std::array<int, 3> n = {0, 0, 0};
        for (int i = 0; i < N; ++i)
          for (int j = i; j < N; ++j) {
            if (Tz != (tz[i] + tz[j]) / 2) continue;
            if (Par != (ll[i] + ll[j]) % 2) continue;
            if (!tri(jj[i], jj[j], Jt)) continue;
            const int cx = con[i] + con[j];
            b->qa[q][cx].push_back(i);
            b->qb[q][cx].push_back(j);
            b->pairpos[((size_t)i * N + j) * NJ + Jt / 2] = n[cx]++;
          }
        b->ncls[q] = n;
        ++q;
      }
  // slab layout
  int64_t o = 1;
  b->off_fhh = o; o += (int64_t)b->A * b->A;
  b->off_fpp = o; o += (int64_t)b->P * b->P;
  b->off_fph = o; o += (int64_t)b->P * b->A;
  b->goff.resize(b->nblocks); b->gn1.resize(b->nblocks); b->gn2.resize(b->nblocks);
  static const int sea1[6] = {0, 0, 0, 1, 2, 1}, sea2[6] = {0, 1, 2, 1, 2, 2};
  for (int qq = 0; qq < b->nblocks; ++qq)
    for (int g = 0; g < 6; ++g) {
      b->gn1[qq][g] = b->ncls[qq][sea1[g]];
      b->gn2[qq][g] = b->ncls[qq][sea2[g]];
      b->goff[qq][g] = o;
      o += (int64_t)b->gn1[qq][g] * b->gn2[qq][g];
    }
  b->slab = o;

  // allocate_CCMAT: channels with JC fastest, then Tz=|tz_a-tz_b|/2, then parity
  b->ncc = (b->JM + 1) * 4;
  b->cc_rlen.assign(b->ncc, 0); b->cc_nph.assign(b->ncc, 0); b->cc_J.assign(b->ncc, 0);
  b->cc_pa.resize(b->ncc); b->cc_pb.resize(b->ncc); b->cc_php.resize(b->ncc); b->cc_phh.resize(b->ncc);
  b->ccr.assign((size_t)N * N * NJ, -1);
  b->ccnb.assign((size_t)N * N * NJ, -1);
  for (int q1 = 0; q1 < b->ncc; ++q1) {
    const int JC = (q1 % (b->JM + 1)) * 2;
    const int PAR = q1 / (2 * b->JM + 2);
    const int TZ = (q1 % (2 * b->JM + 2)) / (b->JM + 1);
    b->cc_J[q1] = JC;
    int r = 0, nb = 0;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        if (!tri(jj[i], jj[j], JC)) continue;
        if ((ll[i] + ll[j]) % 2 != PAR) continue;
        if (std::abs(tz[i] - tz[j]) / 2 != TZ) continue;
        if (con[i] == 0 && con[j] == 1) {
          b->ccnb[((size_t)i * N + j) * NJ + JC / 2] = nb++;
          b->cc_php[q1].push_back(i);
          b->cc_phh[q1].push_back(j);
        }
        b->ccr[((size_t)i * N + j) * NJ + JC / 2] = r++;
        b->cc_pa[q1].push_back(i);
        b->cc_pb[q1].push_back(j);
      }
    b->cc_rlen[q1] = r;
    b->cc_nph[q1] = nb;
  }
  b->cc_off.resize(b->ncc); b->wcc_off.resize(b->ncc);
  int64_t c1 = 0, c2 = 0;
  for (int q1 = 0; q1 < b->ncc; ++q1) {
    b->cc_off[q1] = c1; c1 += (int64_t)b->cc_rlen[q1] * b->cc_nph[q1];
    b->wcc_off[q1] = c2; c2 += (int64_t)b->cc_rlen[q1] * b->cc_rlen[q1];
  }
  b->cc_size = c1;
  b->wcc_size = c2;
  return b;
}

// ---------------------------------------------------------------- accessors
// f_elem (src/basic_IMSRG.f90:1191-1221)
inline double f_elem(const Basis& B, const double* op, int herm, int a, int b) {
  const int c1 = B.con[a], c2 = B.con[b];
  switch (c1 + c2) {
    case 0: return op[B.off_fpp + B.loc[a] + (int64_t)B.loc[b] * B.P];
    case 1:
      if (c1 > c2) return op[B.off_fph + B.loc[b] + (int64_t)B.loc[a] * B.P] * herm;
      return op[B.off_fph + B.loc[a] + (int64_t)B.loc[b] * B.P];
    default: return op[B.off_fhh + B.loc[a] + (int64_t)B.loc[b] * B.A];
  }
}
inline double& fhh(const Basis& B, double* op, int i, int j) { return op[B.off_fhh + i + (int64_t)j * B.A]; }
inline double& fpp(const Basis& B, double* op, int i, int j) { return op[B.off_fpp + i + (int64_t)j * B.P]; }
inline double& fph(const Basis& B, double* op, int i, int j) { return op[B.off_fph + i + (int64_t)j * B.P]; }
inline double cfhh(const Basis& B, const double* op, int i, int j) { return op[B.off_fhh + i + (int64_t)j * B.A]; }
inline double cfpp(const Basis& B, const double* op, int i, int j) { return op[B.off_fpp + i + (int64_t)j * B.P]; }
inline double cfph(const Basis& B, const double* op, int i, int j) { return op[B.off_fph + i + (int64_t)j * B.P]; }

// the six storage classes: (class of bra pair, class of ket pair) -> g (src/basic_IMSRG.f90:1380-1385)
inline int qx_of(int C1, int C2) {  // C = con sum (0 pp, 1 ph, 2 hh), C1 <= C2 assumed by caller
  static const int tab[3][3] = {{0, 1, 2}, {1, 3, 5}, {2, 5, 4}};
  return tab[C1][C2];
}

// v_elem (src/basic_IMSRG.f90:1314-1429)
double v_elem(const Basis& B, const double* op, int herm, int a, int b, int c, int d, int J) {
  const int ja = B.jj[a], jb = B.jj[b], jc = B.jj[c], jd = B.jj[d];
  if (!(tri(ja, jb, J) && tri(jc, jd, J))) return 0.0;
  const int P = (B.ll[a] + B.ll[b]) % 2;
  if ((B.ll[c] + B.ll[d]) % 2 != P) return 0.0;
  const int T = (B.tz[a] + B.tz[b]) / 2;
  if (B.tz[c] + B.tz[d] != 2 * T) return 0.0;
  const int q = B.block(J, T, P);
  const int C1 = B.con[a] + B.con[b], C2 = B.con[c] + B.con[d];
  const int g = qx_of(std::min(C1, C2), std::max(C1, C2));
  double pre = 1.0;
  const int N = B.N, NJ = B.NJ;
  int i1, i2;
  if (a > b) {
    i1 = B.pairpos[((size_t)b * N + a) * NJ + J / 2];
    pre = sgn(1 + (ja + jb - J) / 2);
  } else {
    if (a == b) pre *= std::sqrt(2.0);
    i1 = B.pairpos[((size_t)a * N + b) * NJ + J / 2];
  }
  if (c > d) {
    i2 = B.pairpos[((size_t)d * N + c) * NJ + J / 2];
    pre *= sgn(1 + (jc + jd - J) / 2);
  } else {
    if (c == d) pre *= std::sqrt(2.0);
    i2 = B.pairpos[((size_t)c * N + d) * NJ + J / 2];
  }
  const double* X = B.X(op, q, g);
  const int n1 = B.gn1[q][g];
  if (C1 > C2) return X[i2 + (int64_t)i1 * n1] * herm * pre;
  return X[i1 + (int64_t)i2 * n1] * pre;
}

// twobody_monopole (src/basic_IMSRG.f90:2075-2090)
double monopole(const Basis& B, const double* op, int herm, int a, int b) {
  const int ja = B.jj[a], jb = B.jj[b];
  double sm = 0.0;
  for (int JT = std::abs(ja - jb); JT <= ja + jb; JT += 2) sm += (JT + 1) * v_elem(B, op, herm, a, b, a, b, JT);
  return sm / (ja + 1.0) / (jb + 1.0);
}

// Tabulated 6j symbols {j1 j2 j3; j4 j5 j6} with j1,j2,j4,j5 half-integer orbit spins and
// j3, j6 integer, as store_6j/sixj do (src/basic_IMSRG.f90:2227-2332, 2553-2599): one block
// per (j1,j2,j4,j5) quadruple holding every allowed (j3, j6).
struct SixjTable {
  int nh = 0;
  std::vector<int64_t> off;
  std::vector<int> j3min, j6min, n6;
  std::vector<double> val;
  void build(int jmax2) {
    nh = (jmax2 + 1) / 2;
    const size_t nq = (size_t)nh * nh * nh * nh;
    off.assign(nq, 0); j3min.assign(nq, 0); j6min.assign(nq, 0); n6.assign(nq, 0);
    int64_t o = 0;
    for (int h1 = 0; h1 < nh; ++h1) for (int h2 = 0; h2 < nh; ++h2)
    for (int h4 = 0; h4 < nh; ++h4) for (int h5 = 0; h5 < nh; ++h5) {
      const int j1 = 2 * h1 + 1, j2 = 2 * h2 + 1, j4 = 2 * h4 + 1, j5 = 2 * h5 + 1;
      const size_t k = (((size_t)h1 * nh + h2) * nh + h4) * nh + h5;
      const int a = std::max(std::abs(j1 - j2), std::abs(j4 - j5)), b = std::min(j1 + j2, j4 + j5);
      const int c = std::max(std::abs(j1 - j5), std::abs(j4 - j2)), d = std::min(j1 + j5, j4 + j2);
      off[k] = o; j3min[k] = a; j6min[k] = c;
      const int n3 = a <= b ? (b - a) / 2 + 1 : 0, m6 = c <= d ? (d - c) / 2 + 1 : 0;
      n6[k] = m6;
      o += (int64_t)n3 * m6;
    }
    val.assign(o, 0.0);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t kk = 0; kk < (int64_t)nq; ++kk) {
      const size_t k = (size_t)kk;
      const int h5 = k % nh, h4 = (k / nh) % nh, h2 = (k / nh / nh) % nh, h1 = (int)(k / nh / nh / nh);
      const int j1 = 2 * h1 + 1, j2 = 2 * h2 + 1, j4 = 2 * h4 + 1, j5 = 2 * h5 + 1;
      const int b = std::min(j1 + j2, j4 + j5), d = std::min(j1 + j5, j4 + j2);
      for (int j3 = j3min[k]; j3 <= b; j3 += 2)
        for (int j6 = j6min[k]; j6 <= d; j6 += 2)
          val[off[k] + ((j3 - j3min[k]) / 2) * n6[k] + (j6 - j6min[k]) / 2] = angmom().sixj(j1, j2, j3, j4, j5, j6);
    }
  }
  double get(int j1, int j2, int j3, int j4, int j5, int j6) const {
    if (!(tri(j1, j2, j3) && tri(j4, j5, j3) && tri(j1, j5, j6) && tri(j4, j2, j6))) return 0.0;
    const size_t k = ((((size_t)(j1 >> 1) * nh + (j2 >> 1)) * nh + (j4 >> 1)) * nh + (j5 >> 1));
    return val[off[k] + ((j3 - j3min[k]) / 2) * n6[k] + (j6 - j6min[k]) / 2];
  }
};
SixjTable* g_sixj = nullptr;
void ensure_sixj(int jmax2) {
  if (g_sixj && g_sixj->nh >= (jmax2 + 1) / 2) return;
  SixjTable* t = new SixjTable();
  t->build(jmax2);
  g_sixj = t;  // an earlier, smaller table stays allocated: bases may still be in use
}
inline double sixj(int j1, int j2, int j3, int j4, int j5, int j6) { return g_sixj->get(j1, j2, j3, j4, j5, j6); }

// ---------------------------------------------------------------- commutators
// commutator_110 (src/commutators.f90:10-33)
double comm110(const Basis& B, const double* L, int hL, const double* R, int hR) {
  double sm = 0.0;
  for (int i = 0; i < B.A; ++i) {
    const int ji = B.jj[B.holes[i]];
    for (int a = 0; a < B.P; ++a)
      sm += (cfph(B, L, a, i) * cfph(B, R, a, i) * hL - cfph(B, R, a, i) * cfph(B, L, a, i) * hR) * (ji + 1);
  }
  return sm;
}

// commutator_111 (src/commutators.f90:36-80)
void comm111(const Basis& B, const double* L, int hL, const double* R, int hR, double* RES, int hRES) {
  (void)hRES;
  const int A = B.A, P = B.P;
  std::vector<double> th1(A * A), th2(A * A), tb1(P * A), tb2(P * A), tp1((size_t)P * P), tp2((size_t)P * P);
  const double *Lhh = L + B.off_fhh, *Rhh = R + B.off_fhh, *Lph = L + B.off_fph, *Rph = R + B.off_fph;
  const double *Lpp = L + B.off_fpp, *Rpp = R + B.off_fpp;
  dgemm('N', 'N', A, A, A, 1.0, Lhh, A, Rhh, A, 0.0, th1.data(), A);
  dgemm('T', 'N', A, A, P, 1.0, Lph, P, Rph, P, 0.0, th2.data(), A);
  for (int j = 0; j < A; ++j)
    for (int i = 0; i < A; ++i)
      fhh(B, RES, i, j) = th1[i + j * A] + th2[i + j * A] * hL - (th1[j + i * A] * hL + th2[j + i * A]) * hR;
  dgemm('N', 'N', P, A, A, 1.0, Lph, P, Rhh, A, 0.0, tb1.data(), P);
  dgemm('N', 'N', P, A, P, 1.0, Lpp, P, Rph, P, 0.0, tb2.data(), P);
  for (int k = 0; k < P * A; ++k) RES[B.off_fph + k] = tb1[k] + tb2[k];
  dgemm('N', 'N', P, A, A, 1.0, Rph, P, Lhh, A, 0.0, tb1.data(), P);
  dgemm('N', 'N', P, A, P, 1.0, Rpp, P, Lph, P, 0.0, tb2.data(), P);
  for (int k = 0; k < P * A; ++k) RES[B.off_fph + k] = RES[B.off_fph + k] - tb1[k] - tb2[k];
  dgemm('N', 'T', P, P, A, 1.0, Lph, P, Rph, P, 0.0, tp1.data(), P);
  dgemm('N', 'N', P, P, P, 1.0, Lpp, P, Rpp, P, 0.0, tp2.data(), P);
  for (int j = 0; j < P; ++j)
    for (int i = 0; i < P; ++i)
      fpp(B, RES, i, j) = tp1[i + (size_t)j * P] * hR + tp2[i + (size_t)j * P] -
                          (tp1[j + (size_t)i * P] + tp2[j + (size_t)i * P] * hR) * hL;
}

// commutator_121 (src/commutators.f90:83-280).  v_same(L) reads L at the position of
// the preceding v_elem(...,R,...) call, i.e. v_elem(...,L,...) for these operators.
void comm121(const Basis& B, const double* L, int hL, const double* R, int hR, double* RES, int hRES) {
  auto inner = [&](int pk, int qk) {
    const int jq = B.jj[qk];
    double sm = 0.0;
    for (int a = 0; a < B.P; ++a) {
      const int ak = B.parts[a];
      for (int i = 0; i < B.A; ++i) {
        const int ik = B.holes[i];
        if (B.jj[ik] != B.jj[ak] || B.ll[ik] != B.ll[ak] || B.tz[ik] != B.tz[ak]) continue;
        const int ji = B.jj[ik];
        double smx = 0, smy = 0, smx2 = 0, smy2 = 0;
        for (int JT = std::abs(ji - jq); JT <= ji + jq; JT += 2) {
          smx += v_elem(B, R, hR, ak, pk, ik, qk, JT) * (JT + 1);
          smx2 += v_elem(B, L, hL, ak, pk, ik, qk, JT) * (JT + 1);
          smy += v_elem(B, R, hR, ik, pk, ak, qk, JT) * (JT + 1);
          smy2 += v_elem(B, L, hL, ik, pk, ak, qk, JT) * (JT + 1);
        }
        sm += cfph(B, L, a, i) * (hL * smx - smy) - cfph(B, R, a, i) * (hR * smx2 - smy2);
      }
    }
    return sm;
  };
  auto same = [&](int x, int y) { return B.jj[x] == B.jj[y] && B.ll[x] == B.ll[y] && B.tz[x] == B.tz[y]; };
  for (int p = 0; p < B.A; ++p)
    for (int q = p; q < B.A; ++q) {
      const int pk = B.holes[p], qk = B.holes[q];
      if (!same(pk, qk)) continue;
      const double sm = inner(pk, qk);
      fhh(B, RES, p, q) += sm / (B.jj[pk] + 1.0);
      fhh(B, RES, q, p) = fhh(B, RES, p, q) * hRES;
    }
  for (int p = 0; p < B.P; ++p)
    for (int q = p; q < B.P; ++q) {
      const int pk = B.parts[p], qk = B.parts[q];
      if (!same(pk, qk)) continue;
      const double sm = inner(pk, qk);
      fpp(B, RES, p, q) += sm / (B.jj[pk] + 1.0);
      fpp(B, RES, q, p) = fpp(B, RES, p, q) * hRES;
    }
  for (int p = 0; p < B.P; ++p)
    for (int q = 0; q < B.A; ++q) {
      const int pk = B.parts[p], qk = B.holes[q];
      if (!same(pk, qk)) continue;
      const double sm = inner(pk, qk);
      fph(B, RES, p, q) += sm / (B.jj[pk] + 1.0);
    }
}

static const int SEA1[6] = {0, 0, 0, 1, 2, 1}, SEA2[6] = {0, 1, 2, 1, 2, 2};
static const bool SQS[6] = {true, false, false, true, true, false};

// commutator_122 (src/commutators.f90:283-396): ASSIGNS every 2b element
void comm122(const Basis& B, const double* L, int hL, const double* R, int hR, double* RES, int hRES) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int q = 0; q < B.nblocks; ++q) {
    const int JT = B.lamJ[q];
    for (int g = 0; g < 6; ++g) {
      const int n1 = B.gn1[q][g], n2 = B.gn2[q][g];
      if (n1 * n2 == 0) continue;
      const int c1 = SEA1[g], c2 = SEA2[g];
      double* X = B.X(RES, q, g);
      for (int IX = 0; IX < n1; ++IX) {
        const int a = B.qa[q][c1][IX], b = B.qb[q][c1][IX];
        for (int JX = SQS[g] ? IX : 0; JX < n2; ++JX) {
          const int c = B.qa[q][c2][JX], d = B.qb[q][c2][JX];
          double sm = 0.0;
          for (int i : B.same[a])
            sm += f_elem(B, L, hL, a, i) * v_elem(B, R, hR, i, b, c, d, JT) -
                  f_elem(B, R, hR, a, i) * v_elem(B, L, hL, i, b, c, d, JT);
          for (int i : B.same[b])
            sm += f_elem(B, L, hL, b, i) * v_elem(B, R, hR, a, i, c, d, JT) -
                  f_elem(B, R, hR, b, i) * v_elem(B, L, hL, a, i, c, d, JT);
          for (int i : B.same[c])
            sm += -f_elem(B, L, hL, i, c) * v_elem(B, R, hR, a, b, i, d, JT) +
                  f_elem(B, R, hR, i, c) * v_elem(B, L, hL, a, b, i, d, JT);
          for (int i : B.same[d])
            sm += -f_elem(B, L, hL, i, d) * v_elem(B, R, hR, a, b, c, i, JT) +
                  f_elem(B, R, hR, i, d) * v_elem(B, L, hL, a, b, c, i, JT);
          sm = sm / std::sqrt(1.0 + kd(a, b)) / std::sqrt(1.0 + kd(c, d));
          X[IX + (int64_t)JX * n1] = sm;
          if (SQS[g]) X[JX + (int64_t)IX * n1] = sm * hRES;
        }
      }
    }
  }
}

// commutator_220 (src/commutators.f90:399-432)
double comm220(const Basis& B, const double* L, int hL, const double* R, int hR) {
  if (hR * hL != -1) return 0.0;
  double sm = 0.0;
  for (int q = 0; q < B.nblocks; ++q) {
    const int np = B.ncls[q][0], nh = B.ncls[q][2];
    const double *XL = B.X(L, q, 2), *XR = B.X(R, q, 2);
    double smx = 0.0;
    for (int IX = 0; IX < np; ++IX)
      for (int JX = 0; JX < nh; ++JX) smx = smx - XL[IX + (int64_t)JX * np] * XR[IX + (int64_t)JX * np] * hR;
    sm += smx * (B.lamJ[q] + 1);
  }
  return sm * 2.0;
}

// commutator_222_pp_hh (src/commutators.f90:581-768): fills w1, w2, accumulates into RES
void comm222pphh(const Basis& B, const double* L, int hL, const double* R, int hR, double* RES, int hRES,
                 double* w1, double* w2) {
  (void)hRES;
  const double pm = hR * hL;
  for (int q = 0; q < B.nblocks; ++q) {
    const int np = B.ncls[q][0], nb = B.ncls[q][1], nh = B.ncls[q][2];
    for (int g = 0; g < 6; ++g) {
      const int64_t n = (int64_t)B.gn1[q][g] * B.gn2[q][g];
      std::fill(B.X(w1, q, g), B.X(w1, q, g) + n, 0.0);
      std::fill(B.X(w2, q, g), B.X(w2, q, g) + n, 0.0);
    }
    const double *L1 = B.X(L, q, 0), *L2 = B.X(L, q, 1), *L3 = B.X(L, q, 2), *L5 = B.X(L, q, 4), *L6 = B.X(L, q, 5);
    const double *R1 = B.X(R, q, 0), *R2 = B.X(R, q, 1), *R3 = B.X(R, q, 2), *R5 = B.X(R, q, 4), *R6 = B.X(R, q, 5);
    double *W11 = B.X(w1, q, 0), *W12 = B.X(w1, q, 1), *W13 = B.X(w1, q, 2), *W14 = B.X(w1, q, 3),
           *W15 = B.X(w1, q, 4), *W16 = B.X(w1, q, 5);
    double *W21 = B.X(w2, q, 0), *W22 = B.X(w2, q, 1), *W23 = B.X(w2, q, 2), *W24 = B.X(w2, q, 3),
           *W25 = B.X(w2, q, 4), *W26 = B.X(w2, q, 5);
    if (np != 0) dgemm('N', 'N', np, np, np, 1.0, L1, np, R1, np, 0.0, W11, np);
    if (nh != 0) dgemm('N', 'N', nh, nh, nh, 1.0, L5, nh, R5, nh, 0.0, W25, nh);
    if (np * nh != 0) {
      dgemm('T', 'N', nh, nh, np, 1.0, L3, np, R3, np, 0.0, W15, nh);
      for (int k = 0; k < nh * nh; ++k) W15[k] *= hL;
      dgemm('N', 'T', np, np, nh, 1.0, L3, np, R3, np, 0.0, W21, np);
      for (int64_t k = 0; k < (int64_t)np * np; ++k) W21[k] *= hR;
      dgemm('N', 'N', np, nh, np, -1.0, R1, np, L3, np, 0.0, W13, np);
      dgemm('N', 'N', np, nh, np, 1.0, L1, np, R3, np, 1.0, W13, np);
      dgemm('N', 'N', np, nh, nh, 1.0, R3, np, L5, nh, 0.0, W23, np);
      dgemm('N', 'N', np, nh, nh, 1.0, L3, np, R5, nh, -1.0, W23, np);
    }
    auto antisym_add = [&](double* Y, const double* Wa, const double* Wb, int n) {
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const int64_t ij = i + (int64_t)j * n, ji = j + (int64_t)i * n;
          Y[ij] = Y[ij] + Wa[ij] - Wb[ij] - (Wa[ji] - Wb[ji]) * pm;
        }
    };
    antisym_add(B.X(RES, q, 0), W11, W21, np);
    antisym_add(B.X(RES, q, 4), W15, W25, nh);
    {
      double* Y = B.X(RES, q, 2);
      for (int64_t k = 0; k < (int64_t)np * nh; ++k) Y[k] = Y[k] + W13[k] - W23[k];
    }
    if (nb * nh != 0) {
      dgemm('N', 'T', nb, nb, nh, 1.0, L6, nb, R6, nb, 0.0, W24, nb);
      for (int k = 0; k < nb * nb; ++k) W24[k] *= hR;
    }
    if (nb * np != 0) {
      dgemm('T', 'N', nb, nb, np, 1.0, L2, np, R2, np, 0.0, W14, nb);
      for (int k = 0; k < nb * nb; ++k) W14[k] *= hL;
    }
    antisym_add(B.X(RES, q, 3), W14, W24, nb);
    if (nb * nh != 0) {
      dgemm('N', 'N', nb, nh, nh, 1.0, R6, nb, L5, nh, 0.0, W26, nb);
      dgemm('N', 'N', nb, nh, nh, 1.0, L6, nb, R5, nh, -1.0, W26, nb);
    }
    if (nb * np != 0) {
      dgemm('N', 'N', np, nb, np, 1.0, R1, np, L2, np, 0.0, W12, np);
      dgemm('N', 'N', np, nb, np, 1.0, L1, np, R2, np, -1.0, W12, np);
    }
    if (nb * np * nh != 0) {
      dgemm('T', 'N', nb, nh, np, -1.0 * hR, R2, np, L3, np, 0.0, W16, nb);
      dgemm('T', 'N', nb, nh, np, 1.0 * hL, L2, np, R3, np, 1.0, W16, nb);
      dgemm('N', 'T', np, nb, nh, 1.0, R3, np, L6, nb, 0.0, W22, np);
      dgemm('N', 'T', np, nb, nh, 1.0 * hR, L3, np, R6, nb, -1.0 * hL, W22, np);
    }
    {
      double* Y = B.X(RES, q, 5);
      for (int64_t k = 0; k < (int64_t)nb * nh; ++k) Y[k] = Y[k] + W16[k] - W26[k];
      Y = B.X(RES, q, 1);
      for (int64_t k = 0; k < (int64_t)np * nb; ++k) Y[k] = Y[k] + W12[k] - W22[k];
    }
  }
}

// commutator_221 (src/commutators.f90:435-578); w1, w2 are hermitian workspaces (herm = 1)
void comm221(const Basis& B, int hL, int hR, double* RES, int hRES, const double* w1, const double* w2) {
  const int pm = hR * hL;
  auto same = [&](int x, int y) { return B.jj[x] == B.jj[y] && B.ll[x] == B.ll[y] && B.tz[x] == B.tz[y]; };
  auto trace = [&](int ik, int jk, bool antisym) {
    const int ji = B.jj[ik];
    double sm = 0.0;
    for (int c = 0; c < B.A; ++c) {
      const int ck = B.holes[c], jc = B.jj[ck];
      for (int JT = std::abs(jc - ji); JT <= jc + ji; JT += 2) {
        if (antisym)
          sm += (v_elem(B, w1, 1, ck, ik, ck, jk, JT) - pm * v_elem(B, w1, 1, ck, jk, ck, ik, JT)) * (JT + 1);
        else
          sm += v_elem(B, w1, 1, ck, ik, ck, jk, JT) * (JT + 1);
      }
    }
    for (int c = 0; c < B.P; ++c) {
      const int ck = B.parts[c], jc = B.jj[ck];
      for (int JT = std::abs(jc - ji); JT <= jc + ji; JT += 2) {
        if (antisym)
          sm += (v_elem(B, w2, 1, ck, ik, ck, jk, JT) - pm * v_elem(B, w2, 1, ck, jk, ck, ik, JT)) * (JT + 1);
        else
          sm += v_elem(B, w2, 1, ck, ik, ck, jk, JT) * (JT + 1);
      }
    }
    return sm;
  };
  for (int i = 0; i < B.A; ++i)
    for (int j = i; j < B.A; ++j) {
      const int ik = B.holes[i], jk = B.holes[j];
      if (!same(ik, jk)) continue;
      fhh(B, RES, i, j) += trace(ik, jk, true) / (B.jj[ik] + 1.0);
      fhh(B, RES, j, i) = fhh(B, RES, i, j) * hRES;
    }
  for (int i = 0; i < B.P; ++i)
    for (int j = i; j < B.P; ++j) {
      const int ik = B.parts[i], jk = B.parts[j];
      if (!same(ik, jk)) continue;
      fpp(B, RES, i, j) += trace(ik, jk, true) / (B.jj[ik] + 1.0);
      fpp(B, RES, j, i) = fpp(B, RES, i, j) * hRES;
    }
  for (int i = 0; i < B.P; ++i)
    for (int j = 0; j < B.A; ++j) {
      const int ik = B.parts[i], jk = B.holes[j];
      if (!same(ik, jk)) continue;
      fph(B, RES, i, j) += trace(ik, jk, false) / (B.jj[ik] + 1.0);
    }
}

// calculate_cross_coupled (src/cross_coupled.f90:1190-1300)
void cross_coupled(const Basis& B, const double* op, int herm, double* cc) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int q1 = 0; q1 < B.ncc; ++q1) {
    const int JC = B.cc_J[q1];
    const int rlen = B.cc_rlen[q1];
    double* CC = cc + B.cc_off[q1];
    std::fill(CC, CC + (int64_t)rlen * B.cc_nph[q1], 0.0);
    for (int nbx = 0; nbx < B.cc_nph[q1]; ++nbx) {
      const int p = B.cc_php[q1][nbx], h = B.cc_phh[q1][nbx];
      const int jp = B.jj[p], jh = B.jj[h], lp = B.ll[p], lh = B.ll[h], tp = B.tz[p], th = B.tz[h];
      for (int r = 0; r < rlen; ++r) {
        const int a = B.cc_pa[q1][r], b = B.cc_pb[q1][r];
        const int ja = B.jj[a], jb = B.jj[b], la = B.ll[a], lb = B.ll[b], ta = B.tz[a], tb = B.tz[b];
        if (((la + lh) % 2 == (lb + lp) % 2) && (ta + th == tb + tp)) {
          const int Jmin = std::max(std::abs(jp - jb), std::abs(ja - jh));
          const int Jmax = std::min(jp + jb, ja + jh);
          double sm = 0.0;
          for (int JT = Jmin; JT <= Jmax; JT += 2)
            sm += sgn(JT / 2) * (JT + 1) * sixj(jp, jh, JC, ja, jb, JT) * v_elem(B, op, herm, h, a, p, b, JT);
          CC[r + (int64_t)nbx * rlen] = sm * sgn((jh + jb + JC) / 2) * std::sqrt(JC + 1.0);
        }
      }
    }
  }
}

// commutator_222_ph (src/commutators.f90:771-925)
void comm222ph(const Basis& B, const double* LCC, int hL, const double* RCC, int hR, double* RES, int hRES,
               double* WCC) {
  for (int q = 0; q < B.ncc; ++q) {
    const int nb = B.cc_nph[q], r = B.cc_rlen[q];
    if (nb * r == 0) continue;
    dgemm('N', 'T', r, r, nb, 1.0, LCC + B.cc_off[q], r, RCC + B.cc_off[q], r, 0.0, WCC + B.wcc_off[q], r);
  }
  const int N = B.N, NJ = B.NJ;
  auto rv = [&](int a, int b, int JP) { return B.ccr[((size_t)a * N + b) * NJ + JP / 2]; };
#pragma omp parallel for schedule(dynamic, 1)
  for (int q = 0; q < B.nblocks; ++q) {
    const int Jtot = B.lamJ[q];
    for (int g = 0; g < 6; ++g) {
      const int n1 = B.gn1[q][g], n2 = B.gn2[q][g];
      if (n1 * n2 == 0) continue;
      const int c1 = SEA1[g], c2 = SEA2[g];
      double* X = B.X(RES, q, g);
      for (int IX = 0; IX < n1; ++IX) {
        const int i = B.qa[q][c1][IX], j = B.qb[q][c1][IX];
        const double pre = (i == j) ? .70710678118 : 1.0;
        const int ji = B.jj[i], jj_ = B.jj[j], li = B.ll[i], lj = B.ll[j], ti = B.tz[i], tj = B.tz[j];
        for (int JX = SQS[g] ? IX : 0; JX < n2; ++JX) {
          const int k = B.qa[q][c2][JX], l = B.qb[q][c2][JX];
          const double pre2 = (k == l) ? .70710678118 : 1.0;
          const int jk = B.jj[k], jl = B.jj[l], lk = B.ll[k], ll = B.ll[l], tk = B.tz[k], tl = B.tz[l];
          double sm = 0.0;
          int jmin = std::max(std::abs(jj_ - jl), std::abs(ji - jk));
          int jmax = std::min(jj_ + jl, ji + jk);
          int Tz = std::abs(ti - tk) / 2;
          if (std::abs(tl - tj) != Tz * 2) continue;
          int PAR = (li + lk) % 2;
          if ((ll + lj) % 2 != PAR) continue;
          double phase = sgn((ji + jj_ + jk + jl) / 2);
          for (int JP = jmin; JP <= jmax; JP += 2) {
            const int qx = B.ccq(JP, Tz, PAR);
            const double* W = WCC + B.wcc_off[qx];
            const int64_t rl = B.cc_rlen[qx];
            const int rjl = rv(j, l, JP), rik = rv(i, k, JP), gjl = rv(l, j, JP), gik = rv(k, i, JP);
            sm -= sgn((jl + jk + Jtot) / 2) *
                  ((W[gik + rjl * rl] + phase * W[gjl + rik * rl]) * hL -
                   (phase * W[rik + gjl * rl] + W[rjl + gik * rl]) * hR) *
                  sixj(ji, jj_, Jtot, jl, jk, JP);
          }
          Tz = std::abs(ti - tl) / 2;
          if (std::abs(tk - tj) != Tz * 2) continue;
          PAR = (li + ll) % 2;
          if ((lk + lj) % 2 != PAR) continue;
          jmin = std::max(std::abs(ji - jl), std::abs(jj_ - jk));
          jmax = std::min(ji + jl, jj_ + jk);
          phase = sgn((ji + jj_ + jk + jl) / 2);
          for (int JP = jmin; JP <= jmax; JP += 2) {
            const int qx = B.ccq(JP, Tz, PAR);
            const double* W = WCC + B.wcc_off[qx];
            const int64_t rl = B.cc_rlen[qx];
            const int ril = rv(i, l, JP), rjk = rv(j, k, JP), gil = rv(l, i, JP), gjk = rv(k, j, JP);
            sm += ((W[gil + rjk * rl] + phase * W[gjk + ril * rl]) * hL -
                   (phase * W[ril + gjk * rl] + W[rjk + gil * rl]) * hR) *
                  sixj(ji, jj_, Jtot, jk, jl, JP);
          }
          X[IX + (int64_t)JX * n1] = X[IX + (int64_t)JX * n1] + sm * pre * pre2;
          if (SQS[g]) X[JX + (int64_t)IX * n1] = X[IX + (int64_t)JX * n1] * hRES;
        }
      }
    }
  }
}

// The full IMSRG(2) commutator in the reference's call order
// (src/IMSRG_MAGNUS.f90:207-219; src/brute_force_testing.f90:513-532)
struct Work {
  std::vector<double> w1, w2, lcc, rcc, wcc;
  explicit Work(const Basis& B) : w1(B.slab), w2(B.slab), lcc(B.cc_size), rcc(B.cc_size), wcc(B.wcc_size) {}
};

void full_commutator(const Basis& B, const double* L, int hL, const double* R, int hR, double* RES, int hRES,
                     Work& w, bool with_e0) {
  cross_coupled(B, R, hR, w.rcc.data());
  cross_coupled(B, L, hL, w.lcc.data());
  if (with_e0) RES[0] = comm110(B, L, hL, R, hR) + comm220(B, L, hL, R, hR);
  comm111(B, L, hL, R, hR, RES, hRES);
  comm121(B, L, hL, R, hR, RES, hRES);
  comm122(B, L, hL, R, hR, RES, hRES);
  comm222pphh(B, L, hL, R, hR, RES, hRES, w.w1.data(), w.w2.data());
  comm221(B, hL, hR, RES, hRES, w.w1.data(), w.w2.data());
  comm222ph(B, w.lcc.data(), hL, w.rcc.data(), hR, RES, hRES, w.wcc.data());
}

// mat_frob_norm (src/basic_IMSRG.f90:4056-4087)
double frob(const Basis& B, const double* op) {
  double sm = 0.0;
  for (int64_t k = 0; k < (int64_t)B.A * B.A; ++k) sm += op[B.off_fhh + k] * op[B.off_fhh + k];
  double s2 = 0.0;
  for (int64_t k = 0; k < (int64_t)B.P * B.A; ++k) s2 += op[B.off_fph + k] * op[B.off_fph + k];
  sm += 2 * s2;
  double s3 = 0.0;
  for (int64_t k = 0; k < (int64_t)B.P * B.P; ++k) s3 += op[B.off_fpp + k] * op[B.off_fpp + k];
  sm += s3;
  for (int q = 0; q < B.nblocks; ++q)
    for (int g = 0; g < 6; ++g) {
      const double* X = B.X(op, q, g);
      const int64_t n = (int64_t)B.gn1[q][g] * B.gn2[q][g];
      double s = 0.0;
      for (int64_t k = 0; k < n; ++k) s += X[k] * X[k];
      sm += s;
      if (!SQS[g]) sm += s;
    }
  return std::sqrt(sm);
}

// add_sq_op (src/basic_IMSRG.f90:3551-3579): C = ax*A + bx*B (whole operator incl. E0)
void add_op(const Basis& B, const double* A, double ax, const double* Bop, double bx, double* C) {
  for (int64_t k = 0; k < B.slab; ++k) C[k] = A[k] * ax + Bop[k] * bx;
}

// build_gs_white (src/generators.f90:4-106): ETA herm = -1
void white(const Basis& B, const double* H, int hH, double* ETA) {
  std::fill(ETA, ETA + B.slab, 0.0);
  for (int a = 0; a < B.P; ++a) {
    const int ak = B.parts[a];
    for (int i = 0; i < B.A; ++i) {
      const int ik = B.holes[i];
      if (B.jj[ik] != B.jj[ak] || B.ll[ik] != B.ll[ak] || B.tz[ik] != B.tz[ak]) continue;
      const int ji = B.jj[ik];
      double Eden = 0.0;
      for (int JT = 0; JT <= 2 * ji; JT += 2) Eden -= (JT + 1) * v_elem(B, H, hH, ak, ik, ak, ik, JT);
      Eden = Eden / (ji + 1.0) / (ji + 1.0);
      Eden = Eden + cfpp(B, H, a, a) - cfhh(B, H, i, i);
      fph(B, ETA, a, i) = cfph(B, H, a, i) / Eden;
    }
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int q = 0; q < B.nblocks; ++q) {
    const int np = B.ncls[q][0], nh = B.ncls[q][2];
    const double* HX = B.X(H, q, 2);
    double* EX = B.X(ETA, q, 2);
    for (int IX = 0; IX < np; ++IX) {
      const int a = B.qa[q][0][IX], b = B.qb[q][0][IX];
      for (int JX = 0; JX < nh; ++JX) {
        const int i = B.qa[q][2][JX], j = B.qb[q][2][JX];
        double Eden = 0.0;
        Eden += monopole(B, H, hH, a, b);
        Eden += monopole(B, H, hH, i, j);
        Eden -= monopole(B, H, hH, a, i);
        Eden -= monopole(B, H, hH, a, j);
        Eden -= monopole(B, H, hH, i, b);
        Eden -= monopole(B, H, hH, j, b);
        Eden += f_elem(B, H, hH, a, a) + f_elem(B, H, hH, b, b) - f_elem(B, H, hH, i, i) - f_elem(B, H, hH, j, j);
        EX[IX + (int64_t)JX * np] = HX[IX + (int64_t)JX * np] / Eden;
      }
    }
  }
}

// build_gs_atan / build_gs_atanxx (src/generators.f90:163-374): eta = atan(2 N / Eden) * 0.5
// with the White denominators of Hden and the numerators of Hnum (atan: both H)
void atan_gen(const Basis& B, const double* Hden, int hden, const double* Hnum, double* ETA) {
  std::fill(ETA, ETA + B.slab, 0.0);
  for (int a = 0; a < B.P; ++a) {
    const int ak = B.parts[a];
    for (int i = 0; i < B.A; ++i) {
      const int ik = B.holes[i];
      if (B.jj[ik] != B.jj[ak] || B.ll[ik] != B.ll[ak] || B.tz[ik] != B.tz[ak]) continue;
      const int ji = B.jj[ik];
      double Eden = 0.0;
      for (int JT = 0; JT <= 2 * ji; JT += 2) Eden -= (JT + 1) * v_elem(B, Hden, hden, ak, ik, ak, ik, JT);
      Eden = Eden / (ji + 1.0) / (ji + 1.0);
      Eden = Eden + cfpp(B, Hden, a, a) - cfhh(B, Hden, i, i);
      fph(B, ETA, a, i) = std::atan(2 * cfph(B, Hnum, a, i) / Eden) * 0.5;
    }
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int q = 0; q < B.nblocks; ++q) {
    const int np = B.ncls[q][0], nh = B.ncls[q][2];
    const double* HX = B.X(Hnum, q, 2);
    double* EX = B.X(ETA, q, 2);
    for (int IX = 0; IX < np; ++IX) {
      const int a = B.qa[q][0][IX], b = B.qb[q][0][IX];
      for (int JX = 0; JX < nh; ++JX) {
        const int i = B.qa[q][2][JX], j = B.qb[q][2][JX];
        double Eden = 0.0;
        Eden += monopole(B, Hden, hden, a, b);
        Eden += monopole(B, Hden, hden, i, j);
        Eden -= monopole(B, Hden, hden, a, i);
        Eden -= monopole(B, Hden, hden, a, j);
        Eden -= monopole(B, Hden, hden, i, b);
        Eden -= monopole(B, Hden, hden, j, b);
        Eden += f_elem(B, Hden, hden, a, a) + f_elem(B, Hden, hden, b, b) - f_elem(B, Hden, hden, i, i) -
                f_elem(B, Hden, hden, j, j);
        EX[IX + (int64_t)JX * np] = 0.5 * std::atan(2 * HX[IX + (int64_t)JX * np] / Eden);
      }
    }
  }
}

// mbpt2 (src/basic_IMSRG.f90:4165-4199)
double mbpt2(const Basis& B, const double* H, int hH) {
  double sm = 0.0;
  for (int q = 0; q < B.nblocks; ++q) {
    const int np = B.ncls[q][0], nh = B.ncls[q][2];
    const double* X = B.X(H, q, 2);
    double s1 = 0.0;
    for (int II = 0; II < np; ++II) {
      const int i = B.qa[q][0][II], j = B.qb[q][0][II];
      const double fi = f_elem(B, H, hH, i, i), fj = f_elem(B, H, hH, j, j);
      for (int JJ = 0; JJ < nh; ++JJ) {
        const int k = B.qa[q][2][JJ], l = B.qb[q][2][JJ];
        const double eden = f_elem(B, H, hH, k, k) + f_elem(B, H, hH, l, l) - fi - fj;
        const double v = X[II + (int64_t)JJ * np];
        s1 += v * v / eden;
      }
    }
    sm += (B.lamJ[q] + 1.0) * s1;
  }
  return sm;
}

// MAGNUS_EXPAND (src/IMSRG_MAGNUS.f90:620-691).  DG in: eta (herm -1); out: dOmega.
// G = Omega.  Returns number of nested commutators evaluated.
int magnus_expand(const Basis& B, double* DG, const double* G, Work& w) {
  const double conv = (double)1e-6f;   // default-real literal in the reference
  static const double cof[7] = {1.0, -0.5, .0833333333, 0.0, -0.00138888888, 0.0, 3.306878e-5};
  std::vector<double> INT1(B.slab), INT2(DG, DG + B.slab), AD(B.slab);
  double advals[8] = {0};
  advals[1] = frob(B, INT2.data());
  const double fullnorm = frob(B, G);
  if (fullnorm < (double)1e-9f) return 0;
  int qq = 1, used = 0;
  for (int i = 2; i <= 7; ++i) {
    std::copy(DG, DG + B.slab, INT1.begin());
    AD = INT2;
    const double adnorm = advals[i - qq];
    qq = (std::fabs(cof[i - 1]) > (double)1e-6f) ? 1 : 2;
    if (std::fabs(adnorm / fullnorm) < conv) break;
    full_commutator(B, G, -1, AD.data(), -1, INT2.data(), -1, w, false);
    ++used;
    add_op(B, INT1.data(), 1.0, INT2.data(), cof[i - 1], DG);
    advals[i] = frob(B, INT2.data()) * std::fabs(cof[i - 1]);
  }
  return used;
}

// BCH_EXPAND (src/IMSRG_MAGNUS.f90:149-234): HS = exp(G) H exp(-G).  Returns terms used,
// or -1 when the series did not converge within max_terms (the reference STOPs at 40).
// cr: CR_EXPAND (src/IMSRG_MAGNUS.f90:532-617), coef = coef/iw, no failure after max_terms
int bch_expand(const Basis& B, double* HS, const double* G, const double* H, int max_terms, double conv, Work& w,
               bool cr = false) {
  std::vector<double> INT1(B.slab), INT2(H, H + B.slab), AD(B.slab);
  std::copy(H, H + B.slab, HS);
  double coef = 1.0;
  int iw;
  for (iw = 2; iw <= max_terms; ++iw) {
    coef = cr ? coef / iw : coef / (iw - 1.0);
    std::copy(HS, HS + B.slab, INT1.begin());
    AD = INT2;
    std::fill(INT2.begin(), INT2.end(), 0.0);
    full_commutator(B, G, -1, AD.data(), 1, INT2.data(), 1, w, true);
    add_op(B, INT1.data(), 1.0, INT2.data(), coef, HS);
    if (frob(B, INT2.data()) * coef < conv) break;
  }
  if (cr) return (iw > max_terms) ? max_terms - 1 : iw - 1;
  return (iw > max_terms) ? -1 : iw - 1;
}

// ---------------------------------------------------------------- random operators
// construct_random_rank0 (src/brute_force_testing.f90:15-120) with this file's own RNG
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  double uni() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
  double x() { return 10.0 * uni() - 5.0; }
};

void random_op(const Basis& B, uint64_t seed, int herm, double* op) {
  Rng rng(seed);
  std::fill(op, op + B.slab, 0.0);
  auto same = [&](int x, int y) { return B.jj[x] == B.jj[y] && B.ll[x] == B.ll[y] && B.tz[x] == B.tz[y]; };
  for (int ig = 0; ig < B.A; ++ig) {
    for (int jg = ig; jg < B.A; ++jg) {
      if (!same(B.holes[ig], B.holes[jg])) continue;
      const double x = rng.x();
      fhh(B, op, ig, jg) = x;
      fhh(B, op, jg, ig) = herm * x;
    }
    fhh(B, op, ig, ig) = (herm + 1) * fhh(B, op, ig, ig) / 2.0;
  }
  for (int ig = 0; ig < B.P; ++ig)
    for (int jg = 0; jg < B.A; ++jg) {
      if (!same(B.parts[ig], B.holes[jg])) continue;
      fph(B, op, ig, jg) = rng.x();
    }
  for (int ig = 0; ig < B.P; ++ig) {
    for (int jg = ig; jg < B.P; ++jg) {
      if (!same(B.parts[ig], B.parts[jg])) continue;
      const double x = rng.x();
      fpp(B, op, ig, jg) = x;
      fpp(B, op, jg, ig) = herm * x;
    }
    fpp(B, op, ig, ig) = (herm + 1) * fpp(B, op, ig, ig) / 2.0;
  }
  for (int q = 0; q < B.nblocks; ++q) {
    const bool oddJ = ((B.lamJ[q] / 2) % 2) == 1;
    for (int g = 0; g < 6; ++g) {
      const int n1 = B.gn1[q][g], n2 = B.gn2[q][g];
      double* X = B.X(op, q, g);
      for (int IX = 0; IX < n1; ++IX)
        for (int JX = SQS[g] ? IX : 0; JX < n2; ++JX) {
          double x = rng.x();
          if (B.qa[q][SEA1[g]][IX] == B.qb[q][SEA1[g]][IX] && oddJ) x = 0.0;
          if (B.qa[q][SEA2[g]][JX] == B.qb[q][SEA2[g]][JX] && oddJ) x = 0.0;
          X[IX + (int64_t)JX * n1] = x * (1 + herm * kd(IX, JX) * (SQS[g] ? 1 : 0));
          if (SQS[g]) X[JX + (int64_t)IX * n1] = herm * X[IX + (int64_t)JX * n1];
        }
    }
  }
}

// ---------------------------------------------------------------- brute force (known answers)
// scalar_scalar_0body_comm (src/brute_force_testing.f90:1887-1928)
double bf0(const Basis& B, const double* A, int hA, const double* Bo, int hB) {
  const int T = B.N, JTM = B.JM * 2;
  double sm = 0.0;
  for (int i = 0; i < T; ++i)
    for (int j = 0; j < T; ++j)
      sm += (B.con[i] - B.con[j]) * (B.jj[i] + 1.0) * f_elem(B, A, hA, i, j) * f_elem(B, Bo, hB, j, i);
  for (int i = 0; i < T; ++i)
    for (int j = 0; j < T; ++j)
      for (int k = 0; k < T; ++k)
        for (int l = 0; l < T; ++l) {
          const int w = B.con[i] * B.con[j] * (1 - B.con[k]) * (1 - B.con[l]) -
                        B.con[k] * B.con[l] * (1 - B.con[i]) * (1 - B.con[j]);
          if (!w) continue;
          for (int J = 0; J <= JTM; J += 2)
            sm += w * (J + 1.0) * v_elem(B, A, hA, i, j, k, l, J) * v_elem(B, Bo, hB, k, l, i, j, J) / 4.0;
        }
  return sm;
}

// scalar_scalar_1body_comm (src/brute_force_testing.f90:1765-1823)
double bf1(const Basis& B, const double* A, int hA, const double* Bo, int hB, int a, int b) {
  const int T = B.N, JTM = B.JM * 2;
  const int ja = B.jj[a], jb = B.jj[b];
  double sm = 0.0;
  for (int i = 0; i < T; ++i)
    sm += f_elem(B, A, hA, a, i) * f_elem(B, Bo, hB, i, b) - f_elem(B, Bo, hB, a, i) * f_elem(B, A, hA, i, b);
  if (ja == jb) {
    for (int i = 0; i < T; ++i)
      for (int j = 0; j < T; ++j) {
        const int w = B.con[i] - B.con[j];
        if (!w) continue;
        for (int J = 0; J <= JTM; J += 2)
          sm += w * (J + 1.0) / (ja + 1.0) *
                (f_elem(B, A, hA, i, j) * v_elem(B, Bo, hB, j, a, i, b, J) -
                 f_elem(B, Bo, hB, i, j) * v_elem(B, A, hA, j, a, i, b, J));
      }
    for (int i = 0; i < T; ++i)
      for (int j = 0; j < T; ++j)
        for (int k = 0; k < T; ++k) {
          const int w = B.con[i] * B.con[j] * (1 - B.con[k]) + (1 - B.con[i]) * (1 - B.con[j]) * B.con[k];
          if (!w) continue;
          for (int J = 0; J <= JTM; J += 2)
            sm += w * (J + 1.0) / (ja + 1.0) *
                  (v_elem(B, A, hA, a, k, i, j, J) * v_elem(B, Bo, hB, i, j, b, k, J) -
                   v_elem(B, Bo, hB, a, k, i, j, J) * v_elem(B, A, hA, i, j, b, k, J)) / 2.0;
        }
  }
  return sm;
}

// scalar_scalar_2body_comm (src/brute_force_testing.f90:1975-2076)
double bf2(const Basis& B, const double* A, int hA, const double* Bo, int hB, int a, int b, int c, int d, int Jtot) {
  const int T = B.N, JTM = B.JM * 2;
  const int ja = B.jj[a], jb = B.jj[b], jc = B.jj[c], jd = B.jj[d];
  const AngMom& am = angmom();
  double sm = 0.0;
  for (int i = 0; i < T; ++i) {
    sm += f_elem(B, A, hA, a, i) * v_elem(B, Bo, hB, i, b, c, d, Jtot) +
          f_elem(B, A, hA, b, i) * v_elem(B, Bo, hB, a, i, c, d, Jtot) -
          f_elem(B, A, hA, i, c) * v_elem(B, Bo, hB, a, b, i, d, Jtot) -
          f_elem(B, A, hA, i, d) * v_elem(B, Bo, hB, a, b, c, i, Jtot);
    sm = sm - f_elem(B, Bo, hB, a, i) * v_elem(B, A, hA, i, b, c, d, Jtot) -
         f_elem(B, Bo, hB, b, i) * v_elem(B, A, hA, a, i, c, d, Jtot) +
         f_elem(B, Bo, hB, i, c) * v_elem(B, A, hA, a, b, i, d, Jtot) +
         f_elem(B, Bo, hB, i, d) * v_elem(B, A, hA, a, b, c, i, Jtot);
  }
  for (int i = 0; i < T; ++i)
    for (int j = 0; j < T; ++j)
      sm += 0.5 * (1 - B.con[i] - B.con[j]) *
            (v_elem(B, A, hA, a, b, i, j, Jtot) * v_elem(B, Bo, hB, i, j, c, d, Jtot) -
             v_elem(B, Bo, hB, a, b, i, j, Jtot) * v_elem(B, A, hA, i, j, c, d, Jtot));
  for (int i = 0; i < T; ++i) {
    const int ji = B.jj[i];
    for (int j = 0; j < T; ++j) {
      const int jj = B.jj[j];
      const int w = B.con[i] - B.con[j];
      if (w == 0) continue;
      for (int J1 = 0; J1 <= JTM; J1 += 2)
        for (int J2 = 0; J2 <= JTM; J2 += 2) {
          const double f = (J1 + 1.0) * (J2 + 1.0);
          double t = 0.0;
          t += sgn((J1 + J2 + ja - jc) / 2) * f * am.ninej(jj, J1, ja, J2, ji, jb, jc, jd, Jtot) *
               v_elem(B, A, hA, j, a, i, d, J1) * v_elem(B, Bo, hB, i, b, j, c, J2);
          t -= sgn((J1 + J2 + jb - jc) / 2) * f * am.ninej(jj, J1, jb, J2, ji, ja, jc, jd, Jtot) *
               v_elem(B, A, hA, j, b, i, d, J1) * v_elem(B, Bo, hB, i, a, j, c, J2) * sgn((ja + jb - Jtot) / 2);
          t -= sgn((J1 + J2 + ja - jd) / 2) * f * am.ninej(jj, J1, ja, J2, ji, jb, jd, jc, Jtot) *
               v_elem(B, A, hA, j, a, i, c, J1) * v_elem(B, Bo, hB, i, b, j, d, J2) * sgn((jc + jd - Jtot) / 2);
          t += sgn((J1 + J2 + jb - jd) / 2) * f * am.ninej(jj, J1, jb, J2, ji, ja, jd, jc, Jtot) *
               v_elem(B, A, hA, j, b, i, c, J1) * v_elem(B, Bo, hB, i, a, j, d, J2) * sgn((ja + jb + jc + jd) / 2);
          sm += w * t;
        }
    }
  }
  return sm;
}

}  // namespace

// ====================================================================== reverse mode
// Exact transposes (vector-Jacobian products) of the forward routines above, used to
// check the device adjoint of the Magnus flow (dE0/dtheta).  The reference has no
// derivative code: each routine below is the reverse of this file's own restatement,
// statement by statement, so <Cbar, F(L, R)> = <Lbar, L> = <Rbar, R> holds for the
// bilinear pieces on ANY slabs (hermitian or not), which is what the tests check.

struct Addr {
  int64_t idx;  // slab index read by f_elem / v_elem (-1: the element is identically zero)
  double c;     // value read = c * slab[idx]
};

inline Addr f_addr(const Basis& B, int herm, int a, int b) {
  const int c1 = B.con[a], c2 = B.con[b];
  switch (c1 + c2) {
    case 0: return {B.off_fpp + B.loc[a] + (int64_t)B.loc[b] * B.P, 1.0};
    case 1:
      if (c1 > c2) return {B.off_fph + B.loc[b] + (int64_t)B.loc[a] * B.P, (double)herm};
      return {B.off_fph + B.loc[a] + (int64_t)B.loc[b] * B.P, 1.0};
    default: return {B.off_fhh + B.loc[a] + (int64_t)B.loc[b] * B.A, 1.0};
  }
}

// the slab position v_elem reads, with its factor (same branches as v_elem)
Addr v_addr(const Basis& B, int herm, int a, int b, int c, int d, int J) {
  const int ja = B.jj[a], jb = B.jj[b], jc = B.jj[c], jd = B.jj[d];
  if (!(tri(ja, jb, J) && tri(jc, jd, J))) return {-1, 0.0};
  const int P = (B.ll[a] + B.ll[b]) % 2;
  if ((B.ll[c] + B.ll[d]) % 2 != P) return {-1, 0.0};
  const int T = (B.tz[a] + B.tz[b]) / 2;
  if (B.tz[c] + B.tz[d] != 2 * T) return {-1, 0.0};
  const int q = B.block(J, T, P);
  const int C1 = B.con[a] + B.con[b], C2 = B.con[c] + B.con[d];
  const int g = qx_of(std::min(C1, C2), std::max(C1, C2));
  double pre = 1.0;
  const int N = B.N, NJ = B.NJ;
  int i1, i2;
  if (a > b) {
    i1 = B.pairpos[((size_t)b * N + a) * NJ + J / 2];
    pre = sgn(1 + (ja + jb - J) / 2);
  } else {
    if (a == b) pre *= std::sqrt(2.0);
    i1 = B.pairpos[((size_t)a * N + b) * NJ + J / 2];
  }
  if (c > d) {
    i2 = B.pairpos[((size_t)d * N + c) * NJ + J / 2];
    pre *= sgn(1 + (jc + jd - J) / 2);
  } else {
    if (c == d) pre *= std::sqrt(2.0);
    i2 = B.pairpos[((size_t)c * N + d) * NJ + J / 2];
  }
  const int n1 = B.gn1[q][g];
  if (C1 > C2) return {B.goff[q][g] + i2 + (int64_t)i1 * n1, herm * pre};
  return {B.goff[q][g] + i1 + (int64_t)i2 * n1, pre};
}

inline void add_at(double* bar, const Addr& ad, double g) {
  if (ad.idx >= 0) bar[ad.idx] += ad.c * g;
}
inline double val_at(const double* op, const Addr& ad) { return ad.idx >= 0 ? ad.c * op[ad.idx] : 0.0; }

// Reverse of a square-array write "X(i,j) (+)= s; X(j,i) = X(i,j) * h" (i <= j) on the
// running cotangent cb of X.  Returns the cotangent of s.  accumulate: the old X(i,j)
// keeps a cotangent (it was added to); assign: the old values are overwritten.
inline double fold_square(double* cb, int64_t ij, int64_t ji, bool diag, int h, bool accumulate) {
  const double g = diag ? h * cb[ij] : cb[ij] + h * cb[ji];
  cb[ij] = accumulate ? g : 0.0;
  if (!diag) cb[ji] = 0.0;
  return g;
}

// commutator_110 / commutator_220: d E0 / d(L, R) times ebar
void comm110_vjp(const Basis& B, const double* L, int hL, const double* R, int hR, double ebar, double* Lb,
                 double* Rb) {
  for (int i = 0; i < B.A; ++i) {
    const double w = ebar * (hL - hR) * (B.jj[B.holes[i]] + 1);
    for (int a = 0; a < B.P; ++a) {
      const int64_t k = B.off_fph + a + (int64_t)i * B.P;
      Lb[k] += w * R[k];
      Rb[k] += w * L[k];
    }
  }
}

void comm220_vjp(const Basis& B, const double* L, int hL, const double* R, int hR, double ebar, double* Lb,
                 double* Rb) {
  if (hR * hL != -1) return;
  for (int q = 0; q < B.nblocks; ++q) {
    const int64_t n = (int64_t)B.ncls[q][0] * B.ncls[q][2];
    const double w = -2.0 * hR * (B.lamJ[q] + 1) * ebar;
    const int64_t o = B.goff[q][2];
    for (int64_t k = 0; k < n; ++k) {
      Lb[o + k] += w * R[o + k];
      Rb[o + k] += w * L[o + k];
    }
  }
}

// commutator_111: every one-body element of RES is assigned
void comm111_vjp(const Basis& B, const double* L, int hL, const double* R, int hR, double* cb, double* Lb,
                 double* Rb) {
  const int A = B.A, P = B.P;
  const double *Lhh = L + B.off_fhh, *Rhh = R + B.off_fhh, *Lph = L + B.off_fph, *Rph = R + B.off_fph;
  const double *Lpp = L + B.off_fpp, *Rpp = R + B.off_fpp;
  double *Lhhb = Lb + B.off_fhh, *Rhhb = Rb + B.off_fhh, *Lphb = Lb + B.off_fph, *Rphb = Rb + B.off_fph;
  double *Lppb = Lb + B.off_fpp, *Rppb = Rb + B.off_fpp;
  const double* Chh = cb + B.off_fhh;
  const double* Cph = cb + B.off_fph;
  const double* Cpp = cb + B.off_fpp;
  std::vector<double> t1((size_t)std::max(A * A, P * P)), t2((size_t)std::max(A * A, P * P));
  // fhh = th1 + hL th2 - hR (hL th1^T + th2^T), th1 = Lhh Rhh, th2 = Lph^T Rph
  for (int j = 0; j < A; ++j)
    for (int i = 0; i < A; ++i) {
      t1[i + j * A] = Chh[i + j * A] - hL * hR * Chh[j + i * A];
      t2[i + j * A] = hL * Chh[i + j * A] - hR * Chh[j + i * A];
    }
  if (A) {
    dgemm('N', 'T', A, A, A, 1.0, t1.data(), A, Rhh, A, 1.0, Lhhb, A);
    dgemm('T', 'N', A, A, A, 1.0, Lhh, A, t1.data(), A, 1.0, Rhhb, A);
    if (P) {
      dgemm('N', 'T', P, A, A, 1.0, Rph, P, t2.data(), A, 1.0, Lphb, P);
      dgemm('N', 'N', P, A, A, 1.0, Lph, P, t2.data(), A, 1.0, Rphb, P);
    }
  }
  // fph = Lph Rhh + Lpp Rph - Rph Lhh - Rpp Lph
  if (P && A) {
    dgemm('N', 'T', P, A, A, 1.0, Cph, P, Rhh, A, 1.0, Lphb, P);
    dgemm('T', 'N', A, A, P, 1.0, Lph, P, Cph, P, 1.0, Rhhb, A);
    dgemm('N', 'T', P, P, A, 1.0, Cph, P, Rph, P, 1.0, Lppb, P);
    dgemm('T', 'N', P, A, P, 1.0, Lpp, P, Cph, P, 1.0, Rphb, P);
    dgemm('N', 'T', P, A, A, -1.0, Cph, P, Lhh, A, 1.0, Rphb, P);
    dgemm('T', 'N', A, A, P, -1.0, Rph, P, Cph, P, 1.0, Lhhb, A);
    dgemm('N', 'T', P, P, A, -1.0, Cph, P, Lph, P, 1.0, Rppb, P);
    dgemm('T', 'N', P, A, P, -1.0, Rpp, P, Cph, P, 1.0, Lphb, P);
  }
  // fpp = hR tp1 + tp2 - hL (tp1^T + hR tp2^T), tp1 = Lph Rph^T, tp2 = Lpp Rpp
  for (int j = 0; j < P; ++j)
    for (int i = 0; i < P; ++i) {
      t1[i + (size_t)j * P] = hR * Cpp[i + (size_t)j * P] - hL * Cpp[j + (size_t)i * P];
      t2[i + (size_t)j * P] = Cpp[i + (size_t)j * P] - hL * hR * Cpp[j + (size_t)i * P];
    }
  if (P) {
    if (A) {
      dgemm('N', 'N', P, A, P, 1.0, t1.data(), P, Rph, P, 1.0, Lphb, P);
      dgemm('T', 'N', P, A, P, 1.0, t1.data(), P, Lph, P, 1.0, Rphb, P);
    }
    dgemm('N', 'T', P, P, P, 1.0, t2.data(), P, Rpp, P, 1.0, Lppb, P);
    dgemm('T', 'N', P, P, P, 1.0, Lpp, P, t2.data(), P, 1.0, Rppb, P);
  }
  std::fill(cb + B.off_fhh, cb + B.off_fph + (int64_t)P * A, 0.0);
}

// commutator_121: one-body outputs accumulate (hh / pp squares then mirrored)
void comm121_vjp(const Basis& B, const double* L, int hL, const double* R, int hR, int hRES, double* cb,
                 double* Lb, double* Rb) {
  auto inner_vjp = [&](int pk, int qk, double sbar) {
    const int jq = B.jj[qk];
    for (int a = 0; a < B.P; ++a) {
      const int ak = B.parts[a];
      for (int i = 0; i < B.A; ++i) {
        const int ik = B.holes[i];
        if (B.jj[ik] != B.jj[ak] || B.ll[ik] != B.ll[ak] || B.tz[ik] != B.tz[ak]) continue;
        const int ji = B.jj[ik];
        const int64_t ph = B.off_fph + a + (int64_t)i * B.P;
        const double lai = L[ph], rai = R[ph];
        double smx = 0, smy = 0, smx2 = 0, smy2 = 0;
        for (int JT = std::abs(ji - jq); JT <= ji + jq; JT += 2) {
          const Addr rx = v_addr(B, hR, ak, pk, ik, qk, JT), ry = v_addr(B, hR, ik, pk, ak, qk, JT);
          const Addr lx = v_addr(B, hL, ak, pk, ik, qk, JT), ly = v_addr(B, hL, ik, pk, ak, qk, JT);
          smx += val_at(R, rx) * (JT + 1);
          smy += val_at(R, ry) * (JT + 1);
          smx2 += val_at(L, lx) * (JT + 1);
          smy2 += val_at(L, ly) * (JT + 1);
          add_at(Rb, rx, sbar * lai * hL * (JT + 1));
          add_at(Rb, ry, -sbar * lai * (JT + 1));
          add_at(Lb, lx, -sbar * rai * hR * (JT + 1));
          add_at(Lb, ly, sbar * rai * (JT + 1));
        }
        Lb[ph] += sbar * (hL * smx - smy);
        Rb[ph] -= sbar * (hR * smx2 - smy2);
      }
    }
  };
  auto same = [&](int x, int y) { return B.jj[x] == B.jj[y] && B.ll[x] == B.ll[y] && B.tz[x] == B.tz[y]; };
  for (int p = 0; p < B.A; ++p)
    for (int q = p; q < B.A; ++q) {
      const int pk = B.holes[p], qk = B.holes[q];
      if (!same(pk, qk)) continue;
      const double g = fold_square(cb, B.off_fhh + p + (int64_t)q * B.A, B.off_fhh + q + (int64_t)p * B.A, p == q,
                                   hRES, true);
      inner_vjp(pk, qk, g / (B.jj[pk] + 1.0));
    }
  for (int p = 0; p < B.P; ++p)
    for (int q = p; q < B.P; ++q) {
      const int pk = B.parts[p], qk = B.parts[q];
      if (!same(pk, qk)) continue;
      const double g = fold_square(cb, B.off_fpp + p + (int64_t)q * B.P, B.off_fpp + q + (int64_t)p * B.P, p == q,
                                   hRES, true);
      inner_vjp(pk, qk, g / (B.jj[pk] + 1.0));
    }
  for (int p = 0; p < B.P; ++p)
    for (int q = 0; q < B.A; ++q) {
      const int pk = B.parts[p], qk = B.holes[q];
      if (!same(pk, qk)) continue;
      inner_vjp(pk, qk, cb[B.off_fph + p + (int64_t)q * B.P] / (B.jj[pk] + 1.0));
    }
}

// commutator_122: every two-body element is assigned
void comm122_vjp(const Basis& B, const double* L, int hL, const double* R, int hR, int hRES, double* cb,
                 double* Lb, double* Rb) {
  for (int q = 0; q < B.nblocks; ++q) {
    const int JT = B.lamJ[q];
    for (int g = 0; g < 6; ++g) {
      const int n1 = B.gn1[q][g], n2 = B.gn2[q][g];
      if (n1 * n2 == 0) continue;
      const int c1 = SEA1[g], c2 = SEA2[g];
      const int64_t o = B.goff[q][g];
      for (int IX = 0; IX < n1; ++IX) {
        const int a = B.qa[q][c1][IX], b = B.qb[q][c1][IX];
        for (int JX = SQS[g] ? IX : 0; JX < n2; ++JX) {
          const int c = B.qa[q][c2][JX], d = B.qb[q][c2][JX];
          const int64_t ij = o + IX + (int64_t)JX * n1, ji = o + JX + (int64_t)IX * n1;
          double s;
          if (SQS[g]) {
            s = fold_square(cb, ij, ji, IX == JX, hRES, false);
          } else {
            s = cb[ij];
            cb[ij] = 0.0;
          }
          s = s / std::sqrt(1.0 + kd(a, b)) / std::sqrt(1.0 + kd(c, d));
          if (s == 0.0) continue;
          // each term sm += X * Y contributes Xbar += s * Y, Ybar += s * X
          auto term = [&](const Addr& fL, const Addr& vR, const Addr& fR, const Addr& vL, double sign) {
            add_at(Lb, fL, sign * s * val_at(R, vR));
            add_at(Rb, vR, sign * s * val_at(L, fL));
            add_at(Rb, fR, -sign * s * val_at(L, vL));
            add_at(Lb, vL, -sign * s * val_at(R, fR));
          };
          for (int i : B.same[a])
            term(f_addr(B, hL, a, i), v_addr(B, hR, i, b, c, d, JT), f_addr(B, hR, a, i),
                 v_addr(B, hL, i, b, c, d, JT), 1.0);
          for (int i : B.same[b])
            term(f_addr(B, hL, b, i), v_addr(B, hR, a, i, c, d, JT), f_addr(B, hR, b, i),
                 v_addr(B, hL, a, i, c, d, JT), 1.0);
          for (int i : B.same[c])
            term(f_addr(B, hL, i, c), v_addr(B, hR, a, b, i, d, JT), f_addr(B, hR, i, c),
                 v_addr(B, hL, a, b, i, d, JT), -1.0);
          for (int i : B.same[d])
            term(f_addr(B, hL, i, d), v_addr(B, hR, a, b, c, i, JT), f_addr(B, hR, i, d),
                 v_addr(B, hL, a, b, c, i, JT), -1.0);
        }
      }
    }
  }
}

// commutator_222_pp_hh: RES accumulates W1 - W2 combinations (cb passes through); w1b, w2b
// carry the cotangents of the w1 / w2 workspaces from commutator_221
void comm222pphh_vjp(const Basis& B, const double* L, int hL, const double* R, int hR, const double* cb,
                     const double* w1b, const double* w2b, double* Lb, double* Rb) {
  const double pm = hR * hL;
  for (int q = 0; q < B.nblocks; ++q) {
    const int np = B.ncls[q][0], nb = B.ncls[q][1], nh = B.ncls[q][2];
    auto blk = [&](const double* op, int g) { return B.X(op, q, g); };
    auto blkw = [&](double* op, int g) { return B.X(op, q, g); };
    const double *L1 = blk(L, 0), *L2 = blk(L, 1), *L3 = blk(L, 2), *L5 = blk(L, 4), *L6 = blk(L, 5);
    const double *R1 = blk(R, 0), *R2 = blk(R, 1), *R3 = blk(R, 2), *R5 = blk(R, 4), *R6 = blk(R, 5);
    double *L1b = blkw(Lb, 0), *L2b = blkw(Lb, 1), *L3b = blkw(Lb, 2), *L5b = blkw(Lb, 4), *L6b = blkw(Lb, 5);
    double *R1b = blkw(Rb, 0), *R2b = blkw(Rb, 1), *R3b = blkw(Rb, 2), *R5b = blkw(Rb, 4), *R6b = blkw(Rb, 5);
    // cotangents of the twelve W blocks
    std::vector<double> W1[6], W2[6];
    for (int g = 0; g < 6; ++g) {
      const int64_t n = (int64_t)B.gn1[q][g] * B.gn2[q][g];
      W1[g].assign(blk(w1b, g), blk(w1b, g) + n);
      W2[g].assign(blk(w2b, g), blk(w2b, g) + n);
    }
    auto antisym = [&](int g, int n) {
      const double* C = blk(cb, g);
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
          const double v = C[i + (int64_t)j * n] - pm * C[j + (int64_t)i * n];
          W1[g][i + (int64_t)j * n] += v;
          W2[g][i + (int64_t)j * n] -= v;
        }
    };
    auto plain = [&](int g) {
      const double* C = blk(cb, g);
      const int64_t n = (int64_t)B.gn1[q][g] * B.gn2[q][g];
      for (int64_t k = 0; k < n; ++k) {
        W1[g][k] += C[k];
        W2[g][k] -= C[k];
      }
    };
    antisym(0, np);
    antisym(4, nh);
    antisym(3, nb);
    plain(2);
    plain(5);
    plain(1);
    const double *W11 = W1[0].data(), *W12 = W1[1].data(), *W13 = W1[2].data(), *W14 = W1[3].data(),
                 *W15 = W1[4].data(), *W16 = W1[5].data();
    const double *W21 = W2[0].data(), *W22 = W2[1].data(), *W23 = W2[2].data(), *W24 = W2[3].data(),
                 *W25 = W2[4].data(), *W26 = W2[5].data();
    if (np != 0) {  // W11 = L1 R1
      dgemm('N', 'T', np, np, np, 1.0, W11, np, R1, np, 1.0, L1b, np);
      dgemm('T', 'N', np, np, np, 1.0, L1, np, W11, np, 1.0, R1b, np);
    }
    if (nh != 0) {  // W25 = L5 R5
      dgemm('N', 'T', nh, nh, nh, 1.0, W25, nh, R5, nh, 1.0, L5b, nh);
      dgemm('T', 'N', nh, nh, nh, 1.0, L5, nh, W25, nh, 1.0, R5b, nh);
    }
    if (np * nh != 0) {
      // W15 = hL L3^T R3
      dgemm('N', 'T', np, nh, nh, 1.0 * hL, R3, np, W15, nh, 1.0, L3b, np);
      dgemm('N', 'N', np, nh, nh, 1.0 * hL, L3, np, W15, nh, 1.0, R3b, np);
      // W21 = hR L3 R3^T
      dgemm('N', 'N', np, nh, np, 1.0 * hR, W21, np, R3, np, 1.0, L3b, np);
      dgemm('T', 'N', np, nh, np, 1.0 * hR, W21, np, L3, np, 1.0, R3b, np);
      // W13 = L1 R3 - R1 L3
      dgemm('N', 'T', np, np, nh, 1.0, W13, np, R3, np, 1.0, L1b, np);
      dgemm('T', 'N', np, nh, np, 1.0, L1, np, W13, np, 1.0, R3b, np);
      dgemm('N', 'T', np, np, nh, -1.0, W13, np, L3, np, 1.0, R1b, np);
      dgemm('T', 'N', np, nh, np, -1.0, R1, np, W13, np, 1.0, L3b, np);
      // W23 = L3 R5 - R3 L5
      dgemm('N', 'T', np, nh, nh, 1.0, W23, np, R5, nh, 1.0, L3b, np);
      dgemm('T', 'N', nh, nh, np, 1.0, L3, np, W23, np, 1.0, R5b, nh);
      dgemm('N', 'T', np, nh, nh, -1.0, W23, np, L5, nh, 1.0, R3b, np);
      dgemm('T', 'N', nh, nh, np, -1.0, R3, np, W23, np, 1.0, L5b, nh);
    }
    if (nb * nh != 0) {  // W24 = hR L6 R6^T
      dgemm('N', 'N', nb, nh, nb, 1.0 * hR, W24, nb, R6, nb, 1.0, L6b, nb);
      dgemm('T', 'N', nb, nh, nb, 1.0 * hR, W24, nb, L6, nb, 1.0, R6b, nb);
    }
    if (nb * np != 0) {  // W14 = hL L2^T R2
      dgemm('N', 'T', np, nb, nb, 1.0 * hL, R2, np, W14, nb, 1.0, L2b, np);
      dgemm('N', 'N', np, nb, nb, 1.0 * hL, L2, np, W14, nb, 1.0, R2b, np);
    }
    if (nb * nh != 0) {  // W26 = L6 R5 - R6 L5
      dgemm('N', 'T', nb, nh, nh, 1.0, W26, nb, R5, nh, 1.0, L6b, nb);
      dgemm('T', 'N', nh, nh, nb, 1.0, L6, nb, W26, nb, 1.0, R5b, nh);
      dgemm('N', 'T', nb, nh, nh, -1.0, W26, nb, L5, nh, 1.0, R6b, nb);
      dgemm('T', 'N', nh, nh, nb, -1.0, R6, nb, W26, nb, 1.0, L5b, nh);
    }
    if (nb * np != 0) {  // W12 = L1 R2 - R1 L2
      dgemm('N', 'T', np, np, nb, 1.0, W12, np, R2, np, 1.0, L1b, np);
      dgemm('T', 'N', np, nb, np, 1.0, L1, np, W12, np, 1.0, R2b, np);
      dgemm('N', 'T', np, np, nb, -1.0, W12, np, L2, np, 1.0, R1b, np);
      dgemm('T', 'N', np, nb, np, -1.0, R1, np, W12, np, 1.0, L2b, np);
    }
    if (nb * np * nh != 0) {
      // W16 = hL L2^T R3 - hR R2^T L3
      dgemm('N', 'T', np, nb, nh, 1.0 * hL, R3, np, W16, nb, 1.0, L2b, np);
      dgemm('N', 'N', np, nh, nb, 1.0 * hL, L2, np, W16, nb, 1.0, R3b, np);
      dgemm('N', 'T', np, nb, nh, -1.0 * hR, L3, np, W16, nb, 1.0, R2b, np);
      dgemm('N', 'N', np, nh, nb, -1.0 * hR, R2, np, W16, nb, 1.0, L3b, np);
      // W22 = hR L3 R6^T - hL R3 L6^T
      dgemm('N', 'N', np, nh, nb, 1.0 * hR, W22, np, R6, nb, 1.0, L3b, np);
      dgemm('T', 'N', nb, nh, np, 1.0 * hR, W22, np, L3, np, 1.0, R6b, nb);
      dgemm('N', 'N', np, nh, nb, -1.0 * hL, W22, np, L6, nb, 1.0, R3b, np);
      dgemm('T', 'N', nb, nh, np, -1.0 * hL, W22, np, R3, np, 1.0, L6b, nb);
    }
  }
}

// commutator_221: one-body outputs accumulate traces of w1 (hole c) and w2 (particle c)
void comm221_vjp(const Basis& B, int hL, int hR, int hRES, double* cb, double* w1b, double* w2b) {
  const int pm = hR * hL;
  auto same = [&](int x, int y) { return B.jj[x] == B.jj[y] && B.ll[x] == B.ll[y] && B.tz[x] == B.tz[y]; };
  auto trace_vjp = [&](int ik, int jk, bool antisym, double tb) {
    const int ji = B.jj[ik];
    for (int side = 0; side < 2; ++side) {
      const std::vector<int>& cs = side == 0 ? B.holes : B.parts;
      double* wb = side == 0 ? w1b : w2b;
      for (int ck : cs) {
        const int jc = B.jj[ck];
        for (int JT = std::abs(jc - ji); JT <= jc + ji; JT += 2) {
          add_at(wb, v_addr(B, 1, ck, ik, ck, jk, JT), tb * (JT + 1));
          if (antisym) add_at(wb, v_addr(B, 1, ck, jk, ck, ik, JT), -pm * tb * (JT + 1));
        }
      }
    }
  };
  for (int i = 0; i < B.A; ++i)
    for (int j = i; j < B.A; ++j) {
      const int ik = B.holes[i], jk = B.holes[j];
      if (!same(ik, jk)) continue;
      const double g = fold_square(cb, B.off_fhh + i + (int64_t)j * B.A, B.off_fhh + j + (int64_t)i * B.A, i == j,
                                   hRES, true);
      trace_vjp(ik, jk, true, g / (B.jj[ik] + 1.0));
    }
  for (int i = 0; i < B.P; ++i)
    for (int j = i; j < B.P; ++j) {
      const int ik = B.parts[i], jk = B.parts[j];
      if (!same(ik, jk)) continue;
      const double g = fold_square(cb, B.off_fpp + i + (int64_t)j * B.P, B.off_fpp + j + (int64_t)i * B.P, i == j,
                                   hRES, true);
      trace_vjp(ik, jk, true, g / (B.jj[ik] + 1.0));
    }
  for (int i = 0; i < B.P; ++i)
    for (int j = 0; j < B.A; ++j) {
      const int ik = B.parts[i], jk = B.holes[j];
      if (!same(ik, jk)) continue;
      trace_vjp(ik, jk, false, cb[B.off_fph + i + (int64_t)j * B.P] / (B.jj[ik] + 1.0));
    }
}

// calculate_cross_coupled: every CC element is assigned from v_elem values of op
void cross_coupled_vjp(const Basis& B, int herm, const double* ccb, double* opb) {
  for (int q1 = 0; q1 < B.ncc; ++q1) {
    const int JC = B.cc_J[q1];
    const int rlen = B.cc_rlen[q1];
    const double* CC = ccb + B.cc_off[q1];
    for (int nbx = 0; nbx < B.cc_nph[q1]; ++nbx) {
      const int p = B.cc_php[q1][nbx], h = B.cc_phh[q1][nbx];
      const int jp = B.jj[p], jh = B.jj[h], lp = B.ll[p], lh = B.ll[h], tp = B.tz[p], th = B.tz[h];
      for (int r = 0; r < rlen; ++r) {
        const int a = B.cc_pa[q1][r], b = B.cc_pb[q1][r];
        const int ja = B.jj[a], jb = B.jj[b], la = B.ll[a], lb = B.ll[b], ta = B.tz[a], tb = B.tz[b];
        if (!(((la + lh) % 2 == (lb + lp) % 2) && (ta + th == tb + tp))) continue;
        const double g = CC[r + (int64_t)nbx * rlen] * sgn((jh + jb + JC) / 2) * std::sqrt(JC + 1.0);
        if (g == 0.0) continue;
        const int Jmin = std::max(std::abs(jp - jb), std::abs(ja - jh));
        const int Jmax = std::min(jp + jb, ja + jh);
        for (int JT = Jmin; JT <= Jmax; JT += 2)
          add_at(opb, v_addr(B, herm, h, a, p, b, JT), g * sgn(JT / 2) * (JT + 1) * sixj(jp, jh, JC, ja, jb, JT));
      }
    }
  }
}

// commutator_222_ph: WCC = LCC RCC^T, then the recoupled WCC accumulates into RES
void comm222ph_vjp(const Basis& B, const double* LCC, int hL, const double* RCC, int hR, int hRES, double* cb,
                   double* LCCb, double* RCCb) {
  std::vector<double> Wb(std::max<int64_t>(B.wcc_size, 1), 0.0);
  const int N = B.N, NJ = B.NJ;
  auto rv = [&](int a, int b, int JP) { return B.ccr[((size_t)a * N + b) * NJ + JP / 2]; };
  for (int q = 0; q < B.nblocks; ++q) {
    const int Jtot = B.lamJ[q];
    for (int g = 0; g < 6; ++g) {
      const int n1 = B.gn1[q][g], n2 = B.gn2[q][g];
      if (n1 * n2 == 0) continue;
      const int c1 = SEA1[g], c2 = SEA2[g];
      const int64_t o = B.goff[q][g];
      for (int IX = 0; IX < n1; ++IX) {
        const int i = B.qa[q][c1][IX], j = B.qb[q][c1][IX];
        const double pre = (i == j) ? .70710678118 : 1.0;
        const int ji = B.jj[i], jj_ = B.jj[j], li = B.ll[i], lj = B.ll[j], ti = B.tz[i], tj = B.tz[j];
        for (int JX = SQS[g] ? IX : 0; JX < n2; ++JX) {
          const int k = B.qa[q][c2][JX], l = B.qb[q][c2][JX];
          const double pre2 = (k == l) ? .70710678118 : 1.0;
          const int jk = B.jj[k], jl = B.jj[l], lk = B.ll[k], ll = B.ll[l], tk = B.tz[k], tl = B.tz[l];
          // the forward skips the element (no update, no mirror) unless both checks pass
          const int Tz1 = std::abs(ti - tk) / 2, PAR1 = (li + lk) % 2;
          if (std::abs(tl - tj) != Tz1 * 2 || (ll + lj) % 2 != PAR1) continue;
          const int Tz2 = std::abs(ti - tl) / 2, PAR2 = (li + ll) % 2;
          if (std::abs(tk - tj) != Tz2 * 2 || (lk + lj) % 2 != PAR2) continue;
          const int64_t ij = o + IX + (int64_t)JX * n1, ji_ = o + JX + (int64_t)IX * n1;
          const double s = (SQS[g] ? fold_square(cb, ij, ji_, IX == JX, hRES, true) : cb[ij]) * pre * pre2;
          if (s == 0.0) continue;
          const double phase = sgn((ji + jj_ + jk + jl) / 2);
          int jmin = std::max(std::abs(jj_ - jl), std::abs(ji - jk));
          int jmax = std::min(jj_ + jl, ji + jk);
          for (int JP = jmin; JP <= jmax; JP += 2) {
            const int qx = B.ccq(JP, Tz1, PAR1);
            double* W = Wb.data() + B.wcc_off[qx];
            const int64_t rl = B.cc_rlen[qx];
            const int rjl = rv(j, l, JP), rik = rv(i, k, JP), gjl = rv(l, j, JP), gik = rv(k, i, JP);
            const double c = -sgn((jl + jk + Jtot) / 2) * sixj(ji, jj_, Jtot, jl, jk, JP) * s;
            W[gik + rjl * rl] += c * hL;
            W[gjl + rik * rl] += c * phase * hL;
            W[rik + gjl * rl] -= c * phase * hR;
            W[rjl + gik * rl] -= c * hR;
          }
          jmin = std::max(std::abs(ji - jl), std::abs(jj_ - jk));
          jmax = std::min(ji + jl, jj_ + jk);
          for (int JP = jmin; JP <= jmax; JP += 2) {
            const int qx = B.ccq(JP, Tz2, PAR2);
            double* W = Wb.data() + B.wcc_off[qx];
            const int64_t rl = B.cc_rlen[qx];
            const int ril = rv(i, l, JP), rjk = rv(j, k, JP), gil = rv(l, i, JP), gjk = rv(k, j, JP);
            const double c = sixj(ji, jj_, Jtot, jk, jl, JP) * s;
            W[gil + rjk * rl] += c * hL;
            W[gjk + ril * rl] += c * phase * hL;
            W[ril + gjk * rl] -= c * phase * hR;
            W[rjk + gil * rl] -= c * hR;
          }
        }
      }
    }
  }
  for (int q = 0; q < B.ncc; ++q) {
    const int nb = B.cc_nph[q], r = B.cc_rlen[q];
    if (nb * r == 0) continue;
    const double* W = Wb.data() + B.wcc_off[q];
    dgemm('N', 'N', r, nb, r, 1.0, W, r, RCC + B.cc_off[q], r, 1.0, LCCb + B.cc_off[q], r);
    dgemm('T', 'N', r, nb, r, 1.0, W, r, LCC + B.cc_off[q], r, 1.0, RCCb + B.cc_off[q], r);
  }
}

// Reverse of full_commutator: Lb += d<Cb, [L,R]>/dL, Rb += d<Cb, [L,R]>/dR.  RES enters the
// forward only through E0 when with_e0 is false; that carried value has no cotangent here.
void full_commutator_vjp(const Basis& B, const double* L, int hL, const double* R, int hR, int hRES,
                         bool with_e0, const double* Cb, double* Lb, double* Rb) {
  std::vector<double> cb(Cb, Cb + B.slab), w1b(B.slab, 0.0), w2b(B.slab, 0.0);
  std::vector<double> lcc(std::max<int64_t>(B.cc_size, 1)), rcc(std::max<int64_t>(B.cc_size, 1));
  std::vector<double> lccb(std::max<int64_t>(B.cc_size, 1), 0.0), rccb(std::max<int64_t>(B.cc_size, 1), 0.0);
  cross_coupled(B, L, hL, lcc.data());
  cross_coupled(B, R, hR, rcc.data());
  comm222ph_vjp(B, lcc.data(), hL, rcc.data(), hR, hRES, cb.data(), lccb.data(), rccb.data());
  comm221_vjp(B, hL, hR, hRES, cb.data(), w1b.data(), w2b.data());
  comm222pphh_vjp(B, L, hL, R, hR, cb.data(), w1b.data(), w2b.data(), Lb, Rb);
  comm122_vjp(B, L, hL, R, hR, hRES, cb.data(), Lb, Rb);
  comm121_vjp(B, L, hL, R, hR, hRES, cb.data(), Lb, Rb);
  comm111_vjp(B, L, hL, R, hR, cb.data(), Lb, Rb);
  if (with_e0) {
    comm110_vjp(B, L, hL, R, hR, cb[0], Lb, Rb);
    comm220_vjp(B, L, hL, R, hR, cb[0], Lb, Rb);
  }
  cross_coupled_vjp(B, hL, lccb.data(), Lb);
  cross_coupled_vjp(B, hR, rccb.data(), Rb);
}

// build_gs_white: Hb += d<ETAb, eta(H)>/dH (eta = H_ai / D_ai and V_abij / D_abij with the
// denominators' one-body diagonals and monopoles differentiated too)
void white_vjp(const Basis& B, const double* H, int hH, const double* ETAb, double* Hb) {
  for (int a = 0; a < B.P; ++a) {
    const int ak = B.parts[a];
    for (int i = 0; i < B.A; ++i) {
      const int ik = B.holes[i];
      if (B.jj[ik] != B.jj[ak] || B.ll[ik] != B.ll[ak] || B.tz[ik] != B.tz[ak]) continue;
      const int ji = B.jj[ik];
      const int64_t ph = B.off_fph + a + (int64_t)i * B.P;
      const double eb = ETAb[ph];
      if (eb == 0.0) continue;
      double Eden = 0.0;
      for (int JT = 0; JT <= 2 * ji; JT += 2) Eden -= (JT + 1) * v_elem(B, H, hH, ak, ik, ak, ik, JT);
      Eden = Eden / (ji + 1.0) / (ji + 1.0);
      Eden = Eden + cfpp(B, H, a, a) - cfhh(B, H, i, i);
      Hb[ph] += eb / Eden;
      const double db = -eb * H[ph] / (Eden * Eden);
      Hb[B.off_fpp + a + (int64_t)a * B.P] += db;
      Hb[B.off_fhh + i + (int64_t)i * B.A] -= db;
      for (int JT = 0; JT <= 2 * ji; JT += 2)
        add_at(Hb, v_addr(B, hH, ak, ik, ak, ik, JT), -db * (JT + 1) / (ji + 1.0) / (ji + 1.0));
    }
  }
  auto mono_vjp = [&](int a, int b, double g) {
    const int ja = B.jj[a], jb = B.jj[b];
    for (int JT = std::abs(ja - jb); JT <= ja + jb; JT += 2)
      add_at(Hb, v_addr(B, hH, a, b, a, b, JT), g * (JT + 1) / (ja + 1.0) / (jb + 1.0));
  };
  for (int q = 0; q < B.nblocks; ++q) {
    const int np = B.ncls[q][0], nh = B.ncls[q][2];
    const double* HX = B.X(H, q, 2);
    const double* EB = B.X(ETAb, q, 2);
    const int64_t o = B.goff[q][2];
    for (int IX = 0; IX < np; ++IX) {
      const int a = B.qa[q][0][IX], b = B.qb[q][0][IX];
      for (int JX = 0; JX < nh; ++JX) {
        const double eb = EB[IX + (int64_t)JX * np];
        if (eb == 0.0) continue;
        const int i = B.qa[q][2][JX], j = B.qb[q][2][JX];
        double Eden = 0.0;
        Eden += monopole(B, H, hH, a, b);
        Eden += monopole(B, H, hH, i, j);
        Eden -= monopole(B, H, hH, a, i);
        Eden -= monopole(B, H, hH, a, j);
        Eden -= monopole(B, H, hH, i, b);
        Eden -= monopole(B, H, hH, j, b);
        Eden += f_elem(B, H, hH, a, a) + f_elem(B, H, hH, b, b) - f_elem(B, H, hH, i, i) - f_elem(B, H, hH, j, j);
        const double hx = HX[IX + (int64_t)JX * np];
        Hb[o + IX + (int64_t)JX * np] += eb / Eden;
        const double db = -eb * hx / (Eden * Eden);
        mono_vjp(a, b, db);
        mono_vjp(i, j, db);
        mono_vjp(a, i, -db);
        mono_vjp(a, j, -db);
        mono_vjp(i, b, -db);
        mono_vjp(j, b, -db);
        add_at(Hb, f_addr(B, hH, a, a), db);
        add_at(Hb, f_addr(B, hH, b, b), db);
        add_at(Hb, f_addr(B, hH, i, i), -db);
        add_at(Hb, f_addr(B, hH, j, j), -db);
      }
    }
  }
}

namespace {
#include "oracle_tensor.inc"
#include "oracle_hf.inc"
#include "oracle_eom.inc"
#include "oracle_triples.inc"
#include "oracle_quads.inc"
#include "oracle_input.inc"
}  // namespace

// ====================================================================== C interface
extern "C" {

void* orc_basis_create(int N, const int* nn, const int* ll, const int* jj, const int* tz, const int* con,
                       int eMax, double hw, int Aprot, int Aneut) {
  Basis* b = build_basis(N, nn, ll, jj, tz, con, eMax, hw, Aprot, Aneut);
  ensure_sixj(b->JM);
  return b;
}
void orc_basis_destroy(void* b) { delete (Basis*)b; }
int64_t orc_slab_size(void* b) { return ((Basis*)b)->slab; }
int orc_nblocks(void* b) { return ((Basis*)b)->nblocks; }
int orc_ncc(void* b) { return ((Basis*)b)->ncc; }
int64_t orc_cc_size(void* b) { return ((Basis*)b)->cc_size; }
int64_t orc_wcc_size(void* b) { return ((Basis*)b)->wcc_size; }
void orc_block_info(void* bp, int* lamJ, int* lamP, int* lamT, int* npp, int* nph, int* nhh) {
  Basis& B = *(Basis*)bp;
  for (int q = 0; q < B.nblocks; ++q) {
    lamJ[q] = B.lamJ[q]; lamP[q] = B.lamP[q]; lamT[q] = B.lamT[q];
    npp[q] = B.ncls[q][0]; nph[q] = B.ncls[q][1]; nhh[q] = B.ncls[q][2];
  }
}
// pair list of class cls (0 pp, 1 ph, 2 hh) of block q, 0-based orbits: out[2*k], out[2*k+1]
void orc_block_pairs(void* bp, int q, int cls, int* out) {
  Basis& B = *(Basis*)bp;
  for (size_t k = 0; k < B.qa[q][cls].size(); ++k) { out[2 * k] = B.qa[q][cls][k]; out[2 * k + 1] = B.qb[q][cls][k]; }
}
void orc_cc_info(void* bp, int* rlen, int* nph, int* J) {
  Basis& B = *(Basis*)bp;
  for (int q = 0; q < B.ncc; ++q) { rlen[q] = B.cc_rlen[q]; nph[q] = B.cc_nph[q]; J[q] = B.cc_J[q]; }
}
void orc_set_num_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_get_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_dgemm(void* fn, int ilp64) { g_blas = fn; g_blas_ilp64 = ilp64; }

double orc_sixj(int j1, int j2, int j3, int j4, int j5, int j6) { return angmom().sixj(j1, j2, j3, j4, j5, j6); }
double orc_ninej(int j1, int j2, int j3, int j4, int j5, int j6, int j7, int j8, int j9) {
  return angmom().ninej(j1, j2, j3, j4, j5, j6, j7, j8, j9);
}
double orc_v_elem(void* b, const double* op, int herm, int a, int bb, int c, int d, int J) {
  return v_elem(*(Basis*)b, op, herm, a, bb, c, d, J);
}
double orc_f_elem(void* b, const double* op, int herm, int a, int bb) { return f_elem(*(Basis*)b, op, herm, a, bb); }

void orc_random_op(void* b, uint64_t seed, int herm, double* op) { random_op(*(Basis*)b, seed, herm, op); }
void orc_synthetic_bare(void* b, uint64_t seed, double v_scale, double* H) {
  synthetic_bare(*(Basis*)b, seed, v_scale, H);
}

double orc_commutator_110(void* b, const double* L, int hL, const double* R, int hR) {
  return comm110(*(Basis*)b, L, hL, R, hR);
}
double orc_commutator_220(void* b, const double* L, int hL, const double* R, int hR) {
  return comm220(*(Basis*)b, L, hL, R, hR);
}
void orc_commutator_111(void* b, const double* L, int hL, const double* R, int hR, double* RES, int hRES) {
  comm111(*(Basis*)b, L, hL, R, hR, RES, hRES);
}
void orc_commutator_121(void* b, const double* L, int hL, const double* R, int hR, double* RES, int hRES) {
  comm121(*(Basis*)b, L, hL, R, hR, RES, hRES);
}
void orc_commutator_122(void* b, const double* L, int hL, const double* R, int hR, double* RES, int hRES) {
  comm122(*(Basis*)b, L, hL, R, hR, RES, hRES);
}
void orc_commutator_222_pp_hh(void* b, const double* L, int hL, const double* R, int hR, double* RES, int hRES,
                              double* w1, double* w2) {
  comm222pphh(*(Basis*)b, L, hL, R, hR, RES, hRES, w1, w2);
}
void orc_commutator_221(void* b, const double* L, int hL, const double* R, int hR, double* RES, int hRES,
                        const double* w1, const double* w2) {
  (void)L; (void)R;
  comm221(*(Basis*)b, hL, hR, RES, hRES, w1, w2);
}
void orc_calculate_cross_coupled(void* b, const double* op, int herm, double* cc) {
  cross_coupled(*(Basis*)b, op, herm, cc);
}
void orc_commutator_222_ph(void* b, const double* LCC, int hL, const double* RCC, int hR, double* RES, int hRES,
                           double* WCC) {
  comm222ph(*(Basis*)b, LCC, hL, RCC, hR, RES, hRES, WCC);
}
void orc_full_commutator(void* b, const double* L, int hL, const double* R, int hR, double* RES, int hRES) {
  Basis& B = *(Basis*)b;
  Work w(B);
  full_commutator(B, L, hL, R, hR, RES, hRES, w, true);
}
void orc_build_gs_white(void* b, const double* H, int hH, double* ETA) { white(*(Basis*)b, H, hH, ETA); }
void orc_build_gs_atanxx(void* b, const double* Hold, int hold, const double* H, double* ETA) {
  atan_gen(*(Basis*)b, Hold, hold, H, ETA);
}
void orc_commutator_e0(void* b, const double* L, int hL, const double* R, int hR, double* RES, int hRES,
                       int with_e0) {
  Basis& B = *(Basis*)b;
  Work w(B);
  full_commutator(B, L, hL, R, hR, RES, hRES, w, with_e0 != 0);
}
void orc_commutator_vjp(void* b, const double* L, int hL, const double* R, int hR, int hRES, int with_e0,
                        const double* Cb, double* Lb, double* Rb) {
  full_commutator_vjp(*(Basis*)b, L, hL, R, hR, hRES, with_e0 != 0, Cb, Lb, Rb);
}
void orc_white_vjp(void* b, const double* H, int hH, const double* ETAb, double* Hb) {
  white_vjp(*(Basis*)b, H, hH, ETAb, Hb);
}
double orc_mat_frob_norm(void* b, const double* op) { return frob(*(Basis*)b, op); }
double orc_mbpt2(void* b, const double* H, int hH) { return mbpt2(*(Basis*)b, H, hH); }
void orc_add_sq_op(void* b, const double* A, double ax, const double* Bop, double bx, double* C) {
  add_op(*(Basis*)b, A, ax, Bop, bx, C);
}
int orc_magnus_expand(void* b, double* DG, const double* G) {
  Basis& B = *(Basis*)b;
  Work w(B);
  return magnus_expand(B, DG, G, w);
}
int orc_bch_expand(void* b, double* HS, const double* G, const double* H, int max_terms, double conv) {
  Basis& B = *(Basis*)b;
  Work w(B);
  return bch_expand(B, HS, G, H, max_terms, conv, w);
}
int orc_cr_expand(void* b, double* HS, const double* G, const double* H, int max_terms, double conv) {
  Basis& B = *(Basis*)b;
  Work w(B);
  return bch_expand(B, HS, G, H, max_terms, conv, w, true);
}
double orc_bf_0body(void* b, const double* A, int hA, const double* Bo, int hB) { return bf0(*(Basis*)b, A, hA, Bo, hB); }
double orc_bf_1body(void* b, const double* A, int hA, const double* Bo, int hB, int a, int bb) {
  return bf1(*(Basis*)b, A, hA, Bo, hB, a, bb);
}
double orc_bf_2body(void* b, const double* A, int hA, const double* Bo, int hB, int a, int bb, int c, int d, int J) {
  return bf2(*(Basis*)b, A, hA, Bo, hB, a, bb, c, d, J);
}

// ---- tensor operators (oracle_tensor.inc)
void* orc_tbasis_create(void* b, int rank, int dpar) { return build_tbasis((Basis*)b, rank, dpar); }
void orc_tbasis_destroy(void* t) { delete (TBasis*)t; }
int64_t orc_tslab_size(void* t) { return ((TBasis*)t)->slab; }
int orc_tnblocks(void* t) { return ((TBasis*)t)->nblocks; }
void orc_tblock_info(void* t, int* J1, int* J2, int* Tz, int* P1, int* q1, int* q2) {
  const TBasis& T = *(TBasis*)t;
  for (int q = 0; q < T.nblocks; ++q) {
    J1[q] = T.J1[q]; J2[q] = T.J2[q]; Tz[q] = T.T[q]; P1[q] = T.P1[q]; q1[q] = T.q1[q]; q2[q] = T.q2[q];
  }
}
void orc_random_tensor(void* t, uint64_t seed, int herm, double* op) { random_tensor_op(*(TBasis*)t, seed, herm, op); }
void orc_tensor_commutator(void* t, const double* L, int hL, const double* R, int hR, double* RES, int mask) {
  tensor_commutator(*(TBasis*)t, L, hL, R, hR, RES, mask);
}
double orc_tensor_elem(void* t, const double* op, int herm, int a, int b, int c, int d, int J1, int J2) {
  return tensor_elem(*(TBasis*)t, op, herm, a, b, c, d, J1, J2);
}
double orc_f_tensor_elem(void* t, const double* op, int herm, int a, int b) {
  return f_tensor_elem(*(TBasis*)t, op, herm, a, b);
}
double orc_tensor_frob(void* t, const double* op) { return tensor_frob(*(TBasis*)t, op); }
int orc_bch_tensor(void* t, const double* G, double* HS, int max_terms, double conv) {
  return bch_tensor(*(TBasis*)t, G, HS, max_terms, conv);
}
double orc_tensor_bf1(void* t, const double* A, int hA, const double* Bo, int hB, int a, int b) {
  return tensor_bf1(*(TBasis*)t, A, hA, Bo, hB, a, b);
}
double orc_tensor_bf2(void* t, const double* A, int hA, const double* Bo, int hB, int a, int b, int c, int d, int J1,
                      int J2) {
  return tensor_bf2(*(TBasis*)t, A, hA, Bo, hB, a, b, c, d, J1, J2);
}


// ---- Hartree-Fock input preparation (oracle_hf.inc)
void orc_gamma_matrix(void* b, const double* op, int herm, const double* rho, double* gam) {
  gamma_matrix(*(Basis*)b, op, herm, rho, gam);
}
void orc_transform_2b_to_hf(void* b, double* op, const double* D) { transform_2b_to_hf(*(Basis*)b, op, D); }
void orc_normal_order(void* b, const double* in, int herm, double* out) { normal_order(*(Basis*)b, in, herm, out); }
int64_t orc_vectorize(void* b, const double* op, double* v) { return vectorize(*(Basis*)b, op, v); }
double orc_p1_p2(void* b, int a, int bb, int c, int d, int J) { return dot12(*(Basis*)b, a, bb, c, d, J, true); }
double orc_r1_r2(void* b, int a, int bb, int c, int d, int J) { return dot12(*(Basis*)b, a, bb, c, d, J, false); }

// ---- EOM-IMSRG ladder operators (oracle_eom.inc)
void* orc_eom_create(void* t) { return new EomMap(build_eom_map(*(TBasis*)t)); }
void orc_eom_destroy(void* m) { delete (EomMap*)m; }
int64_t orc_eom_dim(void* m, int64_t* n1b) {
  *n1b = ((EomMap*)m)->n1b;
  return ((EomMap*)m)->n;
}
void orc_eom_map(void* m, int64_t* pos, int8_t* kind, int8_t* phase, int64_t* mirror) {
  const EomMap& M = *(EomMap*)m;
  for (int64_t k = 0; k < M.n; ++k) { pos[k] = M.pos[k]; kind[k] = M.kind[k]; phase[k] = M.phase[k]; mirror[k] = M.mirror[k]; }
}
void orc_eom_unwrap(void* t, void* m, const double* v, double* X) { eom_unwrap(*(TBasis*)t, *(EomMap*)m, v, X); }
void orc_eom_rewrap(void* m, const double* X, double* v) { eom_rewrap(*(EomMap*)m, X, v); }
double orc_eom_bf1(void* t, const double* A, int hA, const double* X, int a, int b) {
  return eom_bf1(*(TBasis*)t, A, hA, X, a, b);
}
double orc_eom_bf2(void* t, const double* A, int hA, const double* X, int a, int b, int c, int d, int J1, int J2) {
  return eom_bf2(*(TBasis*)t, A, hA, X, a, b, c, d, J1, J2);
}
double orc_pphh_ladder_elem(void* t, const double* X, int a, int b, int c, int d, int J1, int J2) {
  return pphh_ladder_elem(*(TBasis*)t, X, a, b, c, d, J1, J2);
}
void orc_eom_matvec(void* t, void* m, const double* H, const double* v, double* w) {
  eom_matvec(*(TBasis*)t, *(EomMap*)m, H, v, w);
}

// ---- perturbative triples (oracle_triples.inc)
int orc_three_channels(void* b, int* J, int* Tz, int* P, int* nppp, int* nhhh) {
  const std::vector<ThreeChannel> ch = enumerate_three_body(*(Basis*)b);
  for (size_t q = 0; q < ch.size(); ++q) {
    if (J) { J[q] = ch[q].J; Tz[q] = ch[q].Tz; P[q] = ch[q].P; nppp[q] = (int)ch[q].ppp.size(); nhhh[q] = (int)ch[q].hhh.size(); }
  }
  return (int)ch.size();
}
double orc_comm223(void* b, const double* L, int hL, const double* R, int hR, int p, int q, int r, int s, int t, int u,
                   int Jtot, int jpq, int jst) {
  return comm223(*(Basis*)b, L, hL, R, hR, p, q, r, s, t, u, Jtot, jpq, jst);
}
double orc_restore_triples(void* b, const double* H, const double* OM, int chan) {
  return restore_triples(*(Basis*)b, H, OM, chan);
}

// ---- quadrupoles in BCH_EXPAND (oracle_quads.inc)
void orc_restore_quadrupoles(void* b, const double* X, int hX, const double* OM, int hOM, double* RES) {
  restore_quadrupoles(*(Basis*)b, X, hX, OM, hOM, RES);
}
int orc_bch_expand_quads(void* b, double* HS, const double* G, const double* H, int max_terms, double conv) {
  Basis& B = *(Basis*)b;
  Work w(B);
  return bch_expand_quads(B, HS, G, H, max_terms, conv, w);
}

}  // extern "C"
