// Basis and channel layout for the commutator engine (host side).
//
// The orders below are the drop-in contract with the reference's sq_op / cc_mat:
//  * sq_op channels: 2J outer (0..2*jmax), Tz = -1..1, parity 0..1 inner, pairs (i<=j)
//    enumerated with i outer, j inner, split into pp/ph/hh by occupation
//    (allocate_blocks, src/basic_IMSRG.f90:521-685);
//  * cross-coupled channels: JC fastest, then |Tz|, then parity, rows = all ordered
//    pairs (i outer, j inner), columns = the (particle, hole) rows
//    (allocate_CCMAT, src/cross_coupled.f90:61-177).
// Lookups the reference does with linear searches (xmap, rmap/qmap, specific_rval)
// become dense [a][b][J] tables here so device code needs one load per lookup.
#include "layout.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>

namespace imsrg {
namespace {

bool tri(int a, int b, int J) { return J <= a + b && J >= std::abs(a - b); }
double sgn(int n) { return (n & 1) ? -1.0 : 1.0; }

struct LogFact {
  double v[1001];
  LogFact() {
    v[0] = 0.0;
    for (int i = 1; i <= 1000; ++i) v[i] = v[i - 1] + std::log((double)i);
  }
};
const LogFact& lf() {
  static LogFact f;
  return f;
}
double log_delta(int a, int b, int c) {
  const double* v = lf().v;
  return 0.5 * (v[(a + b - c) / 2] + v[(a - b + c) / 2] + v[(-a + b + c) / 2] - v[(a + b + c) / 2 + 1]);
}

}  // namespace

// Racah's closed form of the 6j symbol (doubled arguments), evaluated with log-factorials.
double sixj_racah(int j1, int j2, int j3, int j4, int j5, int j6) {
  if (!tri(j1, j2, j3) || !tri(j1, j5, j6) || !tri(j4, j2, j6) || !tri(j4, j5, j3)) return 0.0;
  if (((j1 + j2 + j3) | (j1 + j5 + j6) | (j4 + j2 + j6) | (j4 + j5 + j3)) & 1) return 0.0;
  const double* v = lf().v;
  const double d = log_delta(j1, j2, j3) + log_delta(j1, j5, j6) + log_delta(j4, j2, j6) + log_delta(j4, j5, j3);
  const int a1 = (j1 + j2 + j3) / 2, a2 = (j1 + j5 + j6) / 2, a3 = (j4 + j2 + j6) / 2, a4 = (j4 + j5 + j3) / 2;
  const int b1 = (j1 + j2 + j4 + j5) / 2, b2 = (j2 + j3 + j5 + j6) / 2, b3 = (j3 + j1 + j6 + j4) / 2;
  const int t0 = std::max(std::max(a1, a2), std::max(a3, a4)), t1 = std::min(b1, std::min(b2, b3));
  double s = 0.0;
  for (int t = t0; t <= t1; ++t)
    s += sgn(t) * std::exp(d + v[t + 1] - v[t - a1] - v[t - a2] - v[t - a3] - v[t - a4] - v[b1 - t] - v[b2 - t] -
                           v[b3 - t]);
  return s;
}

std::string build_layout(Layout& L, int N, const int* nn, const int* ll, const int* jj, const int* tz,
                         const int* con, int eMax, double hw, int Aprot, int Aneut) {
  if (N <= 0 || N > 32767) return "number of orbits must be in 1..32767";
  for (int i = 0; i < N; ++i) {
    if (jj[i] < 1 || (jj[i] & 1) == 0) return "2j must be a positive odd integer";
    if (tz[i] != -1 && tz[i] != 1) return "2tz must be -1 or +1";
    if (con[i] != 0 && con[i] != 1) return "occupation must be 0 or 1";
    if (ll[i] < 0 || nn[i] < 0) return "n and l must be non-negative";
  }
  L = Layout();
  L.N = N;
  L.eMax = eMax;
  L.hw = hw;
  L.Aprot = Aprot;
  L.Aneut = Aneut;
  L.nn.assign(nn, nn + N);
  L.ll.assign(ll, ll + N);
  L.jj.assign(jj, jj + N);
  L.tz.assign(tz, tz + N);
  L.con.assign(con, con + N);
  L.loc.resize(N);
  for (int i = 0; i < N; ++i) {
    if (con[i]) { L.loc[i] = (int)L.holes.size(); L.holes.push_back(i); }
    else { L.loc[i] = (int)L.parts.size(); L.parts.push_back(i); }
  }
  L.A = (int)L.holes.size();
  L.P = N - L.A;
  L.JM = *std::max_element(jj, jj + N);
  L.lmax = *std::max_element(ll, ll + N);
  L.NJ = L.JM + 1;
  L.same_start.resize(N);
  L.same_count.resize(N);
  for (int i = 0; i < N; ++i) {
    L.same_start[i] = (int)L.same_list.size();
    for (int k = 0; k < N; ++k)
      if (jj[k] == jj[i] && ll[k] == ll[i] && tz[k] == tz[i]) L.same_list.push_back(k);
    L.same_count[i] = (int)L.same_list.size() - L.same_start[i];
  }

  // ---- sq_op channels
  const int NJ = L.NJ;
  L.nblocks = (L.JM + 1) * 6;
  L.lamJ.resize(L.nblocks);
  L.lamP.resize(L.nblocks);
  L.lamT.resize(L.nblocks);
  L.ncls.resize(L.nblocks);
  L.pair_off.resize(L.nblocks * 3 + 1);
  L.pairpos.assign((size_t)N * N * NJ, -1);
  std::vector<std::array<std::vector<int16_t>, 3>> pa(L.nblocks), pb(L.nblocks);
  for (int J2 = 0, q = 0; J2 <= 2 * L.JM; J2 += 2)
    for (int T = -1; T <= 1; ++T)
      for (int Par = 0; Par <= 1; ++Par, ++q) {
        L.lamJ[q] = J2; L.lamT[q] = T; L.lamP[q] = Par;
        for (int i = 0; i < N; ++i)
          for (int j = i; j < N; ++j) {
            if ((tz[i] + tz[j]) != 2 * T || (ll[i] + ll[j]) % 2 != Par || !tri(jj[i], jj[j], J2)) continue;
            const int c = con[i] + con[j];
            L.pairpos[((size_t)i * N + j) * NJ + J2 / 2] = (int)pa[q][c].size();
            pa[q][c].push_back((int16_t)i);
            pb[q][c].push_back((int16_t)j);
          }
        for (int c = 0; c < 3; ++c) L.ncls[q][c] = (int)pa[q][c].size();
      }
  for (int q = 0; q < L.nblocks; ++q)
    for (int c = 0; c < 3; ++c) {
      L.pair_off[q * 3 + c] = (int)L.pair_a.size();
      L.pair_a.insert(L.pair_a.end(), pa[q][c].begin(), pa[q][c].end());
      L.pair_b.insert(L.pair_b.end(), pb[q][c].begin(), pb[q][c].end());
    }
  L.pair_off[L.nblocks * 3] = (int)L.pair_a.size();

  int64_t o = 1;
  L.off_fhh = o; o += (int64_t)L.A * L.A;
  L.off_fpp = o; o += (int64_t)L.P * L.P;
  L.off_fph = o; o += (int64_t)L.P * L.A;
  L.goff.resize(L.nblocks * 6);
  L.gn1.resize(L.nblocks * 6);
  L.gn2.resize(L.nblocks * 6);
  L.uoff.resize(L.nblocks * 6 + 1);
  int64_t u = 0;
  for (int q = 0; q < L.nblocks; ++q)
    for (int g = 0; g < 6; ++g) {
      const int k = q * 6 + g;
      L.gn1[k] = L.ncls[q][kSea1[g]];
      L.gn2[k] = L.ncls[q][kSea2[g]];
      L.goff[k] = o;
      o += (int64_t)L.gn1[k] * L.gn2[k];
      L.uoff[k] = u;
      u += kSquare[g] ? (int64_t)L.gn1[k] * (L.gn1[k] + 1) / 2 : (int64_t)L.gn1[k] * L.gn2[k];
    }
  L.uoff[L.nblocks * 6] = u;
  L.n_unique = u;
  L.slab = o;

  // ---- cross-coupled channels
  L.ncc = (L.JM + 1) * 4;
  L.cc_rlen.assign(L.ncc, 0);
  L.cc_nph.assign(L.ncc, 0);
  L.cc_J.assign(L.ncc, 0);
  L.cc_row_off.resize(L.ncc + 1);
  L.cc_col_off.resize(L.ncc + 1);
  L.ccr.assign((size_t)N * N * NJ, -1);
  for (int q = 0; q < L.ncc; ++q) {
    const int JC = (q % (L.JM + 1)) * 2;
    const int TZ = (q % (2 * L.JM + 2)) / (L.JM + 1);
    const int PAR = q / (2 * L.JM + 2);
    L.cc_J[q] = JC;
    L.cc_row_off[q] = (int)L.cc_ra.size();
    L.cc_col_off[q] = (int)L.cc_cp.size();
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        if (!tri(jj[i], jj[j], JC) || (ll[i] + ll[j]) % 2 != PAR || std::abs(tz[i] - tz[j]) / 2 != TZ) continue;
        if (con[i] == 0 && con[j] == 1) {
          L.cc_cp.push_back((int16_t)i);
          L.cc_ch.push_back((int16_t)j);
        }
        L.ccr[((size_t)i * N + j) * NJ + JC / 2] = (int)(L.cc_ra.size() - L.cc_row_off[q]);
        L.cc_ra.push_back((int16_t)i);
        L.cc_rb.push_back((int16_t)j);
      }
    L.cc_rlen[q] = (int)L.cc_ra.size() - L.cc_row_off[q];
    L.cc_nph[q] = (int)L.cc_cp.size() - L.cc_col_off[q];
  }
  L.cc_row_off[L.ncc] = (int)L.cc_ra.size();
  L.cc_col_off[L.ncc] = (int)L.cc_cp.size();
  L.cc_off.resize(L.ncc + 1);
  L.wcc_off.resize(L.ncc + 1);
  int64_t c1 = 0, c2 = 0;
  for (int q = 0; q < L.ncc; ++q) {
    L.cc_off[q] = c1; c1 += (int64_t)L.cc_rlen[q] * L.cc_nph[q];
    L.wcc_off[q] = c2; c2 += (int64_t)L.cc_rlen[q] * L.cc_rlen[q];
  }
  L.cc_off[L.ncc] = c1;
  L.wcc_off[L.ncc] = c2;
  L.cc_size = c1;
  L.wcc_size = c2;

  // ---- one-body output lists (commutator_121 / _221 loops)
  auto same = [&](int x, int y) { return jj[x] == jj[y] && ll[x] == ll[y] && tz[x] == tz[y]; };
  auto add_ob = [&](int kind, int p, int q, int pk, int qk) {
    L.ob_kind.push_back(kind); L.ob_p.push_back(p); L.ob_q.push_back(q);
    L.ob_pk.push_back(pk); L.ob_qk.push_back(qk);
  };
  for (int p = 0; p < L.A; ++p)
    for (int q = p; q < L.A; ++q)
      if (same(L.holes[p], L.holes[q])) add_ob(0, p, q, L.holes[p], L.holes[q]);
  for (int p = 0; p < L.P; ++p)
    for (int q = p; q < L.P; ++q)
      if (same(L.parts[p], L.parts[q])) add_ob(1, p, q, L.parts[p], L.parts[q]);
  for (int p = 0; p < L.P; ++p)
    for (int q = 0; q < L.A; ++q)
      if (same(L.parts[p], L.holes[q])) add_ob(2, p, q, L.parts[p], L.holes[q]);

  for (int a = 0; a < L.P; ++a)
    for (int i = 0; i < L.A; ++i)
      if (same(L.parts[a], L.holes[i])) { L.ai_a.push_back(a); L.ai_i.push_back(i); }

  // ---- 6j table
  const int nh = (L.JM + 1) / 2;
  L.sj_nh = nh;
  const size_t nq = (size_t)nh * nh * nh * nh;
  L.sj_off.resize(nq);
  L.sj_j3min.resize(nq);
  L.sj_j6min.resize(nq);
  L.sj_n6.resize(nq);
  int64_t so = 0;
  for (size_t k = 0; k < nq; ++k) {
    const int h5 = (int)(k % nh), h4 = (int)((k / nh) % nh), h2 = (int)((k / nh / nh) % nh), h1 = (int)(k / nh / nh / nh);
    const int j1 = 2 * h1 + 1, j2 = 2 * h2 + 1, j4 = 2 * h4 + 1, j5 = 2 * h5 + 1;
    const int a = std::max(std::abs(j1 - j2), std::abs(j4 - j5)), b = std::min(j1 + j2, j4 + j5);
    const int c = std::max(std::abs(j1 - j5), std::abs(j4 - j2)), d = std::min(j1 + j5, j4 + j2);
    L.sj_off[k] = (int)so;
    L.sj_j3min[k] = a;
    L.sj_j6min[k] = c;
    const int n3 = a <= b ? (b - a) / 2 + 1 : 0, n6 = c <= d ? (d - c) / 2 + 1 : 0;
    L.sj_n6[k] = n6;
    so += (int64_t)n3 * n6;
  }
  L.sj_val.assign(so, 0.0);
  for (size_t k = 0; k < nq; ++k) {
    const int h5 = (int)(k % nh), h4 = (int)((k / nh) % nh), h2 = (int)((k / nh / nh) % nh), h1 = (int)(k / nh / nh / nh);
    const int j1 = 2 * h1 + 1, j2 = 2 * h2 + 1, j4 = 2 * h4 + 1, j5 = 2 * h5 + 1;
    const int b = std::min(j1 + j2, j4 + j5), d = std::min(j1 + j5, j4 + j2);
    for (int j3 = L.sj_j3min[k]; j3 <= b; j3 += 2)
      for (int j6 = L.sj_j6min[k]; j6 <= d; j6 += 2)
        L.sj_val[L.sj_off[k] + ((j3 - L.sj_j3min[k]) / 2) * L.sj_n6[k] + (j6 - L.sj_j6min[k]) / 2] =
            sixj_racah(j1, j2, j3, j4, j5, j6);
  }
  return std::string();
}

// f_elem (src/basic_IMSRG.f90:1191-1221)
double host_f_elem(const Layout& L, const double* op, int herm, int a, int b) {
  const int c1 = L.con[a], c2 = L.con[b];
  if (c1 + c2 == 0) return op[L.off_fpp + L.loc[a] + (int64_t)L.loc[b] * L.P];
  if (c1 + c2 == 2) return op[L.off_fhh + L.loc[a] + (int64_t)L.loc[b] * L.A];
  if (c1 > c2) return op[L.off_fph + L.loc[b] + (int64_t)L.loc[a] * L.P] * herm;
  return op[L.off_fph + L.loc[a] + (int64_t)L.loc[b] * L.P];
}

// v_elem (src/basic_IMSRG.f90:1314-1429)
double host_v_elem(const Layout& L, const double* op, int herm, int a, int b, int c, int d, int J) {
  if (!tri(L.jj[a], L.jj[b], J) || !tri(L.jj[c], L.jj[d], J)) return 0.0;
  const int P = (L.ll[a] + L.ll[b]) & 1;
  if (((L.ll[c] + L.ll[d]) & 1) != P) return 0.0;
  if (L.tz[a] + L.tz[b] != L.tz[c] + L.tz[d]) return 0.0;
  const int q = L.block(J, (L.tz[a] + L.tz[b]) / 2, P);
  const int C1 = L.con[a] + L.con[b], C2 = L.con[c] + L.con[d];
  static const int tab[3][3] = {{0, 1, 2}, {1, 3, 5}, {2, 5, 4}};
  const int g = tab[C1][C2];
  const size_t N = L.N, NJ = L.NJ;
  double pre = 1.0;
  int i1, i2;
  if (a > b) { i1 = L.pairpos[((size_t)b * N + a) * NJ + J / 2]; pre = sgn(1 + (L.jj[a] + L.jj[b] - J) / 2); }
  else { if (a == b) pre *= std::sqrt(2.0); i1 = L.pairpos[((size_t)a * N + b) * NJ + J / 2]; }
  if (c > d) { i2 = L.pairpos[((size_t)d * N + c) * NJ + J / 2]; pre *= sgn(1 + (L.jj[c] + L.jj[d] - J) / 2); }
  else { if (c == d) pre *= std::sqrt(2.0); i2 = L.pairpos[((size_t)c * N + d) * NJ + J / 2]; }
  const double* X = op + L.goff[q * 6 + g];
  const int n1 = L.gn1[q * 6 + g];
  if (C1 > C2) return X[i2 + (int64_t)i1 * n1] * herm * pre;
  return X[i1 + (int64_t)i2 * n1] * pre;
}

}  // namespace imsrg
