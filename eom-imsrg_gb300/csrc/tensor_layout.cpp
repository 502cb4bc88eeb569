// Host construction of the tensor layout and of the tensor ladder's GEMM problems.
#include <algorithm>
#include <cstdlib>

#include "tensor.h"

namespace imsrg {

namespace {
inline bool tri(int a, int b, int c) { return c <= a + b && c >= std::abs(a - b); }
// (class of bra pair, class of ket pair) -> tgam index (0-based)
inline int tg_of(int c1, int c2) {
  static const int t[3][3] = {{0, 1, 2}, {7, 3, 5}, {6, 8, 4}};
  return t[c1][c2];
}
// scalar storage index of the (c1 <= c2) class block
inline int qx_of(int c1, int c2) {
  static const int t[3][3] = {{0, 1, 2}, {1, 3, 5}, {2, 5, 4}};
  return t[c1][c2];
}
const int kTSea1[9] = {0, 0, 0, 1, 2, 1, 2, 1, 2}, kTSea2[9] = {0, 1, 2, 1, 2, 2, 0, 0, 1};
}  // namespace

std::string build_tlayout(TLayout& T, const Layout& L, int rank, int dpar) {
  if (rank < 0 || (rank & 1) || rank > 2 * L.JM) return "rank must be an even doubled value in 0..2*jmax";
  if (dpar != 0 && dpar != 2) return "dpar must be 0 or 2 (doubled)";
  T = TLayout();
  T.rank = rank;
  T.dpar = dpar;
  const int dp = dpar / 2;
  const int NJ = L.JM + 1;
  T.lut.assign((size_t)NJ * (rank / 2 + 1) * 6, -1);
  int q = 0;
  for (int j1 = 0; j1 <= 2 * L.JM; j1 += 2)
    for (int j2 = std::max(std::abs(j1 - rank), j1); j2 <= j1 + rank; j2 += 2)
      for (int t = -1; t <= 1; ++t)
        for (int p = 0; p <= 1; ++p) {
          const int p2 = dp ? 1 - p : p;
          const bool live = j2 <= 2 * L.JM;
          T.J1.push_back(j1); T.J2.push_back(j2); T.T.push_back(t); T.P1.push_back(p); T.P2.push_back(p2);
          T.q1.push_back(live ? L.block(j1, t, p) : -1);
          T.q2.push_back(live ? L.block(j2, t, p2) : -1);
          T.lut[(((size_t)(j1 / 2) * (rank / 2 + 1) + (j2 - j1) / 2) * 3 + (t + 1)) * 2 + p] = q;
          ++q;
        }
  T.nblocks = q;
  int64_t o = 1;
  T.off_fhh = o; o += (int64_t)L.A * L.A;
  T.off_fpp = o; o += (int64_t)L.P * L.P;
  T.off_fph = o; o += (int64_t)L.P * L.A;
  const int64_t o2 = o;
  T.goff.resize((size_t)q * 9); T.n1.resize((size_t)q * 9); T.n2.resize((size_t)q * 9);
  for (int k = 0; k < q; ++k)
    for (int g = 0; g < 9; ++g) {
      const size_t i = (size_t)k * 9 + g;
      T.n1[i] = T.q1[k] < 0 ? 0 : L.ncls[T.q1[k]][kTSea1[g]];
      T.n2[i] = T.q2[k] < 0 ? 0 : L.ncls[T.q2[k]][kTSea2[g]];
      T.goff[i] = o;
      o += (int64_t)T.n1[i] * T.n2[i];
    }
  T.slab = o;
  T.n2b = o - o2;

  // one-body outputs (allowed couplings of a rank-lambda, parity-dpar one-body operator)
  auto allowed = [&](int a, int b) {
    return tri(L.jj[a], L.jj[b], rank) && L.tz[a] == L.tz[b] && (L.ll[a] % 2) == ((L.ll[b] + dp) % 2);
  };
  auto add_ob = [&](int kind, int p, int qq, int pk, int qk) {
    T.ob_kind.push_back(kind); T.ob_p.push_back(p); T.ob_q.push_back(qq); T.ob_pk.push_back(pk); T.ob_qk.push_back(qk);
  };
  for (int p = 0; p < L.A; ++p)
    for (int qq = p; qq < L.A; ++qq)
      if (allowed(L.holes[p], L.holes[qq])) add_ob(0, p, qq, L.holes[p], L.holes[qq]);
  for (int p = 0; p < L.P; ++p)
    for (int qq = p; qq < L.P; ++qq)
      if (allowed(L.parts[p], L.parts[qq])) add_ob(1, p, qq, L.parts[p], L.parts[qq]);
  for (int p = 0; p < L.P; ++p)
    for (int qq = 0; qq < L.A; ++qq)
      if (allowed(L.parts[p], L.holes[qq])) add_ob(2, p, qq, L.parts[p], L.holes[qq]);

  // 6j tables
  T.six_nJ = L.JM + 1;
  T.six_nh = (L.JM + 1) / 2;
  T.six_nhx = (L.JM + rank + 1) / 2;
  const int nJ = T.six_nJ, nh = T.six_nh, nhx = T.six_nhx;
  T.six.assign((size_t)nJ * nJ * nhx * nh * nh, 0.0);
  for (int a = 0; a < nJ; ++a)
    for (int b = 0; b < nJ; ++b) {
      if (!tri(2 * a, 2 * b, rank)) continue;
      for (int x = 0; x < nhx; ++x)
        for (int y = 0; y < nh; ++y)
          for (int z = 0; z < nh; ++z)
            T.six[(((size_t)a * nJ + b) * nhx + x) * nh * nh + (size_t)y * nh + z] =
                sixj_racah(2 * a, 2 * b, rank, 2 * x + 1, 2 * y + 1, 2 * z + 1);
    }
  T.six_m.assign((size_t)nh * nh * nh * nhx * nJ * nJ, 0.0);
  for (int c = 0; c < nh; ++c)
    for (int d = 0; d < nh; ++d)
      for (int b = 0; b < nh; ++b)
        for (int x = 0; x < nhx; ++x)
          for (int J2 = 0; J2 < nJ; ++J2) {
            if (!tri(2 * c + 1, 2 * d + 1, 2 * J2) || !tri(2 * b + 1, 2 * x + 1, 2 * J2)) continue;
            for (int J4 = 0; J4 < nJ; ++J4)
              T.six_m[((((size_t)c * nh + d) * nh + b) * nhx + x) * nJ * nJ + (size_t)J2 * nJ + J4] =
                  sixj_racah(2 * c + 1, 2 * d + 1, 2 * J2, 2 * b + 1, 2 * x + 1, 2 * J4);
          }

  // ph column index of (p, h) in every cross-coupled channel
  T.ccnb.assign((size_t)L.N * L.N * NJ, -1);
  for (int c = 0; c < L.ncc; ++c)
    for (int k = 0; k < L.cc_nph[c]; ++k) {
      const int p = L.cc_cp[L.cc_col_off[c] + k], h = L.cc_ch[L.cc_col_off[c] + k];
      T.ccnb[((size_t)p * L.N + h) * NJ + L.cc_J[c] / 2] = k;
    }

  // orbits a tensor one-body element f(a, i) can couple to (TS_commutator_212's sums)
  T.tnb_start.assign(L.N, 0);
  T.tnb_count.assign(L.N, 0);
  T.tnb_list.clear();
  for (int a = 0; a < L.N; ++a) {
    T.tnb_start[a] = (int)T.tnb_list.size();
    for (int i = 0; i < L.N; ++i)
      if (L.tz[i] == L.tz[a] && ((L.ll[i] + dpar / 2) & 1) == (L.ll[a] & 1) && tri(L.jj[i], L.jj[a], rank))
        T.tnb_list.push_back(i);
    T.tnb_count[a] = (int)T.tnb_list.size() - T.tnb_start[a];
  }

  // cross-coupled tensor blocks of the particle-hole term
  for (int j3 = 0; j3 <= 2 * L.JM; j3 += 2)
    for (int j4 = std::max(std::abs(j3 - rank), j3); j4 <= j3 + rank; j4 += 2)
      for (int tz = 0; tz <= 1; ++tz)
        for (int par = 0; par <= 1; ++par) {
          if (j4 > 2 * L.JM) continue;
          const int qa = L.ccq(j3, tz, par), qb = L.ccq(j4, tz, (par + dp) % 2);
          const int64_t r1 = L.cc_rlen[qa], r2 = L.cc_rlen[qb];
          if (r1 * r2 == 0) continue;
          T.cb_J3.push_back(j3); T.cb_J4.push_back(j4); T.cb_Tz.push_back(tz); T.cb_PAR.push_back(par);
          T.cb_qa.push_back(qa); T.cb_qb.push_back(qb);
          T.cb_max_w = std::max(T.cb_max_w, r1 * r2);
          T.cb_max_x = std::max(T.cb_max_x, std::max(r1 * L.cc_nph[qb], (int64_t)L.cc_nph[qa] * r2));
          T.cb_max_r = std::max(T.cb_max_r, std::max(r1, r2));
        }

  // Frobenius-norm segments
  auto add_seg = [&](int64_t off, int64_t n, int w) {
    for (int64_t s = 0; s < n; s += 65536) {
      T.seg_start.push_back(off + s);
      T.seg_len.push_back((int)std::min<int64_t>(65536, n - s));
      T.seg_w.push_back((int8_t)w);
    }
  };
  add_seg(T.off_fhh, (int64_t)L.A * L.A, 1);
  add_seg(T.off_fph, (int64_t)L.P * L.A, 2);
  add_seg(T.off_fpp, (int64_t)L.P * L.P, 1);
  for (int k = 0; k < q; ++k)
    for (int g = 0; g < 9; ++g) {
      const size_t i = (size_t)k * 9 + g;
      add_seg(T.goff[i], (int64_t)T.n1[i] * T.n2[i], T.J1[k] == T.J2[k] ? 1 : 2);
    }
  return std::string();
}

std::vector<GemmProb> build_tensor_pphh_problems(const TLayout& T, const Layout& L, bool excitation_only) {
  std::vector<GemmProb> P;
  const int N = 0, TR = 1;
  for (int q = 0; q < T.nblocks; ++q) {
    const int qa = T.q1[q], qb = T.q2[q];
    if (qa < 0) continue;
    for (int g = 0; g < 9; ++g) {
      const int c1 = kTSea1[g], c2 = kTSea2[g];
      const int M = L.ncls[qa][c1], Nn = L.ncls[qb][c2];
      if (M * Nn == 0) continue;
      for (int side = 0; side < 2; ++side) {
        const int k = side == 0 ? 0 : 2;  // pp or hh intermediate pairs
        const int K1 = L.ncls[qa][k], K2 = L.ncls[qb][k];
        GemmProb p{};
        p.c_id = side == 0 ? kOpW1 : kOpW2;
        p.c_off = T.goff[(size_t)q * 9 + g];
        p.M = M; p.N = Nn; p.ldc = M;
        auto excitation = [](int g) { return g == 2 || g == 6; };
        if (K1 && (!excitation_only || excitation(tg_of(k, c2)))) {  // + L(qa)[c1,k] R[k,c2]
          GemmTerm t{};
          if (c1 <= k) {
            t.a_id = kOpL; t.a_off = L.goff[qa * 6 + qx_of(c1, k)]; t.lda = L.ncls[qa][c1]; t.ta = N; t.alpha = kAlphaOne;
          } else {
            t.a_id = kOpL; t.a_off = L.goff[qa * 6 + qx_of(k, c1)]; t.lda = L.ncls[qa][k]; t.ta = TR; t.alpha = kAlphaHL;
          }
          t.b_id = kOpR; t.b_off = T.goff[(size_t)q * 9 + tg_of(k, c2)]; t.ldb = K1; t.tb = N;
          t.K = K1;
          p.t[p.nterm++] = t;
        }
        if (K2 && (!excitation_only || excitation(tg_of(c1, k)))) {  // - R[c1,k] L(qb)[k,c2]
          GemmTerm t{};
          t.a_id = kOpR; t.a_off = T.goff[(size_t)q * 9 + tg_of(c1, k)]; t.lda = M; t.ta = N;
          if (k <= c2) {
            t.b_id = kOpL; t.b_off = L.goff[qb * 6 + qx_of(k, c2)]; t.ldb = L.ncls[qb][k]; t.tb = N;
            t.alpha = kAlphaNeg | kAlphaOne;
          } else {
            t.b_id = kOpL; t.b_off = L.goff[qb * 6 + qx_of(c2, k)]; t.ldb = L.ncls[qb][c2]; t.tb = TR;
            t.alpha = kAlphaNeg | kAlphaHL;
          }
          t.K = K2;
          p.t[p.nterm++] = t;
        }
        if (p.nterm) P.push_back(p);
      }
    }
  }
  return P;
}

}  // namespace imsrg
