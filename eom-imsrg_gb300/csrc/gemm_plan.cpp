// Host construction of the grouped-GEMM problem and tile lists.
#include <algorithm>

#include "gemm.h"

namespace imsrg {
namespace {

GemmTerm term(int a_id, int64_t a_off, int lda, int ta, int b_id, int64_t b_off, int ldb, int tb, int K, int alpha) {
  GemmTerm t{};
  t.a_id = a_id; t.a_off = a_off; t.lda = lda; t.ta = ta;
  t.b_id = b_id; t.b_off = b_off; t.ldb = ldb; t.tb = tb;
  t.K = K; t.alpha = alpha;
  return t;
}
GemmProb prob(int c_id, int64_t c_off, int M, int N, int ldc, const GemmTerm& t0) {
  GemmProb p{};
  p.c_id = c_id; p.c_off = c_off; p.M = M; p.N = N; p.ldc = ldc; p.nterm = 1; p.t[0] = t0;
  return p;
}
GemmProb prob2(int c_id, int64_t c_off, int M, int N, int ldc, const GemmTerm& t0, const GemmTerm& t1) {
  GemmProb p = prob(c_id, c_off, M, N, ldc, t0);
  p.nterm = 2;
  p.t[1] = t1;
  return p;
}

GemmProb probn(int c_id, int64_t c_off, int M, int N, int ldc, const std::vector<GemmTerm>& ts, int accum) {
  GemmProb p{};
  p.c_id = c_id; p.c_off = c_off; p.M = M; p.N = N; p.ldc = ldc; p.accum = accum;
  p.nterm = (int)ts.size();
  for (size_t i = 0; i < ts.size(); ++i) p.t[i] = ts[i];
  return p;
}

}  // namespace

// Problems of commutator_222_pp_hh (src/commutators.f90:596-766) for one channel block
// each; w1 and w2 are zeroed beforehand, as the reference does per block.
std::vector<GemmProb> build_pphh_problems(int nblocks, const std::vector<std::array<int, 3>>& ncls,
                                          const std::vector<int64_t>& goff) {
  std::vector<GemmProb> P;
  const int N = 0, T = 1;
  const int one = kAlphaOne, hl = kAlphaHL, hr = kAlphaHR, neg = kAlphaNeg;
  for (int q = 0; q < nblocks; ++q) {
    const int np = ncls[q][0], nb = ncls[q][1], nh = ncls[q][2];
    auto o = [&](int g) { return goff[q * 6 + g]; };
    // gam indices: 0 pppp 1 ppph 2 pphh 3 phph 4 hhhh 5 phhh
    if (np != 0)  // W1_pppp = L_pppp . R_pppp
      P.push_back(prob(kOpW1, o(0), np, np, np, term(kOpL, o(0), np, N, kOpR, o(0), np, N, np, one)));
    if (nh != 0)  // W2_hhhh = L_hhhh . R_hhhh
      P.push_back(prob(kOpW2, o(4), nh, nh, nh, term(kOpL, o(4), nh, N, kOpR, o(4), nh, N, nh, one)));
    if (np * nh != 0) {
      // W1_hhhh = hL * L_pphh^T . R_pphh
      P.push_back(prob(kOpW1, o(4), nh, nh, nh, term(kOpL, o(2), np, T, kOpR, o(2), np, N, np, hl)));
      // W2_pppp = hR * L_pphh . R_pphh^T
      P.push_back(prob(kOpW2, o(0), np, np, np, term(kOpL, o(2), np, N, kOpR, o(2), np, T, nh, hr)));
      // W1_pphh = L_pppp . R_pphh - R_pppp . L_pphh
      P.push_back(prob2(kOpW1, o(2), np, nh, np, term(kOpL, o(0), np, N, kOpR, o(2), np, N, np, one),
                        term(kOpR, o(0), np, N, kOpL, o(2), np, N, np, neg | one)));
      // W2_pphh = L_pphh . R_hhhh - R_pphh . L_hhhh
      P.push_back(prob2(kOpW2, o(2), np, nh, np, term(kOpL, o(2), np, N, kOpR, o(4), nh, N, nh, one),
                        term(kOpR, o(2), np, N, kOpL, o(4), nh, N, nh, neg | one)));
    }
    if (nb * nh != 0)  // W2_phph = hR * L_phhh . R_phhh^T
      P.push_back(prob(kOpW2, o(3), nb, nb, nb, term(kOpL, o(5), nb, N, kOpR, o(5), nb, T, nh, hr)));
    if (nb * np != 0)  // W1_phph = hL * L_ppph^T . R_ppph
      P.push_back(prob(kOpW1, o(3), nb, nb, nb, term(kOpL, o(1), np, T, kOpR, o(1), np, N, np, hl)));
    if (nb * nh != 0)  // W2_phhh = L_phhh . R_hhhh - R_phhh . L_hhhh
      P.push_back(prob2(kOpW2, o(5), nb, nh, nb, term(kOpL, o(5), nb, N, kOpR, o(4), nh, N, nh, one),
                        term(kOpR, o(5), nb, N, kOpL, o(4), nh, N, nh, neg | one)));
    if (nb * np != 0)  // W1_ppph = L_pppp . R_ppph - R_pppp . L_ppph
      P.push_back(prob2(kOpW1, o(1), np, nb, np, term(kOpL, o(0), np, N, kOpR, o(1), np, N, np, one),
                        term(kOpR, o(0), np, N, kOpL, o(1), np, N, np, neg | one)));
    if (nb * np * nh != 0) {
      // W1_phhh = hL * L_ppph^T . R_pphh - hR * R_ppph^T . L_pphh
      P.push_back(prob2(kOpW1, o(5), nb, nh, nb, term(kOpL, o(1), np, T, kOpR, o(2), np, N, np, hl),
                        term(kOpR, o(1), np, T, kOpL, o(2), np, N, np, neg | hr)));
      // W2_ppph = hR * L_pphh . R_phhh^T - hL * R_pphh . L_phhh^T
      P.push_back(prob2(kOpW2, o(1), np, nb, np, term(kOpL, o(2), np, N, kOpR, o(5), nb, T, nh, hr),
                        term(kOpR, o(2), np, N, kOpL, o(5), nb, T, nh, neg | hl)));
    }
  }
  return P;
}

// WCC(q) = LCC(q) . RCC(q)^T (src/commutators.f90:792-802)
std::vector<GemmProb> build_wcc_problems(int ncc, const std::vector<int>& rlen, const std::vector<int>& nph,
                                         const std::vector<int64_t>& cc_off, const std::vector<int64_t>& wcc_off) {
  std::vector<GemmProb> P;
  for (int q = 0; q < ncc; ++q) {
    const int r = rlen[q], nb = nph[q];
    if (r * nb == 0) continue;
    P.push_back(prob(kOpWCC, wcc_off[q], r, r, r, term(kOpLCC, cc_off[q], r, 0, kOpRCC, cc_off[q], r, 1, nb, kAlphaOne)));
  }
  return P;
}

// Reverse of build_pphh_problems: every product W = alpha op(X) op(Y) of the forward list
// gives Xbar += alpha Wbar op(Y)^T-like terms; the terms of one output block are summed in
// one problem (at most six, for the pphh blocks).
std::vector<GemmProb> build_pphh_vjp_problems(int nblocks, const std::vector<std::array<int, 3>>& ncls,
                                              const std::vector<int64_t>& goff) {
  std::vector<GemmProb> P;
  const int N = 0, T = 1;
  const int one = kAlphaOne, hl = kAlphaHL, hr = kAlphaHR, neg = kAlphaNeg;
  const int L = kOpL, R = kOpR, W1 = kOpW1, W2 = kOpW2;
  for (int q = 0; q < nblocks; ++q) {
    const int np = ncls[q][0], nb = ncls[q][1], nh = ncls[q][2];
    auto o = [&](int g) { return goff[q * 6 + g]; };
    std::vector<GemmTerm> t;
    auto emit = [&](int c_id, int g, int M, int Nn, int ldc) {
      if (M > 0 && Nn > 0 && !t.empty()) P.push_back(probn(c_id, o(g), M, Nn, ldc, t, 1));
      t.clear();
    };
    // pppp (np x np)
    if (np) t.push_back(term(W1, o(0), np, N, R, o(0), np, T, np, one));
    if (np * nh) t.push_back(term(W1, o(2), np, N, R, o(2), np, T, nh, one));
    if (np * nb) t.push_back(term(W1, o(1), np, N, R, o(1), np, T, nb, one));
    emit(L, 0, np, np, np);
    if (np) t.push_back(term(L, o(0), np, T, W1, o(0), np, N, np, one));
    if (np * nh) t.push_back(term(W1, o(2), np, N, L, o(2), np, T, nh, neg | one));
    if (np * nb) t.push_back(term(W1, o(1), np, N, L, o(1), np, T, nb, neg | one));
    emit(R, 0, np, np, np);
    // hhhh (nh x nh)
    if (nh) t.push_back(term(W2, o(4), nh, N, R, o(4), nh, T, nh, one));
    if (np * nh) t.push_back(term(R, o(2), np, T, W2, o(2), np, N, np, neg | one));
    if (nb * nh) t.push_back(term(R, o(5), nb, T, W2, o(5), nb, N, nb, neg | one));
    emit(L, 4, nh, nh, nh);
    if (nh) t.push_back(term(L, o(4), nh, T, W2, o(4), nh, N, nh, one));
    if (np * nh) t.push_back(term(L, o(2), np, T, W2, o(2), np, N, np, one));
    if (nb * nh) t.push_back(term(L, o(5), nb, T, W2, o(5), nb, N, nb, one));
    emit(R, 4, nh, nh, nh);
    // pphh (np x nh)
    if (np * nh) {
      t.push_back(term(R, o(2), np, N, W1, o(4), nh, T, nh, hl));
      t.push_back(term(W2, o(0), np, N, R, o(2), np, N, np, hr));
      t.push_back(term(R, o(0), np, T, W1, o(2), np, N, np, neg | one));
      t.push_back(term(W2, o(2), np, N, R, o(4), nh, T, nh, one));
      if (nb) {
        t.push_back(term(R, o(1), np, N, W1, o(5), nb, N, nb, neg | hr));
        t.push_back(term(W2, o(1), np, N, R, o(5), nb, N, nb, hr));
      }
      emit(L, 2, np, nh, np);
      t.push_back(term(L, o(2), np, N, W1, o(4), nh, N, nh, hl));
      t.push_back(term(W2, o(0), np, T, L, o(2), np, N, np, hr));
      t.push_back(term(L, o(0), np, T, W1, o(2), np, N, np, one));
      t.push_back(term(W2, o(2), np, N, L, o(4), nh, T, nh, neg | one));
      if (nb) {
        t.push_back(term(L, o(1), np, N, W1, o(5), nb, N, nb, hl));
        t.push_back(term(W2, o(1), np, N, L, o(5), nb, N, nb, neg | hl));
      }
      emit(R, 2, np, nh, np);
    }
    // phhh (nb x nh)
    if (nb * nh) {
      t.push_back(term(W2, o(3), nb, N, R, o(5), nb, N, nb, hr));
      t.push_back(term(W2, o(5), nb, N, R, o(4), nh, T, nh, one));
      if (np) t.push_back(term(W2, o(1), np, T, R, o(2), np, N, np, neg | hl));
      emit(L, 5, nb, nh, nb);
      t.push_back(term(W2, o(3), nb, T, L, o(5), nb, N, nb, hr));
      t.push_back(term(W2, o(5), nb, N, L, o(4), nh, T, nh, neg | one));
      if (np) t.push_back(term(W2, o(1), np, T, L, o(2), np, N, np, hr));
      emit(R, 5, nb, nh, nb);
    }
    // ppph (np x nb)
    if (np * nb) {
      t.push_back(term(R, o(1), np, N, W1, o(3), nb, T, nb, hl));
      t.push_back(term(R, o(0), np, T, W1, o(1), np, N, np, neg | one));
      if (nh) t.push_back(term(R, o(2), np, N, W1, o(5), nb, T, nh, hl));
      emit(L, 1, np, nb, np);
      t.push_back(term(L, o(1), np, N, W1, o(3), nb, N, nb, hl));
      t.push_back(term(L, o(0), np, T, W1, o(1), np, N, np, one));
      if (nh) t.push_back(term(L, o(2), np, N, W1, o(5), nb, T, nh, neg | hr));
      emit(R, 1, np, nb, np);
    }
  }
  return P;
}

std::vector<GemmProb> build_wcc_vjp_problems(int ncc, const std::vector<int>& rlen, const std::vector<int>& nph,
                                             const std::vector<int64_t>& cc_off, const std::vector<int64_t>& wcc_off) {
  std::vector<GemmProb> P;
  for (int q = 0; q < ncc; ++q) {
    const int r = rlen[q], nb = nph[q];
    if (r * nb == 0) continue;
    P.push_back(prob(kOpLCC, cc_off[q], r, nb, r, term(kOpWCC, wcc_off[q], r, 0, kOpRCC, cc_off[q], r, 0, r, kAlphaOne)));
    P.push_back(prob(kOpRCC, cc_off[q], r, nb, r, term(kOpWCC, wcc_off[q], r, 1, kOpLCC, cc_off[q], r, 0, r, kAlphaOne)));
  }
  return P;
}

// Output tiles, biggest problems (by K and size) first so the tail of the launch is short.
std::vector<GemmTile> build_tiles(const std::vector<GemmProb>& probs, int BM, int BN) {
  std::vector<GemmTile> tiles;
  for (int p = 0; p < (int)probs.size(); ++p)
    for (int m0 = 0; m0 < probs[p].M; m0 += BM)
      for (int n0 = 0; n0 < probs[p].N; n0 += BN) tiles.push_back(GemmTile{p, m0, n0, 0});
  auto work = [&](const GemmTile& t) {
    const GemmProb& p = probs[t.prob];
    int64_t k = 0;
    for (int i = 0; i < p.nterm; ++i) k += p.t[i].K;
    return k;
  };
  std::stable_sort(tiles.begin(), tiles.end(), [&](const GemmTile& a, const GemmTile& b) { return work(a) > work(b); });
  return tiles;
}

}  // namespace imsrg
