// Grouped GEMM problem lists shared by the FP64 and the tensor-core paths.
//
// A problem is C (+)= sum_t alpha_t * op(A_t) * op(B_t) with at most kMaxTerms terms, every
// matrix column-major and addressed as (operand id, element offset) so that one list,
// built once per basis, serves any set of operator slabs.  alpha_t is +-1, +-herm(L)
// or +-herm(R), resolved at launch time.
#pragma once
#include <array>
#include <cstdint>
#include <vector>

namespace imsrg {

enum OperandId : int { kOpL = 0, kOpR = 1, kOpW1 = 2, kOpW2 = 3, kOpLCC = 4, kOpRCC = 5, kOpWCC = 6, kNumOperands = 8 };

// alpha codes: bits 0-1 select 1 / hL / hR, bit 2 negates
enum AlphaCode : int { kAlphaOne = 0, kAlphaHL = 1, kAlphaHR = 2, kAlphaNeg = 4 };

struct GemmTerm {
  int64_t a_off, b_off;
  int a_id, b_id;
  int lda, ldb;
  int K;
  int ta, tb;  // 0 = 'N', 1 = 'T'
  int alpha;   // AlphaCode
};

constexpr int kMaxTerms = 6;

struct GemmProb {
  int64_t c_off;
  int M, N;
  int ldc;
  int c_id;
  int nterm;
  int accum;  // 0: C = sum, 1: C += sum
  GemmTerm t[kMaxTerms];
};

struct GemmTile {
  int prob, m0, n0, pad;
};

struct GemmOperands {
  const double* in[kNumOperands];
  double* out[kNumOperands];
  int hL, hR;
};

// the reference's per-channel dgemm sequence of commutator_222_pp_hh
// (src/commutators.f90:596-766), as independent problems writing w1 / w2
std::vector<GemmProb> build_pphh_problems(int nblocks, const std::vector<std::array<int, 3>>& ncls,
                                          const std::vector<int64_t>& goff);
std::vector<GemmProb> build_wcc_problems(int ncc, const std::vector<int>& rlen, const std::vector<int>& nph,
                                         const std::vector<int64_t>& cc_off, const std::vector<int64_t>& wcc_off);
// transposes for the adjoint: with w1 / w2 holding the cotangents of the pphh products,
// Lb and Rb (operands kOpL / kOpR of the output side) accumulate d<cotangent, W>/dL, dR
std::vector<GemmProb> build_pphh_vjp_problems(int nblocks, const std::vector<std::array<int, 3>>& ncls,
                                              const std::vector<int64_t>& goff);
// LCCb = WCCb . RCC and RCCb = WCCb^T . LCC per cross-coupled channel (assigned)
std::vector<GemmProb> build_wcc_vjp_problems(int ncc, const std::vector<int>& rlen, const std::vector<int>& nph,
                                             const std::vector<int64_t>& cc_off, const std::vector<int64_t>& wcc_off);
std::vector<GemmTile> build_tiles(const std::vector<GemmProb>& probs, int BM, int BN);

}  // namespace imsrg
