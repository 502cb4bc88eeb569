// Rank-lambda tensor operators: the operand of BCH_TENSOR (src/IMSRG_MAGNUS.f90:389-464).
//
// Layout of allocate_tensor (src/basic_IMSRG.f90:688-951) as one FP64 slab per operator:
//   [E0][fhh A*A][fpp P*P][fph P*A][ block q = (J1 <= J2, Tz, bra parity P1): tgam(1..9) ]
// tgam(g) holds the (bra class, ket class) matrix (pp,pp) (pp,ph) (pp,hh) (ph,ph) (hh,hh)
// (ph,hh) (hh,pp) (ph,pp) (hh,ph), column-major; bra pairs come from the scalar channel
// (J1, Tz, P1) and ket pairs from (J2, Tz, P2), P2 = P1 xor dpar/2 (rank and dpar doubled).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "dev.cuh"
#include "gemm.h"
#include "layout.h"

namespace imsrg {

struct TLayout {
  int rank = 0, dpar = 0, nblocks = 0;
  std::vector<int> J1, J2, T, P1, P2, q1, q2;  // q1/q2: scalar channels of bra/ket pairs (-1: empty block)
  std::vector<int64_t> goff;                   // [q*9+g]
  std::vector<int> n1, n2;                     // [q*9+g]
  std::vector<int> lut;                        // [((J1/2)*(rank/2+1) + (J2-J1)/2)*6 + (Tz+1)*2 + P1] -> q
  int64_t off_fhh = 1, off_fpp = 0, off_fph = 0, slab = 0;
  int64_t n2b = 0;                             // two-body elements (slab - goff[0])
  // one-body outputs of a tensor commutator: kind 0 fhh (p<=q), 1 fpp (p<=q), 2 fph
  std::vector<int> ob_kind, ob_p, ob_q, ob_pk, ob_qk;
  // 6j {J1 J2 rank; j4 j5 j6}, J1, J2 integer, j4..j6 half-integer, j4 up to jmax + rank
  // (the 9j sums reach there), j5, j6 up to jmax:
  // six[(((J1/2)*nJ + J2/2)*nhx + (j4-1)/2)*nh*nh + ((j5-1)/2)*nh + (j6-1)/2]
  int six_nJ = 0, six_nh = 0, six_nhx = 0;
  std::vector<double> six;
  // 6j {c d J2; b x J4} of the 9j sums, c, d, b up to jmax, x up to jmax + rank:
  // six_m[((((c-1)/2*nh + (d-1)/2)*nh + (b-1)/2)*nhx + (x-1)/2)*nJ*nJ + (J2/2)*nJ + J4/2]
  std::vector<double> six_m;
  std::vector<int> ccnb;  // [(p*N+h)*NJ + JC/2] -> ph column of (p,h) in its cross-coupled channel, -1
  // orbits i a tensor one-body element f(a,i) can couple: same tz, parity l_i + dpar/2 = l_a, |j_i - j_a| <= rank
  std::vector<int> tnb_start, tnb_count, tnb_list;
  // cross-coupled tensor blocks of TS_commutator_222_ph: (J3, J4 >= J3, Tz 0/1, PAR) and their
  // scalar cross-coupled channels qa (J3, Tz, PAR), qb (J4, Tz, PAR xor dpar/2)
  std::vector<int> cb_J3, cb_J4, cb_Tz, cb_PAR, cb_qa, cb_qb;
  int64_t cb_max_w = 0, cb_max_x = 0, cb_max_r = 0;  // largest r1*r2, r1*nb2 / nb1*r2, r
  // Frobenius-norm segments (weight 1 for fhh, fpp and J1 == J2 blocks, 2 otherwise)
  std::vector<int64_t> seg_start;
  std::vector<int> seg_len;
  std::vector<int8_t> seg_w;

  int block(int j1, int j2, int t, int p, int JM) const {
    if (j2 < j1 || j2 - j1 > rank || j1 > 2 * JM) return -1;
    return lut[(((size_t)(j1 / 2) * (rank / 2 + 1) + (j2 - j1) / 2) * 3 + (t + 1)) * 2 + p];
  }
};

// Builds the tensor layout on top of the scalar one; empty string or the reason it failed.
std::string build_tlayout(TLayout& T, const Layout& L, int rank, int dpar);

// TS_commutator_222_pp_hh's products as grouped-GEMM problems: per block and class pair,
// W1 = L(q1)[c1,pp] R[pp,c2] - R[c1,pp] L(q2)[pp,c2] and W2 the same through hh pairs
// (operands: kOpL scalar L, kOpR tensor R, outputs kOpW1 / kOpW2 in tensor layout)
// excitation_only keeps the terms whose R operand is a (pp,hh) or (hh,pp) array (the other
// arrays of an EOM ladder operator are zero)
std::vector<GemmProb> build_tensor_pphh_problems(const TLayout& T, const Layout& L, bool excitation_only = false);

// a subset of the two-body elements of a tensor slab for the per-element kernels: segment s
// covers elements off[s] .. off[s] + (pre[s+1] - pre[s]) - 1 (relative to goff[0]); n = 0 means all
struct ElemSegs {
  const int64_t* off = nullptr;
  const int64_t* pre = nullptr;
  int n = 0;
};

// one cross-coupled tensor block of the excitation-mode particle-hole products: packed CCR
// (nb1 x nx) over the (particle, hole) rows of qb listed from xs, packed CCX (ny x nb2) over the
// (hole, particle) rows of qa listed from ys, and the offsets of CCR, CCX, Wx (r1 x nx) and
// Wy (ny x r2) in their buffers (nx = 0 / ny = 0: no Wx / Wy)
struct ExcBlock {
  int J3, J4, qa, qb, nx, ny, xs, ys;
  int64_t ccr, ccx, wx, wy;
};

struct DevTLayout {
  int rank, dpar, nblocks, n_ob, six_nJ, six_nh, six_nhx;
  int64_t off_fhh, off_fpp, off_fph, slab, n2b;
  const int* J1;
  const int* J2;
  const int* q1;
  const int* q2;
  const int* lut;
  const int64_t* goff;
  const int* n1;
  const int* n2;
  const int* ob_kind;
  const int* ob_p;
  const int* ob_q;
  const int* ob_pk;
  const int* ob_qk;
  const double* six;
  const double* six_m;
  const float* six_f;  // six in FP32
  const int* ccnb;
  const int* tnb_start;
  const int* tnb_count;
  const int* tnb_list;
};

}  // namespace imsrg
