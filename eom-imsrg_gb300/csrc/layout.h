// Host-side description of one j-scheme basis and of every table the commutator
// kernels read: the reference's sq_op channel layout (src/basic_IMSRG.f90:521-685),
// its cross-coupled channel layout (src/cross_coupled.f90:61-177), dense pair->index
// maps that replace the reference's xmap / rmap linear searches, and a compact 6j table.
#pragma once
#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace imsrg {

// storage classes of a pair: 0 = pp, 1 = ph, 2 = hh;  arrays g = 0..5 are the
// reference's gam(1..6): pppp ppph pphh phph hhhh phhh
constexpr int kSea1[6] = {0, 0, 0, 1, 2, 1};
constexpr int kSea2[6] = {0, 1, 2, 1, 2, 2};
constexpr bool kSquare[6] = {true, false, false, true, true, false};

struct Layout {
  // orbits
  int N = 0, A = 0, P = 0, JM = 0, NJ = 0, lmax = 0, eMax = 0, Aprot = 0, Aneut = 0;
  double hw = 0;
  std::vector<int> nn, ll, jj, tz, con, loc, holes, parts;
  std::vector<int> same_start, same_count, same_list;  // orbits sharing (j, l, tz)

  // sq_op channels: q = 3*(2J) + 2*(Tz+1) + Par
  int nblocks = 0;
  std::vector<int> lamJ, lamP, lamT;
  std::vector<std::array<int, 3>> ncls;
  std::vector<int> pair_off;            // [q*3+cls] start in pair_a/pair_b
  std::vector<int16_t> pair_a, pair_b;  // pair lists (first orbit <= second)
  std::vector<int> pairpos;             // [(a*N+b)*NJ + J/2], a <= b; -1 if not a member

  // FP64 slab: [E0][fhh A*A][fpp P*P][fph P*A][blocks q, arrays g], column-major
  int64_t off_fhh = 1, off_fpp = 0, off_fph = 0, slab = 0;
  std::vector<int64_t> goff;           // [q*6+g]
  std::vector<int> gn1, gn2;           // [q*6+g]
  // unique 2b elements (upper triangle incl. diagonal for square arrays), per (q,g)
  std::vector<int64_t> uoff;           // [q*6+g] prefix, size nblocks*6+1
  int64_t n_unique = 0;

  // cross-coupled channels: q = JC/2 + Tz*(JM+1) + Par*2*(JM+1)
  int ncc = 0;
  std::vector<int> cc_rlen, cc_nph, cc_J;
  std::vector<int64_t> cc_off, wcc_off;   // sizes cc_off[ncc] == cc_size
  int64_t cc_size = 0, wcc_size = 0;
  std::vector<int> cc_row_off, cc_col_off;  // [q] into cc_ra/cc_rb and cc_cp/cc_ch
  std::vector<int16_t> cc_ra, cc_rb, cc_cp, cc_ch;
  std::vector<int> ccr;                   // [(a*N+b)*NJ + JC/2] -> row index r; -1 if absent

  // one-body outputs of 121/221: (kind, local p, local q, orbit p, orbit q)
  // kind 0 = fhh (p<=q), 1 = fpp (p<=q), 2 = fph
  std::vector<int> ob_kind, ob_p, ob_q, ob_pk, ob_qk;
  // (particle a, hole i) pairs sharing (j, l, tz), local indices, a outer / i inner
  std::vector<int> ai_a, ai_i;

  // 6j table, one block per (j1,j2,j4,j5) half-integer quadruple
  int sj_nh = 0;
  std::vector<int> sj_off, sj_j3min, sj_j6min, sj_n6;
  std::vector<double> sj_val;

  int block(int J2, int T, int Par) const { return 3 * J2 + 2 * (T + 1) + Par; }
  int ccq(int JC, int TZ, int PAR) const { return JC / 2 + TZ * (JM + 1) + PAR * 2 * (JM + 1); }
};

// Builds the layout; returns an empty string or a description of bad input.
std::string build_layout(Layout& L, int N, const int* nn, const int* ll, const int* jj, const int* tz,
                         const int* con, int eMax, double hw, int Aprot, int Aneut);

double sixj_racah(int j1, int j2, int j3, int j4, int j5, int j6);

// host accessors on an FP64 slab (used by input preparation)
double host_f_elem(const Layout& L, const double* op, int herm, int a, int b);
double host_v_elem(const Layout& L, const double* op, int herm, int a, int b, int c, int d, int J);

}  // namespace imsrg
