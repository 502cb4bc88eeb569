// Pair groups of the sq_op channels.  Orbits sharing (l, j, tz) form a block B (its orbits
// ascending); in channel (J, parity, Tz) the pairs (a in B1, b in B2), B1 <= B2, form a group.
// A one-body operator of the reference (f_elem, nonzero only inside a block) maps a group
// onto itself, so a commutator with one, or a change of one-body basis, acts on each
// group-pair sub-block (G1, G2) of a channel matrix separately: in the ordered-pair form
// V_A(ab,cd) that v_elem returns, as one-index products over a, b, c and d.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "layout.h"

namespace imsrg {

struct PairGroups {
  int nspb = 0, nmax = 0;
  std::vector<int> spb_start, spb_n, spb_orb, spb_j, spb_hole;  // per block; spb_orb ascending per block
  std::vector<int> orb_spb, orb_pos;                            // per orbit: block and position in it
  std::vector<int> grp_b1, grp_b2;                              // per group: its blocks (b1 <= b2)
  std::vector<int> grp_first;                                   // groups of channel q: [grp_first[q], grp_first[q+1])
  std::vector<int> blk_off;                                     // per block: offset of its n x n matrix
  int nblk2 = 0;                                                // sum of n^2 over the blocks
  // elements n(B1) n(B2) n(B3) n(B4) of the ordered four-index sub-block of group pair (G1, G2)
  int64_t elems(int G1, int G2) const {
    return (int64_t)spb_n[grp_b1[G1]] * spb_n[grp_b2[G1]] * spb_n[grp_b1[G2]] * spb_n[grp_b2[G2]];
  }
};

void build_pair_groups(PairGroups& G, const Layout& L);

// device view used by the group kernels
struct PairGroupsDev {
  const int* spb_start;
  const int* spb_n;
  const int* spb_orb;
  const int* grp_b1;
  const int* grp_b2;
  const int* blk_off;
  const int4* tasks;  // (channel q, group 1, group 2, unused), group 1 <= group 2
};

}  // namespace imsrg
