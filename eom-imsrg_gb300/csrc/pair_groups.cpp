// Blocks of orbits sharing (l, j, tz) and the pair groups of every channel (pair_groups.h).
#include "pair_groups.h"

#include <algorithm>
#include <cstdlib>

namespace imsrg {

void build_pair_groups(PairGroups& G, const Layout& L) {
  G = PairGroups();
  const int N = L.N;
  G.orb_spb.assign(N, -1);
  G.orb_pos.assign(N, 0);
  for (int i = 0; i < N; ++i) {  // blocks in order of their first orbit
    if (G.orb_spb[i] >= 0) continue;
    const int B = G.nspb++;
    G.spb_start.push_back((int)G.spb_orb.size());
    G.spb_j.push_back(L.jj[i]);
    int n = 0, holes = 0;
    for (int k = i; k < N; ++k)
      if (L.ll[k] == L.ll[i] && L.jj[k] == L.jj[i] && L.tz[k] == L.tz[i]) {
        G.orb_spb[k] = B;
        G.orb_pos[k] = n++;
        G.spb_orb.push_back(k);
        holes += L.con[k];
      }
    G.spb_n.push_back(n);
    G.spb_hole.push_back(holes > 0);
    G.nmax = std::max(G.nmax, n);
    G.blk_off.push_back(G.nblk2);
    G.nblk2 += n * n;
  }
  // groups of a channel: block pairs whose j's couple to J with the channel's parity and Tz
  G.grp_first.assign(L.nblocks + 1, 0);
  for (int q = 0; q < L.nblocks; ++q) {
    G.grp_first[q] = (int)G.grp_b1.size();
    const int J = L.lamJ[q], P = L.lamP[q], T = L.lamT[q];
    for (int B1 = 0; B1 < G.nspb; ++B1)
      for (int B2 = B1; B2 < G.nspb; ++B2) {
        const int a = G.spb_orb[G.spb_start[B1]], b = G.spb_orb[G.spb_start[B2]];
        if ((L.ll[a] + L.ll[b]) % 2 != P || L.tz[a] + L.tz[b] != 2 * T) continue;
        if (J > L.jj[a] + L.jj[b] || J < std::abs(L.jj[a] - L.jj[b])) continue;
        G.grp_b1.push_back(B1);
        G.grp_b2.push_back(B2);
      }
  }
  G.grp_first[L.nblocks] = (int)G.grp_b1.size();
}

}  // namespace imsrg
