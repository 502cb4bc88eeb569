// commutator_122 (src/commutators.f90:283-396) of the mixed path, FP32, by pair-group
// sub-blocks.  Orbits sharing (l, j, tz) form a block; in channel q the pairs (a in B1,
// b in B2) form a group G.  The one-body factors only mix orbits of one block, so on a
// group-pair sub-block (G1, G2) of the ordered-pair form V_A(ab, cd) (what v_elem returns)
// the result is four one-index products:
//   OUT[a,b,c,d] = sum_a' fL(a,a') R_A[a',b,c,d] - fR(a,a') L_A[a',b,c,d]   (and b)
//                - sum_c' fL(c',c) R_A[a,b,c',d] - fR(c',c) L_A[a,b,c',d]   (and d)
// Each element of L and R is gathered once per sub-block into shared memory as an (L, R)
// pair, and every stored element of the sub-block is written once (ASSIGNS), mirrored with
// hRES when G1 != G2, except the lower triangles of the square arrays (pppp, phph, hhhh):
// the mirror pass at the end of the commutator writes those from the upper triangles.
//
// Everything that depends on the basis alone is on the host: per element of every sub-block
// one code word (comm122.h) with its storage position, swap flag and factor (V_A = pre x
// stored: sqrt 2 per pair of identical orbits, the exchange phase when a pair's stored order is
// swapped), per task the block sizes, the offsets of the f blocks and the constants of the
// index divisions.  Every element is read from, and written to, the same place: the
// rectangular array of its class pair, or the upper triangle of a square array (the operators'
// lower triangles are herm times the upper ones, and the pass after the recoupling writes
// RES's lower triangles).  One launch covers every
// task: the largest sub-blocks one per CTA at the front of the grid, the rest as runs of tasks
// that the warps take in channel order from a counter, so the tasks of one channel (which
// read the same arrays of L and R) run close together in time.
#include "comm122.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace imsrg {

namespace {

__device__ __forceinline__ int g122_div(int e, int m) { return (int)(((unsigned)e * (unsigned)m) >> 20); }

// pre and 1 / pre of a code word
__device__ __forceinline__ float g122_pre(unsigned w) {
  const unsigned m = w >> 30;
  const float v = m == 0 ? 1.0f : (m == 1 ? 1.41421356f : 2.0f);
  return (w >> 29) & 1u ? -v : v;
}
__device__ __forceinline__ float g122_ipre(unsigned w) {
  const unsigned m = w >> 30;
  const float v = m == 0 ? 1.0f : (m == 1 ? 0.70710678f : 0.5f);
  return (w >> 29) & 1u ? -v : v;
}

// the (L, R) pair of V_A of one element from its code word and stored values
__device__ __forceinline__ float2 g122_va(unsigned w, double l, double r, int hL, int hR) {
  const bool sw = (w & (1u << kG122IdxBits)) != 0;
  const float pre = g122_pre(w);
  return make_float2(f64_to_f32(l) * ((sw && hL < 0) ? -pre : pre), f64_to_f32(r) * ((sw && hR < 0) ? -pre : pre));
}

__device__ __forceinline__ void g122_sync(bool cta, unsigned mask) {
  if (cta) __syncthreads(); else __syncwarp(mask);
}

// One task on nth threads: 8 or 32 lanes of a warp (under mask), or the whole CTA (cta).  One
// copy of this code serves all three, so the warps of a CTA share their instructions.
__device__ __forceinline__ void g122_run(const DevLayout& D, const G122Task& t, const unsigned* __restrict__ EC,
                                         const double* __restrict__ L, int hL, const double* __restrict__ R, int hR,
                                         double* __restrict__ RES, int hRES, const float2* __restrict__ FB,
                                         float2* __restrict__ X, int tid, int nth, bool cta, unsigned mask) {
  const int n0 = t.nn & 255, n1 = (t.nn >> 8) & 255, n2 = (t.nn >> 16) & 255, n3 = t.nn >> 24;
  const int nb = n0 * n1, ntot = nb * n2 * n3;
  const unsigned* C = EC + t.eoff;
  constexpr unsigned kIdx = (1u << kG122IdxBits) - 1u, kSwap = 1u << kG122IdxBits;
  // gather V_A of L and R, two elements per pass so that two chains of dependent loads are in flight
  int e = tid;
  for (; e + nth < ntot; e += 2 * nth) {
    const unsigned w0 = __ldg(C + e), w1 = __ldg(C + e + nth);
    const double l0 = __ldg(L + (w0 & kIdx)), r0 = __ldg(R + (w0 & kIdx));
    const double l1 = __ldg(L + (w1 & kIdx)), r1 = __ldg(R + (w1 & kIdx));
    X[e] = g122_va(w0, l0, r0, hL, hR);
    X[e + nth] = g122_va(w1, l1, r1, hL, hR);
  }
  if (e < ntot) {
    const unsigned w = __ldg(C + e);
    X[e] = g122_va(w, __ldg(L + (w & kIdx)), __ldg(R + (w & kIdx)), hL, hR);
  }
  g122_sync(cta, mask);
  const int s1 = n0, s2 = nb, s3 = nb * n2;
  const float2* F0 = FB + t.fb[0];
  const float2* F1 = FB + t.fb[1];
  const float2* F2 = FB + t.fb[2];
  const float2* F3 = FB + t.fb[3];
  for (int e = tid; e < ntot; e += nth) {
    const int ek = g122_div(e, t.mb), eb = e - ek * nb;
    const int x1 = g122_div(eb, t.m0), x0 = eb - x1 * n0;
    const int x3 = g122_div(ek, t.m2), x2 = ek - x3 * n2;
    if (((t.flags & 2) && x0 > x1) || ((t.flags & 4) && x2 > x3)) continue;  // the other order is stored
    // written at the code word's position, times hRES when swapped; for G1 == G2 a swapped
    // element's transposed twin of this sub-block writes it
    const unsigned w = __ldg(C + e);
    const bool sw = (w & kSwap) != 0;
    if (sw && !(t.flags & 1)) continue;
    float out = 0.0f;
    {  // sum_a' f(a, a') X[a', ...]
      const float2* f = F0 + x0 * n0;
      const float2* xp = X + (e - x0);
      for (int a = 0; a < n0; ++a) {
        const float2 fv = __ldg(f + a), xv = xp[a];
        out = fmaf(fv.x, xv.y, out);
        out = fmaf(-fv.y, xv.x, out);
      }
    }
    {
      const float2* f = F1 + x1 * n1;
      const float2* xp = X + (e - x1 * s1);
      for (int a = 0; a < n1; ++a) {
        const float2 fv = __ldg(f + a), xv = xp[a * s1];
        out = fmaf(fv.x, xv.y, out);
        out = fmaf(-fv.y, xv.x, out);
      }
    }
    {  // - sum_c' f(c', c) X[..., c', ...]
      const float2* f = F2 + x2;
      const float2* xp = X + (e - x2 * s2);
      for (int a = 0; a < n2; ++a) {
        const float2 fv = __ldg(f + a * n2), xv = xp[a * s2];
        out = fmaf(-fv.x, xv.y, out);
        out = fmaf(fv.y, xv.x, out);
      }
    }
    {
      const float2* f = F3 + x3;
      const float2* xp = X + (e - x3 * s3);
      for (int a = 0; a < n3; ++a) {
        const float2 fv = __ldg(f + a * n3), xv = xp[a * s3];
        out = fmaf(-fv.x, xv.y, out);
        out = fmaf(fv.y, xv.x, out);
      }
    }
    const float v = out * g122_ipre(w);  // stored = V_A / pre
    RES[w & kIdx] = f32_to_f64((sw && hRES < 0) ? -v : v);
  }
  g122_sync(cta, mask);
}

// blocks [0, nbig): one big task each on the whole CTA; the other blocks: eight warps, each with
// a slice of slice_f2 (L, R) pairs (four sub-slices of sub_f2 for the 8-lane groups), taking
// runs of tasks from the counter until none is left
__global__ void __launch_bounds__(kG122Threads, 5) k_comm122_sub(DevLayout D, const G122Task* __restrict__ tasks,
                                                              const int2* __restrict__ items, int nitems, int nbig,
                                                              int* counter, const unsigned* __restrict__ EC,
                                                              int slice_f2, int sub_f2, const double* __restrict__ L,
                                                              int hL, const double* __restrict__ R, int hR,
                                                              double* __restrict__ RES, int hRES,
                                                              const float2* __restrict__ FB) {
  extern __shared__ float2 g122_x[];
  if ((int)blockIdx.x < nbig) {
    const G122Task t = tasks[blockIdx.x];
    g122_run(D, t, EC, L, hL, R, hR, RES, hRES, FB, g122_x, threadIdx.x, kG122Threads, true, 0u);
    return;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2* slice = g122_x + (size_t)warp * slice_f2;
  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(counter, 1);
    it = __shfl_sync(0xffffffffu, it, 0);
    if (it >= nitems) break;
    const int2 w = __ldg(items + it);
    const int cnt = w.y & 0xFFFF;
    // four 8-lane groups (task k on group k mod 4) or the whole warp (one task after another)
    const bool quad = (w.y >> 16) == 0;
    const int grp = quad ? lane >> 3 : 0, nth = quad ? 8 : 32, step = quad ? 4 : 1;
    const unsigned mask = quad ? 0xFFu << (grp * 8) : 0xffffffffu;
    for (int k = grp; k < cnt; k += step) {
      const G122Task t = tasks[w.x + k];
      g122_run(D, t, EC, L, hL, R, hR, RES, hRES, FB, slice + grp * sub_f2, lane & (nth - 1), nth, false, mask);
    }
    __syncwarp();
  }
}

}  // namespace

__global__ void k_comm122_fb2(DevLayout D, PairGroupsDev G, int nspb, const double* __restrict__ L, int hL,
                              const double* __restrict__ R, int hR, float2* __restrict__ FB, int* counter) {
  const int B = blockIdx.x;
  if (B == 0 && threadIdx.x == 0) *counter = 0;
  if (B >= nspb) return;
  const int n = G.spb_n[B];
  const int* o = G.spb_orb + G.spb_start[B];
  for (int r = threadIdx.x; r < n * n; r += blockDim.x) {
    const int x = r / n, y = r - (r / n) * n;
    FB[G.blk_off[B] + r] = make_float2(d_f_elem_f(D, L, hL, o[x], o[y]), d_f_elem_f(D, R, hR, o[x], o[y]));
  }
}

void launch_comm122(int grid, size_t smem, cudaStream_t st, const DevLayout& D, const G122Task* tasks,
                    const int2* items, int nitems, int nbig, int* counter, const unsigned* codes, int slice_f2, int sub_f2,
                    const double* L, int hL, const double* R, int hR, double* RES, int hRES, const float2* FB) {
  k_comm122_sub<<<grid, kG122Threads, smem, st>>>(D, tasks, items, nitems, nbig, counter, codes, slice_f2, sub_f2, L,
                                                  hL, R, hR, RES, hRES, FB);
}

cudaError_t g122_smem_attr(size_t smem) {
  return cudaFuncSetAttribute(k_comm122_sub, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t g122_blocks_per_sm(size_t smem, int* n) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, k_comm122_sub, kG122Threads, smem);
}

size_t g122_smem_bytes(int tiny_cap, int warp_cap, int nmax4) {
  const size_t warp = (size_t)std::max(warp_cap, 4 * tiny_cap);
  return sizeof(float2) * std::max(warp * (kG122Threads / 32), (size_t)nmax4);
}

std::string build_g122_plan(const Layout& L, const PairGroups& G, G122Plan& P) {
  P = G122Plan();
  const int N = L.N, NJ = L.NJ;
  if (L.slab >= (int64_t)1 << kG122IdxBits) return "122 plan: operator slab too large for 28-bit positions";
  // the ordered pairs of every group, in the channel's J: stored position, class, and the
  // factor pre (sqrt 2 for identical orbits, the exchange phase when the stored order is swapped)
  struct PairInfo {
    int pos, cls;
    int sign, sq;  // pre = (sign ? -1 : 1) * (sq ? sqrt 2 : 1)
  };
  const int ngrp = (int)G.grp_b1.size();
  std::vector<int> grp_off(ngrp, 0);
  std::vector<PairInfo> pairs;
  for (int q = 0; q < L.nblocks; ++q) {
    const int J = L.lamJ[q];
    for (int g = G.grp_first[q]; g < G.grp_first[q + 1]; ++g) {
      grp_off[g] = (int)pairs.size();
      const int B1 = G.grp_b1[g], B2 = G.grp_b2[g], na = G.spb_n[B1], nb = G.spb_n[B2];
      for (int y = 0; y < na * nb; ++y) {
        const int oa = G.spb_orb[G.spb_start[B1] + y % na], ob = G.spb_orb[G.spb_start[B2] + y / na];
        const int lo = std::min(oa, ob), hi = std::max(oa, ob);
        PairInfo pi{};
        pi.sq = oa == ob;
        pi.sign = oa > ob && ((1 + ((L.jj[oa] + L.jj[ob] - J) >> 1)) & 1);
        pi.pos = L.pairpos[((size_t)lo * N + hi) * NJ + J / 2];
        pi.cls = L.con[lo] + L.con[hi];
        if (pi.pos < 0) return "122 plan: a group pair is not in its channel";
        pairs.push_back(pi);
      }
    }
  }
  // the group-pair tasks G1 <= G2 of every channel, and the code words of their elements
  auto magic = [](int n) { return (int)(((1u << 20) + (unsigned)n - 1u) / (unsigned)n); };
  static const int kArray[3][3] = {{0, 1, 2}, {1, 3, 5}, {2, 5, 4}};  // gam array of a class pair
  for (int q = 0; q < L.nblocks; ++q)
    for (int G2 = G.grp_first[q]; G2 < G.grp_first[q + 1]; ++G2)
      for (int G1 = G.grp_first[q]; G1 <= G2; ++G1) {
        const int b[4] = {G.grp_b1[G1], G.grp_b2[G1], G.grp_b1[G2], G.grp_b2[G2]};
        const int n[4] = {G.spb_n[b[0]], G.spb_n[b[1]], G.spb_n[b[2]], G.spb_n[b[3]]};
        const int64_t el = (int64_t)n[0] * n[1] * n[2] * n[3];
        if (el > kG122MaxElems || n[0] * n[1] > 255 || n[2] * n[3] > 255)
          return "122 plan: a sub-block exceeds 4095 elements (eMax too large)";
        if (P.codes.size() + (size_t)el >= ((size_t)1 << 31)) return "122 plan: element table too large";
        G122Task t{};
        t.eoff = (int)P.codes.size();
        t.q = q;
        t.nn = (unsigned)n[0] | (unsigned)n[1] << 8 | (unsigned)n[2] << 16 | (unsigned)n[3] << 24;
        for (int x = 0; x < 4; ++x) t.fb[x] = G.blk_off[b[x]];
        t.m0 = magic(n[0]);
        t.m2 = magic(n[2]);
        t.mb = magic(n[0] * n[1]);
        t.flags = (G1 != G2 ? 1 : 0) | (b[0] == b[1] ? 2 : 0) | (b[2] == b[3] ? 4 : 0);
        const int nbra = n[0] * n[1];
        for (int64_t e = 0; e < el; ++e) {
          const PairInfo& pb = pairs[grp_off[G1] + (int)(e % nbra)];
          const PairInfo& pk = pairs[grp_off[G2] + (int)(e / nbra)];
          // the stored element: rectangular array of the class pair, or a square array's upper
          // triangle; swapped when the element is herm times it
          const bool sw = pb.cls > pk.cls || (pb.cls == pk.cls && pb.pos > pk.pos);
          const int row = sw ? pk.pos : pb.pos, col = sw ? pb.pos : pk.pos;
          const int k = q * 6 + kArray[pb.cls][pk.cls];
          const int64_t idx = L.goff[k] + row + (int64_t)col * L.gn1[k];
          const int sq = pb.sq + pk.sq;  // pre = (-1)^sign x sqrt 2^sq
          P.codes.push_back((unsigned)idx | (sw ? 1u : 0u) << kG122IdxBits | (unsigned)(pb.sign ^ pk.sign) << 29 |
                            (unsigned)sq << 30);
        }
        P.all.push_back(t);
        P.elems.push_back(el);
        P.nmax4 = std::max<int>(P.nmax4, (int)el);
      }
  return "";
}

std::string g122_partition(G122Plan& P, int tiny_cap, int warp_cap) {
  if (tiny_cap < 1 || warp_cap < tiny_cap || warp_cap > kG122MaxElems) return "122 task caps out of range";
  P.tasks.clear();
  P.items.clear();
  const size_t n = P.all.size();
  {  // big tasks first, one CTA each, largest first
    std::vector<size_t> big;
    for (size_t i = 0; i < n; ++i)
      if (P.elems[i] > warp_cap) big.push_back(i);
    std::stable_sort(big.begin(), big.end(), [&](size_t a, size_t b) { return P.elems[a] > P.elems[b]; });
    for (size_t k : big) P.tasks.push_back(P.all[k]);
  }
  P.nbig = (int)P.tasks.size();
  // warp work, channel by channel: runs of up to 16 small tasks (four at a time on 8-lane
  // groups, similar sizes together) and runs of warp tasks of about 512 elements
  size_t i = 0;
  while (i < n) {
    const int q = P.all[i].q;
    size_t j = i;
    while (j < n && P.all[j].q == q) ++j;
    std::vector<size_t> tiny, warp;
    for (size_t k = i; k < j; ++k) {
      if (P.elems[k] <= tiny_cap) tiny.push_back(k);
      else if (P.elems[k] <= warp_cap) warp.push_back(k);
    }
    // equal sizes and block shapes side by side: the four tasks of a quad then run their loops
    // in step
    std::stable_sort(tiny.begin(), tiny.end(), [&](size_t a, size_t b) {
      return P.elems[a] != P.elems[b] ? P.elems[a] > P.elems[b] : P.all[a].nn < P.all[b].nn;
    });
    for (size_t k = 0; k < tiny.size(); k += 16) {
      const size_t e = std::min(tiny.size(), k + 16);
      P.items.push_back(make_int2((int)P.tasks.size(), (int)(e - k)));
      for (size_t m = k; m < e; ++m) P.tasks.push_back(P.all[tiny[m]]);
    }
    for (size_t k = 0; k < warp.size();) {
      int64_t sum = 0;
      size_t e = k;
      while (e < warp.size() && e - k < 4 && sum < 512) sum += P.elems[warp[e++]];
      P.items.push_back(make_int2((int)P.tasks.size(), (int)(e - k) | 1 << 16));
      for (size_t m = k; m < e; ++m) P.tasks.push_back(P.all[warp[m]]);
      k = e;
    }
    i = j;
  }
  P.tiny_cap = tiny_cap;
  P.warp_cap = warp_cap;
  P.smem_bytes = g122_smem_bytes(tiny_cap, warp_cap, P.nmax4);
  if (P.smem_bytes > 200 * 1024) return "122 task caps need too much shared memory";
  return "";
}

}  // namespace imsrg
