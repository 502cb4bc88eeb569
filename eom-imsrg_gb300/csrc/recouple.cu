// commutator_222_ph recoupling (src/commutators.f90:804-921) of the mixed-precision path, by
// (i, k, l) groups.
//
// The reference gathers, for every stored element (ij, kl; J) and every J' shared by the
// pairs, four cross-coupled products W_{gik,rjl} etc. and sums them with 6j symbols.  Here
// the particle-hole GEMM (gemm_tc.cu) writes one FP32 matrix per cross-coupled channel,
//   X(r, c) = phi(r) phi(c) Z(r, c) - pm Z(s(r), s(c)),   Z = hL LCC RCC^T - hR RCC LCC^T,
// with phi(r(a,b)) = (-1)^((ja+jb)/2), s(r(a,b)) = r(b,a) and pm = hL hR.  Through the
// antisymmetry Z(x, y) = -pm Z(y, x) the reference's direct and exchange sums become
//   direct   zd(J') = X[(l,j),(i,k)]   for J' in the ranges of (i,k) and (l,j)
//   exchange ze(J') = X[(k,j),(i,l)]   for J' in the ranges of (i,l) and (k,j)
// (one read each), and for every J the pairs share
//   RES(ij, kl; J) += pre * ( sum_J' Sd(J, J') zd(J') + sum_J' Se(J, J') ze(J') )
// with Sd = -(-1)^((jl+jk+J)/2) {ji jj J; jl jk J'}, Se = {ji jj J; jk jl J'} and
// pre = 1/sqrt2 per pair of identical orbits.
//
// Organisation for GB300:
//  * a warp takes one group (i, k, l) of the orbit quadruples (i <= j, k <= l).  Everything
//    that depends on (i, k, l) alone is computed once per group: the X column of every J'
//    (lane u for the u-th J') goes to the warp's shared-memory slots;
//  * the group's quadruples are taken kRcChunk at a time.  First the warp stages, for every
//    (quadruple, J') pair of the chunk, the row index of (l, j) or (k, j) and then the X value
//    into shared memory: all those loads are independent, so many are in flight at once and
//    each X element is read once (rows of consecutive j are adjacent);
//  * then one thread per output element (ij, kl; J) contracts its 6j row with the staged X
//    values of its own J' windows, from shared memory;
//  * groups are sorted by their triple (ji, jk, jl): a CTA takes a run of groups of one
//    triple and stages, once, the 6j blocks Sd, Se of every jj of that triple into shared
//    memory (precomputed per triple on the host, in FP32 as the device 6j table holds them);
//  * RES accumulates in FP64 (one add per element); only the upper triangles of the square
//    arrays are written (a mirror pass follows).
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "dev.cuh"
#include "engine.h"
#include "kernels.h"
#include "recouple.h"

namespace imsrg {

namespace {

// FP32 6j of the device table (d_sixjf): zero outside the triangle conditions
float host_sixjf(const Layout& L, int j1, int j2, int j3, int j4, int j5, int j6) {
  auto tri = [](int a, int b, int c) { return c <= a + b && c >= std::abs(a - b); };
  if (!(tri(j1, j2, j3) && tri(j4, j5, j3) && tri(j1, j5, j6) && tri(j4, j2, j6))) return 0.0f;
  const int nh = L.sj_nh;
  const int k = (((j1 >> 1) * nh + (j2 >> 1)) * nh + (j4 >> 1)) * nh + (j5 >> 1);
  return (float)L.sj_val[L.sj_off[k] + ((j3 - L.sj_j3min[k]) >> 1) * L.sj_n6[k] + ((j6 - L.sj_j6min[k]) >> 1)];
}

constexpr int kGroupsPerTask = 96;

// rows of the staged blocks of jj = 2h+1: J in [|ji - jj|, ji + jj]
__host__ __device__ __forceinline__ int rc_rows(int ji, int h) {
  const int jj = 2 * h + 1;
  return (ji < jj ? ji : jj) + 1;
}

}  // namespace

// Groups, tasks and the per-triple 6j blocks from the quadruple list (ordered i, k, l, j).
std::string build_recouple_plan(const Layout& L, const std::vector<uint64_t>& quads, RecouplePlan& P) {
  P = RecouplePlan();
  const int nh = (L.JM + 1) / 2;
  struct G {
    int i, k, l, q0, nq;
  };
  std::vector<G> groups;
  for (size_t t = 0; t < quads.size();) {
    const uint64_t q = quads[t];
    const int i = (int)(q & 0xFFFF), k = (int)((q >> 32) & 0xFFFF), l = (int)((q >> 48) & 0xFFFF);
    size_t e = t + 1;
    while (e < quads.size() && (quads[e] & 0xFFFF) == (uint64_t)i && ((quads[e] >> 32) & 0xFFFF) == (uint64_t)k &&
           ((quads[e] >> 48) & 0xFFFF) == (uint64_t)l)
      ++e;
    if (e - t > (size_t)kRcMaxGroup) return "recoupling group larger than the kernel's per-warp slots";
    groups.push_back(G{i, k, l, (int)t, (int)(e - t)});
    t = e;
  }
  // triples in first-seen order, groups sorted by (bin, triple), stable
  std::map<int, int> tix;
  std::vector<int> tkey;
  auto key_of = [&](const G& g) { return (L.jj[g.i] << 16) | (L.jj[g.k] << 8) | L.jj[g.l]; };
  for (const G& g : groups) {
    const int key = key_of(g);
    if (!tix.count(key)) {
      tix[key] = (int)tkey.size();
      tkey.push_back(key);
    }
  }
  std::vector<int> order(groups.size());
  for (size_t g = 0; g < groups.size(); ++g) order[g] = (int)g;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return tix[key_of(groups[a])] < tix[key_of(groups[b])]; });
  // staged 6j blocks per triple: for h = 0..nh-1, the direct block (rows x nud) then the
  // exchange block (rows x nue); each triple padded to a multiple of 4 floats
  P.triples.resize(tkey.size());
  for (size_t t = 0; t < tkey.size(); ++t) {
    const int key = tkey[t];
    const int ji = key >> 16, jk = (key >> 8) & 0xFF, jl = key & 0xFF;
    const int nud = std::min(ji, jk) + 1, nue = std::min(ji, jl) + 1;
    const int dbase = std::abs(ji - jk), ebase = std::abs(ji - jl);
    RcTriple& T = P.triples[t];
    T.off = (int64_t)P.table.size();
    T.ji = (int16_t)ji; T.jk = (int16_t)jk; T.jl = (int16_t)jl;
    T.nud = (int16_t)nud; T.nue = (int16_t)nue;
    for (int h = 0; h < nh; ++h) {
      const int jj = 2 * h + 1, r0 = std::abs(ji - jj), nr = rc_rows(ji, h);
      for (int r = 0; r < nr; ++r) {
        const int J = r0 + 2 * r;
        const float sg = ((jl + jk + J) & 2) ? 1.0f : -1.0f;  // -(-1)^((jl+jk+J)/2)
        for (int u = 0; u < nud; ++u) P.table.push_back(sg * host_sixjf(L, ji, jj, J, jl, jk, dbase + 2 * u));
      }
      for (int r = 0; r < nr; ++r) {
        const int J = r0 + 2 * r;
        for (int u = 0; u < nue; ++u) P.table.push_back(host_sixjf(L, ji, jj, J, jk, jl, ebase + 2 * u));
      }
    }
    while (P.table.size() % 4) P.table.push_back(0.0f);
    T.nfl = (int)((int64_t)P.table.size() - T.off);
  }
  if (P.table.size() >= ((size_t)1 << 31)) return "recoupling 6j table too large";
  // groups in task order; tasks of up to kGroupsPerTask groups of one triple
  P.groups.resize(groups.size());
  int max_nfl = 0;
  for (size_t n = 0; n < order.size();) {
    const int key = key_of(groups[order[n]]);
    size_t e = n;
    while (e < order.size() && key_of(groups[order[e]]) == key && e - n < (size_t)kGroupsPerTask) ++e;
    P.tasks.push_back(RcTask{(int)n, (int)(e - n), tix[key], 0});
    max_nfl = std::max(max_nfl, P.triples[tix[key]].nfl);
    n = e;
  }
  for (size_t n = 0; n < order.size(); ++n) {
    const G& g = groups[order[n]];
    P.groups[n] = RcGroup{g.i | (g.k << 16), g.l | (g.nq << 16), g.q0, 0};
  }
  // shared memory: the staged 6j blocks, then per warp the group's X columns, the chunk's j
  // list and output prefix, and its staged (quadruple, J') values
  P.acc_off = max_nfl;
  P.smem_bytes = sizeof(float) * (size_t)max_nfl + (size_t)(kRcThreads / 32) * kRcWarpSlotBytes;
  int max_nu = 0;
  for (const RcTriple& T : P.triples) max_nu = std::max(max_nu, (int)T.nud + (int)T.nue);
  if (max_nu > kRcMaxU) return "recoupling: more J' values than the kernel's per-warp slots";
  return std::string();
}

// The bytes the recoupling must move, counted exactly from the plan: every distinct X element
// it reads (a quadruple with k == l reads one element in both terms), every RES element it
// reads and writes once, and its own index data (quadruples, groups, tasks, triples and the
// staged 6j table, each read once).
RecoupleTraffic recouple_traffic(const Layout& L, const std::vector<uint64_t>& quads, const RecouplePlan& P) {
  RecoupleTraffic t{};
  const int N = L.N, NJ = L.NJ, JM = L.JM;
  std::vector<uint64_t> seen((size_t)(L.wcc_size + 63) / 64, 0);
  auto col = [&](int a, int b, int h, int& qx) {
    qx = h + (std::abs(L.tz[a] - L.tz[b]) >> 1) * (JM + 1) + ((L.ll[a] + L.ll[b]) & 1) * 2 * (JM + 1);
    return L.wcc_off[qx] + (int64_t)L.ccr[((size_t)a * N + b) * NJ + h] * L.cc_rlen[qx];
  };
  for (uint64_t q : quads) {
    const int i = (int)(q & 0xFFFF), j = (int)((q >> 16) & 0xFFFF), k = (int)((q >> 32) & 0xFFFF),
              l = (int)((q >> 48) & 0xFFFF);
    const int ji = L.jj[i], jj = L.jj[j], jk = L.jj[k], jl = L.jj[l];
    for (int term = 0; term < 2; ++term) {
      const int c = term ? l : k, r = term ? k : l;  // column pair (i, c), row pair (r, j)
      const int lo = std::max(std::abs(ji - L.jj[c]), std::abs(jj - L.jj[r]));
      const int hi = std::min(ji + L.jj[c], jj + L.jj[r]);
      for (int JP = lo; JP <= hi; JP += 2) {
        int qx;
        const int64_t x = col(i, c, JP >> 1, qx) + L.ccr[((size_t)r * N + j) * NJ + (JP >> 1)];
        ++t.x_reads;
        uint64_t& w = seen[(size_t)x >> 6];
        const uint64_t bit = 1ull << (x & 63);
        if (!(w & bit)) {
          w |= bit;
          ++t.x_distinct;
        }
      }
    }
    t.res_elems += (std::min(ji + jj, jk + jl) - std::max(std::abs(ji - jj), std::abs(jk - jl))) / 2 + 1;
  }
  t.aux_bytes = (int64_t)(sizeof(uint64_t) * quads.size() + sizeof(RcGroup) * P.groups.size() +
                          sizeof(RcTask) * P.tasks.size() + sizeof(RcTriple) * P.triples.size() +
                          sizeof(float) * P.table.size());
  return t;
}

namespace {

__global__ void __launch_bounds__(kRcThreads) k_recouple_g(DevLayout D, const RcTask* __restrict__ tasks,
                                                           const RcGroup* __restrict__ groups,
                                                           const RcTriple* __restrict__ triples,
                                                           const float* __restrict__ table, int slot_off,
                                                           const uint64_t* __restrict__ quads,
                                                           const int* __restrict__ xcol, const float* __restrict__ X,
                                                           double* __restrict__ RES) {
  extern __shared__ __align__(16) float S[];
  const RcTask task = tasks[blockIdx.x];
  const RcTriple tr = triples[task.triple];
  for (int e = threadIdx.x * 4; e < tr.nfl; e += kRcThreads * 4)
    *reinterpret_cast<float4*>(S + e) = __ldg(reinterpret_cast<const float4*>(table + tr.off + e));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // this warp's slots: X columns of the direct and exchange J'; the chunk's j and output
  // prefix; its staged values xs[t * nu + u] (u < nud direct, nud + u' exchange)
  char* slot = reinterpret_cast<char*>(S + slot_off) + warp * kRcWarpSlotBytes;
  int64_t* wcd = reinterpret_cast<int64_t*>(slot);
  int64_t* wce = wcd + 32;
  int* wj = reinterpret_cast<int*>(wce + 32);
  int* wpre = wj + kRcChunk;
  float* xs = reinterpret_cast<float*>(wpre + kRcChunk);
  int* xr = reinterpret_cast<int*>(xs);  // the same slots hold the row indices first
  __syncthreads();

  const int ji = tr.ji, jk = tr.jk, jl = tr.jl, nud = tr.nud, nue = tr.nue, nu = nud + nue;
  const int dbase = abs(ji - jk), ebase = abs(ji - jl);
  const int N = D.N, NJ = D.NJ;
  const int jkl_lo = abs(jk - jl), jkl_hi = jk + jl;
  for (int gi = task.g0 + warp; gi < task.g0 + task.ng; gi += kRcThreads / 32) {
    const RcGroup G = groups[gi];
    const int i = G.x & 0xFFFF, k = G.x >> 16, l = G.y & 0xFFFF, nq = G.y >> 16, q0 = G.z;
    __syncwarp();  // the previous group's slots are read
    if (lane < nud) wcd[lane] = xcol[(i * N + k) * NJ + (dbase >> 1) + lane];
    if (lane < nue) wce[lane] = xcol[(i * N + l) * NJ + (ebase >> 1) + lane];
    const int C2 = D.con[k] + D.con[l];
    const float prek = (k == l) ? .70710678118f : 1.0f;
    for (int c0 = 0; c0 < nq; c0 += kRcChunk) {
      const int nc = min(kRcChunk, nq - c0);
      __syncwarp();  // the previous chunk's slots are read
      // j of every quadruple of the chunk and the prefix of its output count (J values)
      int j = 0, nj = 0;
      if (lane < nc) {
        j = (int)((quads[q0 + c0 + lane] >> 16) & 0xFFFF);
        const int jj = D.jj[j];
        nj = (min(ji + jj, jkl_hi) - max(abs(ji - jj), jkl_lo)) / 2 + 1;
      }
      int incl = nj;  // inclusive warp scan
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += v;
      }
      if (lane < nc) {
        wj[lane] = j;
        wpre[lane] = incl - nj;
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      __syncwarp();
      // rows of the (quadruple, J') pairs inside their windows, -1 outside
      const int npair = nc * nu;
#pragma unroll 4
      for (int p = lane; p < npair; p += 32) {
        const int t = p / nu, u = p - t * nu;
        const int jt = wj[t], jj = D.jj[jt];
        int row = -1;
        if (u < nud) {
          const int JP = dbase + 2 * u;
          if (JP >= abs(jj - jl) && JP <= jj + jl) row = __ldg(D.ccr_t + (l * NJ + (JP >> 1)) * N + jt);
        } else {
          const int JP = ebase + 2 * (u - nud);
          if (JP >= abs(jj - jk) && JP <= jj + jk) row = __ldg(D.ccr_t + (k * NJ + (JP >> 1)) * N + jt);
        }
        xr[p] = row;
      }
      __syncwarp();
      // the X values of those pairs (0 outside the windows)
#pragma unroll 4
      for (int p = lane; p < npair; p += 32) {
        const int u = p % nu;
        const int row = xr[p];
        const float x = row < 0 ? 0.0f : __ldg(X + (u < nud ? wcd[u] : wce[u - nud]) + row);
        xs[p] = x;
      }
      __syncwarp();
      for (int o0 = 0; o0 < total; o0 += 32) {
        const int o = o0 + lane;
        if (o >= total) continue;
        // the quadruple of output o: the last t with wpre[t] <= o
        int t = 0;
        for (int b = kRcChunk >> 1; b > 0; b >>= 1)
          if (t + b < nc && wpre[t + b] <= o) t += b;
        const int jt = wj[t];
        const int jj = D.jj[jt];
        const int rbase = abs(ji - jj);
        const int J = max(rbase, jkl_lo) + 2 * (o - wpre[t]);
        const int h = jj >> 1;
        int off = 0;
        for (int x = 0; x < h; ++x) off += rc_rows(ji, x);
        const int r = (J - rbase) >> 1;
        const float* Sd = S + off * nu + r * nud;
        const float* Se = S + off * nu + rc_rows(ji, h) * nud + r * nue;
        const float* xt = xs + t * nu;
        float sd = 0.0f, se = 0.0f;  // the same summation order as k_recouple_q
        {  // direct: J' in the ranges of (i,k) and (l,j)
          const int u0 = (max(abs(jj - jl), dbase) - dbase) >> 1, u1 = (min(jj + jl, ji + jk) - dbase) >> 1;
          for (int u = u0; u <= u1; ++u) sd = fmaf(Sd[u], xt[u], sd);
        }
        {  // exchange: J' in the ranges of (i,l) and (k,j)
          const int u0 = (max(abs(jj - jk), ebase) - ebase) >> 1, u1 = (min(jj + jk, ji + jl) - ebase) >> 1;
          for (int u = u0; u <= u1; ++u) se = fmaf(Se[u], xt[nud + u], se);
        }
        const float sm = sd + se;
        const int C1 = D.con[i] + D.con[jt];
        const int g = (C1 == 0) ? C2 : (C1 == 1 ? (C2 == 1 ? 3 : 5) : 4);
        const int T = D.tz[i] + D.tz[jt], P = (D.ll[i] + D.ll[jt]) & 1;
        const float pre = ((i == jt) ? .70710678118f : 1.0f) * prek;
        const int kk = (3 * J + (T + 2) + P) * 6 + g;
        const int IX = D.pairpos_t[(i * NJ + (J >> 1)) * N + jt], JX = D.pairpos[(k * N + l) * NJ + (J >> 1)];
        double* out = RES + D.goff[kk] + IX + (int64_t)JX * D.gn1[kk];
        atomicAdd(out, f32_to_f64(sm * pre));  // the only add to this element: a reduction at L2, no read here
      }
    }
  }
}

// One thread per orbit quadruple (i <= j, k <= l), quadruples in list order (i, k, l, then j):
// the thread gathers its J' inputs X[(l,j),(i,k)] and X[(k,j),(i,l)] (all loads of both terms
// independent, so they are in flight together) and then forms every output J the pairs share,
// with the 6j rows of the device table.  The same summation order as k_recouple_g.
constexpr int kRcMaxJp = 26;  // J' per term: at most 2 jmax + 1 (2j <= 25 for eMax <= 12)
template <int kMinBlocks>
__global__ void __launch_bounds__(256, kMinBlocks) k_recouple_q(DevLayout D, const uint64_t* __restrict__ quads,
                                                                int64_t nquads, const int* __restrict__ xcol,
                                                                const float* __restrict__ X,
                                                                double* __restrict__ RES) {
  const int N = D.N, NJ = D.NJ;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nquads;
       t += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t qd = quads[t];
    const int i = (int)(qd & 0xFFFF), j = (int)((qd >> 16) & 0xFFFF), k = (int)((qd >> 32) & 0xFFFF),
              l = (int)((qd >> 48) & 0xFFFF);
    const int ji = D.jj[i], jj = D.jj[j], jk = D.jj[k], jl = D.jj[l];
    const int dlo = max(abs(jj - jl), abs(ji - jk)), dhi = min(jj + jl, ji + jk);
    const int elo = max(abs(ji - jl), abs(jj - jk)), ehi = min(ji + jl, jj + jk);
    const int nd = (dhi - dlo) / 2 + 1, ne = (ehi - elo) / 2 + 1;
    float zd[kRcMaxJp], ze[kRcMaxJp];
    {
      const int* col = xcol + (i * N + k) * NJ;
      const int* rows = D.ccr_t + l * NJ * N + j;
      for (int m = 0; m < nd; ++m) {
        const int h = (dlo >> 1) + m;
        zd[m] = __ldg(X + col[h] + __ldg(rows + h * N));
      }
    }
    {
      const int* col = xcol + (i * N + l) * NJ;
      const int* rows = D.ccr_t + k * NJ * N + j;
      for (int m = 0; m < ne; ++m) {
        const int h = (elo >> 1) + m;
        ze[m] = __ldg(X + col[h] + __ldg(rows + h * N));
      }
    }
    const int nh = D.sj_nh;
    const int kd = (((ji >> 1) * nh + (jj >> 1)) * nh + (jl >> 1)) * nh + (jk >> 1);
    const int ke = (((ji >> 1) * nh + (jj >> 1)) * nh + (jk >> 1)) * nh + (jl >> 1);
    const float* sjd = D.sj_valf + D.sj_off[kd];
    const float* sje = D.sj_valf + D.sj_off[ke];
    const int d3 = D.sj_j3min[kd], d6 = D.sj_j6min[kd], dn6 = D.sj_n6[kd];
    const int e3 = D.sj_j3min[ke], e6 = D.sj_j6min[ke], en6 = D.sj_n6[ke];
    const int C1 = D.con[i] + D.con[j], C2 = D.con[k] + D.con[l];
    const int g = (C1 == 0) ? C2 : (C1 == 1 ? (C2 == 1 ? 3 : 5) : 4);
    const int T = D.tz[i] + D.tz[j], P = (D.ll[i] + D.ll[j]) & 1;
    const float pre = ((i == j) ? .70710678118f : 1.0f) * ((k == l) ? .70710678118f : 1.0f);
    const int Jlo = max(abs(ji - jj), abs(jk - jl)), Jhi = min(ji + jj, jk + jl);
    for (int J = Jlo; J <= Jhi; J += 2) {
      const float sg = ((jl + jk + J) & 2) ? 1.0f : -1.0f;  // -(-1)^((jl+jk+J)/2), folded into the direct 6j
      const float* rd = sjd + ((J - d3) >> 1) * dn6 + ((dlo - d6) >> 1);
      const float* re = sje + ((J - e3) >> 1) * en6 + ((elo - e6) >> 1);
      float sd = 0.0f, se = 0.0f;
      for (int m = 0; m < nd; ++m) sd = fmaf(sg * __ldg(rd + m), zd[m], sd);
      for (int m = 0; m < ne; ++m) se = fmaf(__ldg(re + m), ze[m], se);
      const float sm = sd + se;
      const int kk = (3 * J + (T + 2) + P) * 6 + g;
      const int IX = D.pairpos_t[(i * NJ + (J >> 1)) * N + j], JX = D.pairpos[(k * N + l) * NJ + (J >> 1)];
      double* out = RES + D.goff[kk] + IX + (int64_t)JX * D.gn1[kk];
      atomicAdd(out, f32_to_f64(sm * pre));  // the only add to this element: a reduction at L2, no read here
    }
  }
}

}  // namespace

void launch_recouple_g(const RecouplePlan& P, cudaStream_t st, const DevLayout& D, const RcTask* tasks,
                       const RcGroup* groups, const RcTriple* triples, const float* table, const uint64_t* quads,
                       const int* xcol, const float* X, double* RES) {
  if (P.tasks.empty()) return;
  k_recouple_g<<<(int)P.tasks.size(), kRcThreads, P.smem_bytes, st>>>(D, tasks, groups, triples, table, P.acc_off,
                                                                       quads, xcol, X, RES);
}

void launch_recouple_q(int min_blocks, int grid, cudaStream_t st, const DevLayout& D, const uint64_t* quads,
                       int64_t nquads, const int* xcol, const float* X, double* RES) {
  if (nquads <= 0) return;
  switch (min_blocks) {
    case 6: k_recouple_q<6><<<grid, 256, 0, st>>>(D, quads, nquads, xcol, X, RES); break;
    case 8: k_recouple_q<8><<<grid, 256, 0, st>>>(D, quads, nquads, xcol, X, RES); break;
    default: k_recouple_q<4><<<grid, 256, 0, st>>>(D, quads, nquads, xcol, X, RES); break;
  }
}

// The X column offset of every pair (a, b) at every J' (-1 where (a, b) is not a row of the
// cross-coupled channel of J'): wcc_off[q] + r(a, b) * rlen[q], [(a * N + b) * NJ + J'/2]
std::vector<int> build_xcol(const Layout& L) {
  std::vector<int> x((size_t)L.N * L.N * L.NJ, -1);
  for (int a = 0; a < L.N; ++a)
    for (int b = 0; b < L.N; ++b)
      for (int h = 0; h < L.NJ; ++h) {
        const int r = L.ccr[((size_t)a * L.N + b) * L.NJ + h];
        if (r < 0) continue;
        const int q = L.ccq(2 * h, std::abs(L.tz[a] - L.tz[b]) / 2, (L.ll[a] + L.ll[b]) % 2);
        x[((size_t)a * L.N + b) * L.NJ + h] = (int)(L.wcc_off[q] + (int64_t)r * L.cc_rlen[q]);
      }
  return x;
}

cudaError_t recouple_g_smem_attr(size_t smem) {
  return cudaFuncSetAttribute(k_recouple_g, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

}  // namespace imsrg
