// commutator_222_ph recoupling (src/commutators.f90:804-921) of the mixed-precision path.
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
// One thread per orbit quadruple (i <= j, k <= l).  The quadruples of one orbit i are ordered by
// (jj, jk, jl), so the threads of a warp mostly share their J and J' ranges and 6j rows.  A thread
// first issues the X loads of both terms (all independent, so they are in flight together),
// then forms every output J the pairs share with the 6j rows of the device table.  Each
// output is the only add the recoupling makes to its element, so it goes out as an FP64
// reduction at L2 (the thread does not wait for a read of RES; the sum is the same IEEE add).
// Only the upper triangles of the square arrays are written (a mirror pass follows).
#include <algorithm>
#include <vector>

#include "dev.cuh"
#include "recouple.h"

namespace imsrg {

namespace {

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
    {  // direct: row pair (l, j), column pair (i, k)
      const int* col = xcol + (i * N + k) * NJ;
      const int* rows = D.ccr_t + l * NJ * N + j;
      for (int m = 0; m < nd; ++m) {
        const int h = (dlo >> 1) + m;
        zd[m] = __ldg(X + col[h] + __ldg(rows + h * N));
      }
    }
    {  // exchange: row pair (k, j), column pair (i, l)
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

void launch_recouple_q(int min_blocks, int grid, cudaStream_t st, const DevLayout& D, const uint64_t* quads,
                       int64_t nquads, const int* xcol, const float* X, double* RES) {
  if (nquads <= 0) return;
  switch (min_blocks) {
    case 6: k_recouple_q<6><<<grid, 256, 0, st>>>(D, quads, nquads, xcol, X, RES); break;
    case 8: k_recouple_q<8><<<grid, 256, 0, st>>>(D, quads, nquads, xcol, X, RES); break;
    default: k_recouple_q<4><<<grid, 256, 0, st>>>(D, quads, nquads, xcol, X, RES); break;
  }
}

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

std::vector<unsigned> build_x_read_mask(const Layout& L, const std::vector<uint64_t>& quads, std::vector<int>& mask_off) {
  const int N = L.N, NJ = L.NJ, JM = L.JM;
  mask_off.assign(L.ncc, -1);
  size_t words = 0;
  for (int q = 0; q < L.ncc; ++q) {
    const int r = L.cc_rlen[q];
    if (r == 0) continue;
    mask_off[q] = (int)words;
    words += (size_t)((r + 31) / 32) * ((r + 31) / 32);
  }
  std::vector<unsigned> m(std::max<size_t>(words, 1), 0u);
  auto mark = [&](int a, int b, int r0, int r1, int h) {  // column pair (a, b), row pair (r0, r1) at J' = 2h
    const int q = h + (std::abs(L.tz[a] - L.tz[b]) >> 1) * (JM + 1) + ((L.ll[a] + L.ll[b]) & 1) * 2 * (JM + 1);
    const int col = L.ccr[((size_t)a * N + b) * NJ + h], row = L.ccr[((size_t)r0 * N + r1) * NJ + h];
    const int nwc = (L.cc_rlen[q] + 31) / 32;
    m[(size_t)mask_off[q] + (size_t)(row >> 5) * nwc + (col >> 5)] |= 1u << (col & 31);
  };
  for (uint64_t qd : quads) {
    const int i = (int)(qd & 0xFFFF), j = (int)((qd >> 16) & 0xFFFF), k = (int)((qd >> 32) & 0xFFFF),
              l = (int)((qd >> 48) & 0xFFFF);
    const int ji = L.jj[i], jj = L.jj[j], jk = L.jj[k], jl = L.jj[l];
    const int dlo = std::max(std::abs(jj - jl), std::abs(ji - jk)), dhi = std::min(jj + jl, ji + jk);
    for (int JP = dlo; JP <= dhi; JP += 2) mark(i, k, l, j, JP >> 1);  // direct: X[(l,j),(i,k)]
    const int elo = std::max(std::abs(ji - jl), std::abs(jj - jk)), ehi = std::min(ji + jl, jj + jk);
    for (int JP = elo; JP <= ehi; JP += 2) mark(i, l, k, j, JP >> 1);  // exchange: X[(k,j),(i,l)]
  }
  return m;
}

RecoupleTraffic recouple_traffic(const Layout& L, const std::vector<uint64_t>& quads) {
  RecoupleTraffic t{};
  const int N = L.N, NJ = L.NJ, JM = L.JM;
  std::vector<uint64_t> seen((size_t)(L.wcc_size + 63) / 64, 0);
  auto col = [&](int a, int b, int h) {
    const int qx = h + (std::abs(L.tz[a] - L.tz[b]) >> 1) * (JM + 1) + ((L.ll[a] + L.ll[b]) & 1) * 2 * (JM + 1);
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
        const int64_t x = col(i, c, JP >> 1) + L.ccr[((size_t)r * N + j) * NJ + (JP >> 1)];
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
  t.aux_bytes = (int64_t)(sizeof(uint64_t) * quads.size() + 2 * sizeof(int) * (size_t)N * N * NJ);
  return t;
}

}  // namespace imsrg
