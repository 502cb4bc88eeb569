// Input preparation on the host (FP64): a seeded synthetic Hamiltonian with the
// structure of the reference's inputs.
//
//  * two-body part: isospin-coupled records in the me2j loop order and converted to the
//    proton-neutron J-scheme exactly as read_me2j_interaction does
//    (src/interaction_IO.f90:320-352, 398-555); each (T=0, T=1) record value is
//    v_scale * N(0,1) * exp(-(e1+e2+e3+e4)/eMax), the T=1 value shared by Mt=-1,0,+1
//    (isospin symmetric), Pauli-forbidden records (identical orbits, J+T even) zero;
//  * one-body part: the harmonic-oscillator kinetic energy with the intrinsic (1-1/A)
//    factor (calculate_h0_harm_osc with Htype 1, src/basic_IMSRG.f90:2093-2191);
//  * normal ordering with respect to the reference state (normal_order,
//    src/basic_IMSRG.f90:2419-2550), i.e. the HO-basis reference of calc_HO.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "engine.h"
#include "layout.h"

namespace {

struct Normal {
  uint64_t s;
  bool have = false;
  double spare = 0.0;
  explicit Normal(uint64_t seed) : s(seed * 0xD1B54A32D192ED03ULL + 0x8CB92BA72F3D8DD7ULL) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  double uni() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
  double gauss() {  // Box-Muller
    if (have) { have = false; return spare; }
    const double u = uni(), v = uni();
    const double r = std::sqrt(-2.0 * std::log(u)), t = 6.283185307179586 * v;
    spare = r * std::sin(t);
    have = true;
    return r * std::cos(t);
  }
};

inline double sgn(int n) { return (n & 1) ? -1.0 : 1.0; }

}  // namespace

namespace {

imsrg_status synthetic(imsrg_ctx* ctx, uint64_t seed, double v_scale, bool bare, double* out) {
  if (!ctx || !out) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  const imsrg::Layout& L = c->L;
  const int N = L.N, NJ = L.NJ;
  // the me2j loop runs over isospin orbits: hk order lists each (n,l,j) as a proton
  // (2tz=-1) followed by its neutron partner
  if (N % 2) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "synthetic Hamiltonian needs proton/neutron orbit pairs");
  for (int k = 0; k < N; k += 2)
    if (L.tz[k] != -1 || L.tz[k + 1] != 1 || L.nn[k] != L.nn[k + 1] || L.ll[k] != L.ll[k + 1] || L.jj[k] != L.jj[k + 1])
      return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "orbits are not in proton/neutron pairs (hk order)");
  std::vector<double> H((size_t)L.slab, 0.0);
  const int M = N / 2;
  const double emax = L.eMax > 0 ? (double)L.eMax : 1.0;
  Normal rng(seed);
  auto e_of = [&](int I) { return 2 * L.nn[2 * I] + L.ll[2 * I]; };
  for (int I1 = 0; I1 < M; ++I1)
    for (int I2 = 0; I2 <= I1; ++I2)
      for (int I3 = 0; I3 <= I1; ++I3) {
        const int end = (I1 == I3) ? I2 : I3;
        for (int I4 = 0; I4 <= end; ++I4) {
          const int l1 = L.ll[2 * I1], l2 = L.ll[2 * I2], l3 = L.ll[2 * I3], l4 = L.ll[2 * I4];
          if ((l1 + l2) % 2 != (l3 + l4) % 2) continue;
          const int j1 = L.jj[2 * I1], j2 = L.jj[2 * I2], j3 = L.jj[2 * I3], j4 = L.jj[2 * I4];
          const int jmin = std::max(std::abs(j1 - j2), std::abs(j3 - j4));
          const int jmax = std::min(j1 + j2, j3 + j4);
          if (jmin > jmax) continue;
          const int Par = (l1 + l2) % 2;
          const double scale = v_scale * std::exp(-(e_of(I1) + e_of(I2) + e_of(I3) + e_of(I4)) / emax);
          for (int JT = jmin; JT <= jmax; JT += 2) {
            const int J = JT / 2;
            double me[4];
            double g0 = rng.gauss() * scale, g1 = rng.gauss() * scale;
            // Pauli: an antisymmetric state of two identical orbits needs J + T odd
            if ((I1 == I2 || I3 == I4) && ((J + 0) % 2 == 0)) g0 = 0.0;
            if ((I1 == I2 || I3 == I4) && ((J + 1) % 2 == 0)) g1 = 0.0;
            me[0] = g0; me[1] = g1; me[2] = g1; me[3] = g1;
            for (int ax = 2 * I1; ax <= 2 * I1 + 1; ++ax)
              for (int bx = 2 * I2; bx <= 2 * I2 + 1; ++bx)
                for (int cx = 2 * I3; cx <= 2 * I3 + 1; ++cx)
                  for (int dx = 2 * I4; dx <= 2 * I4 + 1; ++dx) {
                    const int a = ax, b = bx, cc = cx, d = dx;
                    double pre2 = 1.0;
                    if (a == b) pre2 *= std::sqrt(0.5);
                    if (cc == d) pre2 *= std::sqrt(0.5);
                    // me2j files label isospin with the opposite sign
                    const int ta = -L.tz[a], tb = -L.tz[b], tc = -L.tz[cc], td = -L.tz[d];
                    if (tc + td != ta + tb) continue;
                    const int T = -(ta + tb) / 2;
                    const int q = L.block(JT, T, Par);
                    double V = 0.125 * (ta - tb) * (tc - td) * me[0] +
                               ((ta + tb == -2) && (tc + td == -2) ? me[1] : 0.0) +
                               ((ta + tb == 2) && (tc + td == 2) ? me[3] : 0.0) +
                               0.125 * std::abs((ta - tb) * (tc - td)) * me[2];
                    V *= pre2;
                    const int C1 = L.con[a] + L.con[b], C2 = L.con[cc] + L.con[d];
                    static const int tab[3][3] = {{0, 1, 2}, {1, 3, 5}, {2, 5, 4}};
                    const int g = tab[C1][C2];
                    double pre = 1.0;
                    int i1, i2;
                    if (a > b) { i1 = L.pairpos[((size_t)b * N + a) * NJ + J]; pre = sgn(1 + (L.jj[a] + L.jj[b] - JT) / 2); }
                    else i1 = L.pairpos[((size_t)a * N + b) * NJ + J];
                    if (cc > d) { i2 = L.pairpos[((size_t)d * N + cc) * NJ + J]; pre *= sgn(1 + (L.jj[cc] + L.jj[d] - JT) / 2); }
                    else i2 = L.pairpos[((size_t)cc * N + d) * NJ + J];
                    if (i1 < 0 || i2 < 0) continue;
                    double* X = H.data() + L.goff[q * 6 + g];
                    const int n1 = L.gn1[q * 6 + g];
                    if (g == 0 || g == 4 || g == 3) {
                      X[i2 + (int64_t)i1 * n1] = V * pre;
                      X[i1 + (int64_t)i2 * n1] = V * pre;
                    } else if (C1 > C2) {
                      X[i2 + (int64_t)i1 * n1] = V * pre;
                    } else {
                      X[i1 + (int64_t)i2 * n1] = V * pre;
                    }
                  }
          }
        }
      }

  // one-body kinetic energy (Htype 1), with the reference's FP32 intermediate literals
  const double hw = L.hw;
  const int mass = L.Aprot + L.Aneut;
  std::vector<double> t1((size_t)N * N, 0.0);
  for (int i = 0; i < N; ++i)
    for (int j = i; j < N; ++j) {
      if (L.ll[i] != L.ll[j] || L.jj[i] != L.jj[j] || L.tz[i] != L.tz[j]) continue;
      const int ni = L.nn[i], nj = L.nn[j], lj = L.ll[j];
      if (std::abs(ni - nj) > 1) continue;
      double kij = 0.0;
      if (ni == nj) kij = 0.5 * hw * (double)(float)(2 * nj + lj + 1.5f);
      else if (ni == nj - 1) kij = 0.5 * hw * (double)std::sqrt((float)nj * ((float)(nj + lj) + 0.5f));
      else kij = 0.5 * hw * (double)std::sqrt((float)(nj + 1) * ((float)(nj + lj) + 1.5f));
      const double T = kij * (1.0 - 1.0 / mass);
      t1[(size_t)i * N + j] = T;
      t1[(size_t)j * N + i] = T;
    }
  if (bare) {  // the Hamiltonian as calc_HF receives it: T in the one-body arrays, E0 = 0
    for (int a = 0; a < L.A; ++a)
      for (int b = 0; b < L.A; ++b) H[L.off_fhh + a + (int64_t)b * L.A] = t1[(size_t)L.holes[a] * N + L.holes[b]];
    for (int a = 0; a < L.P; ++a)
      for (int b = 0; b < L.P; ++b) H[L.off_fpp + a + (int64_t)b * L.P] = t1[(size_t)L.parts[a] * N + L.parts[b]];
    for (int a = 0; a < L.P; ++a)
      for (int b = 0; b < L.A; ++b) H[L.off_fph + a + (int64_t)b * L.P] = t1[(size_t)L.parts[a] * N + L.holes[b]];
    std::memcpy(out, H.data(), sizeof(double) * H.size());
    return IMSRG_OK;
  }
  // normal ordering (src/basic_IMSRG.f90:2419-2550)
  double sm = 0.0;
  for (int i = 0; i < N; ++i) sm += t1[(size_t)i * N + i] * L.con[i] * (L.jj[i] + 1);
  sm *= 2.0;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      if (L.con[i] * L.con[j] == 0) continue;
      for (int JT = std::abs(L.jj[i] - L.jj[j]); JT <= L.jj[i] + L.jj[j]; JT += 2)
        sm += imsrg::host_v_elem(L, H.data(), 1, i, j, i, j, JT) * (JT + 1);
    }
  H[0] = sm * 0.5;
  auto fock = [&](int ax, int bx) {
    double s = 0.0;
    for (int ix : L.holes)
      for (int JT = std::abs(L.jj[ix] - L.jj[ax]); JT <= L.jj[ix] + L.jj[ax]; JT += 2)
        s += (JT + 1.0) / (L.jj[ax] + 1) * imsrg::host_v_elem(L, H.data(), 1, ax, ix, bx, ix, JT);
    return t1[(size_t)ax * N + bx] + s;
  };
  auto same = [&](int x, int y) { return L.jj[x] == L.jj[y] && L.ll[x] == L.ll[y] && L.tz[x] == L.tz[y]; };
  for (int a = 0; a < L.A; ++a)
    for (int b = a; b < L.A; ++b) {
      const int ax = L.holes[a], bx = L.holes[b];
      if (!same(ax, bx)) continue;
      const double v = fock(ax, bx);
      H[L.off_fhh + a + (int64_t)b * L.A] = v;
      H[L.off_fhh + b + (int64_t)a * L.A] = v;
    }
  for (int a = 0; a < L.P; ++a)
    for (int b = 0; b < L.A; ++b) {
      const int ax = L.parts[a], bx = L.holes[b];
      if (!same(ax, bx)) continue;
      H[L.off_fph + a + (int64_t)b * L.P] = fock(ax, bx);
    }
  for (int a = 0; a < L.P; ++a)
    for (int b = a; b < L.P; ++b) {
      const int ax = L.parts[a], bx = L.parts[b];
      if (!same(ax, bx)) continue;
      const double v = fock(ax, bx);
      H[L.off_fpp + a + (int64_t)b * L.P] = v;
      H[L.off_fpp + b + (int64_t)a * L.P] = v;
    }
  std::memcpy(out, H.data(), sizeof(double) * H.size());
  return IMSRG_OK;
}

}  // namespace

extern "C" imsrg_status imsrg_synthetic_hamiltonian(imsrg_ctx* ctx, uint64_t seed, double v_scale, double* out) {
  return synthetic(ctx, seed, v_scale, false, out);
}

extern "C" imsrg_status imsrg_synthetic_bare_hamiltonian(imsrg_ctx* ctx, uint64_t seed, double v_scale,
                                                          double* out) {
  return synthetic(ctx, seed, v_scale, true, out);
}
