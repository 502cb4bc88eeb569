// Input preparation on the host (FP64): a seeded synthetic Hamiltonian with the
// structure of the reference's inputs.
//
//  * two-body part: isospin-coupled records in the me2j loop order and converted to the
//    proton-neutron J-scheme exactly as read_me2j_interaction does
//    (src/interaction_IO.f90:320-352, 398-555); each (T=0, T=1) record value is
//    v_scale * N(0,1) * exp(-(e1+e2+e3+e4)/eMax), the T=1 value shared by Mt=-1,0,+1
//    (isospin symmetric), Pauli-forbidden records (identical orbits, J+T even) zero;
//  * one-body part: the harmonic-oscillator kinetic energy with the intrinsic (1-1/A)
//    factor (calculate_h0_harm_osc with Htype 1, src/basic_IMSRG.f90:2093-2191); the records
//    are converted without the two-body centre-of-mass term -p1.p2 hw/A: with a random
//    interaction that term closes the particle-hole gap of the eMax 4-8 HF references and the
//    White-generator flow diverges (E0 -> NaN by s=50 at eMax 4, in FP64 and in the oracle);
//    me2j_convert applies it to interaction files read with htype 1;
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

// one (n, l, j) of an me2j file: a proton / neutron pair of the pn basis
struct IsoOrbit {
  int n, l, j;
};

// the isospin orbits of an me2j file for eMax, in hk order
std::vector<IsoOrbit> file_orbits(int emax) {
  std::vector<IsoOrbit> v;
  for (int e = 0; e <= emax; ++e)
    for (int l = e % 2; l <= e; l += 2)
      for (int j2 : {2 * l - 1, 2 * l + 1})
        if (j2 >= 1) v.push_back(IsoOrbit{(e - l) / 2, l, j2});
  return v;
}

// Visits every record of the me2j loop (src/interaction_IO.f90:320-352): isospin orbits
// I1 >= I2, I3 <= I1 (I4 <= I2 when I3 == I1), equal parity, each J in the overlap of the
// two couplings.  Each record holds four values: T=0, then T=1 with Mt = -1, 0, +1.
template <class F>
void for_each_record(const std::vector<IsoOrbit>& iso, F&& f) {
  const int M = (int)iso.size();
  for (int I1 = 0; I1 < M; ++I1)
    for (int I2 = 0; I2 <= I1; ++I2)
      for (int I3 = 0; I3 <= I1; ++I3) {
        const int end = (I1 == I3) ? I2 : I3;
        for (int I4 = 0; I4 <= end; ++I4) {
          if ((iso[I1].l + iso[I2].l) % 2 != (iso[I3].l + iso[I4].l) % 2) continue;
          const int jmin = std::max(std::abs(iso[I1].j - iso[I2].j), std::abs(iso[I3].j - iso[I4].j));
          const int jmax = std::min(iso[I1].j + iso[I2].j, iso[I3].j + iso[I4].j);
          for (int JT = jmin; JT <= jmax; JT += 2) f(I1, I2, I3, I4, JT);
        }
      }
}

int64_t record_values(const std::vector<IsoOrbit>& iso) {
  int64_t n = 0;
  for_each_record(iso, [&](int, int, int, int, int) { n += 4; });
  return n;
}

// Seeded synthetic record values: T=0 and T=1 drawn from N(0, v_scale) times
// exp(-(e1+e2+e3+e4)/eMax), T=1 shared by Mt = -1, 0, +1, zero where two identical orbits
// would need J + T even.
std::vector<double> synthetic_values(const imsrg::Layout& L, const std::vector<IsoOrbit>& iso, uint64_t seed,
                                     double v_scale) {
  const double emax = L.eMax > 0 ? (double)L.eMax : 1.0;
  Normal rng(seed);
  std::vector<double> v;
  v.reserve((size_t)record_values(iso));
  auto e_of = [&](int I) { return 2 * iso[I].n + iso[I].l; };
  for_each_record(iso, [&](int I1, int I2, int I3, int I4, int JT) {
    const double scale = v_scale * std::exp(-(e_of(I1) + e_of(I2) + e_of(I3) + e_of(I4)) / emax);
    const int J = JT / 2;
    double g0 = rng.gauss() * scale, g1 = rng.gauss() * scale;
    if ((I1 == I2 || I3 == I4) && ((J + 0) % 2 == 0)) g0 = 0.0;
    if ((I1 == I2 || I3 == I4) && ((J + 1) % 2 == 0)) g1 = 0.0;
    v.push_back(g0); v.push_back(g1); v.push_back(g1); v.push_back(g1);
  });
  return v;
}

// reduced_p / reduced_r (src/basic_IMSRG.f90:4567-4656): <a||p||b>, <a||r||b> of the HO
// orbits in oscillator units
double reduced_pr(const imsrg::Layout& L, int a, int b, bool momentum) {
  const int la = L.ll[a], lb = L.ll[b], na = L.nn[a], nb = L.nn[b];
  double c1 = 0.0, p1 = 0.0;
  if (la == lb + 1) {
    c1 = std::sqrt(lb + 1.0);
    if (na == nb) p1 = (momentum ? -1.0 : 1.0) * std::sqrt(nb + lb + 1.5);
    else if (na == nb - 1) p1 = -std::sqrt(nb * 1.0);
  } else if (la == lb - 1) {
    c1 = -std::sqrt(1.0 * lb);
    if (na == nb) p1 = std::sqrt(nb + lb + 0.5);
    else if (na == nb + 1) p1 = (momentum ? 1.0 : -1.0) * std::sqrt(nb + 1.0);
  }
  return p1 * c1;
}

// p1_p2 / r1_r2 (src/basic_IMSRG.f90:4445-4565): the normalised antisymmetrised J-coupled
// matrix element of p1.p2 (or r1.r2) in oscillator units
double two_body_dot(const imsrg::Layout& L, int a, int b, int c, int d, int J, bool momentum) {
  const int ja = L.jj[a], jb = L.jj[b], jc = L.jj[c], jd = L.jj[d];
  auto one = [&](int x, int y) {  // sqrt((jx+1)(jy+1)) (-1)^((3+2lx+jy)/2) {jx 1 jy; ly 1/2 lx} <x||.||y>
    if (L.tz[x] != L.tz[y]) return 0.0;
    return std::sqrt((L.jj[x] + 1.0) * (L.jj[y] + 1.0)) * sgn((3 + 2 * L.ll[x] + L.jj[y]) / 2) *
           imsrg::sixj_racah(L.jj[x], 2, L.jj[y], 2 * L.ll[y], 1, 2 * L.ll[x]) * reduced_pr(L, x, y, momentum);
  };
  const double j_ac = one(a, c), j_bd = one(b, d), j_ad = one(a, d), j_bc = one(b, c);
  const int s1 = momentum ? (jb - jc - J) / 2 : (jb + jc - J) / 2;
  const int s2 = momentum ? (jb - jd - J) / 2 : (jb + jd - J) / 2;
  const double v = sgn(s1) * imsrg::sixj_racah(ja, jb, J, jd, jc, 2) * j_ac * j_bd -
                   sgn((jc + jd - J) / 2) * sgn(s2) * imsrg::sixj_racah(ja, jb, J, jc, jd, 2) * j_ad * j_bc;
  return v / std::sqrt((1.0 + (a == b)) * (1.0 + (c == d)));
}

// The proton-neutron J-scheme two-body arrays from me2j record values
// (src/interaction_IO.f90:398-555): records whose orbits are not all in the basis are skipped.
// With htype 1 (the intrinsic Hamiltonian, Lawson beta 0) each element also receives the
// two-body part of the centre-of-mass kinetic energy, -p1.p2 hw / A.
void me2j_convert(const imsrg::Layout& L, const std::vector<IsoOrbit>& iso, const double* values, int htype,
                  double* H) {
  const double com = (htype == 1) ? L.hw / (L.Aprot + L.Aneut) : 0.0;
  const int N = L.N, NJ = L.NJ;
  std::vector<int> proton((size_t)iso.size(), -1);  // the basis index of the proton orbit of I
  for (size_t I = 0; I < iso.size(); ++I)
    for (int k = 0; k + 1 < N; ++k)
      if (L.tz[k] == -1 && L.nn[k] == iso[I].n && L.ll[k] == iso[I].l && L.jj[k] == iso[I].j &&
          L.tz[k + 1] == 1 && L.nn[k + 1] == iso[I].n && L.ll[k + 1] == iso[I].l && L.jj[k + 1] == iso[I].j) {
        proton[I] = k;
        break;
      }
  int64_t pos = 0;
  for_each_record(iso, [&](int I1, int I2, int I3, int I4, int JT) {
    const double* me = values + pos;
    pos += 4;
    if (proton[I1] < 0 || proton[I2] < 0 || proton[I3] < 0 || proton[I4] < 0) return;
    const int J = JT / 2;
    const int Par = (iso[I1].l + iso[I2].l) % 2;
    for (int ax = proton[I1]; ax <= proton[I1] + 1; ++ax)
      for (int bx = proton[I2]; bx <= proton[I2] + 1; ++bx)
        for (int cx = proton[I3]; cx <= proton[I3] + 1; ++cx)
          for (int dx = proton[I4]; dx <= proton[I4] + 1; ++dx) {
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
            if (com != 0.0) V -= two_body_dot(L, a, b, cc, d, JT, true) * com;
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
            double* X = H + L.goff[q * 6 + g];
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
  });
}

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
  std::vector<IsoOrbit> iso;
  for (int k = 0; k < N; k += 2) iso.push_back(IsoOrbit{L.nn[k], L.ll[k], L.jj[k]});
  const std::vector<double> values = synthetic_values(L, iso, seed, v_scale);
  me2j_convert(L, iso, values.data(), 0, H.data());

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

namespace {
imsrg_status check_pairs(Ctx* c, std::vector<IsoOrbit>& iso) {
  const imsrg::Layout& L = c->L;
  if (L.N % 2) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "me2j records need proton/neutron orbit pairs");
  for (int k = 0; k < L.N; k += 2) {
    if (L.tz[k] != -1 || L.tz[k + 1] != 1 || L.nn[k] != L.nn[k + 1] || L.ll[k] != L.ll[k + 1] ||
        L.jj[k] != L.jj[k + 1])
      return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "orbits are not in proton/neutron pairs (hk order)");
    iso.push_back(IsoOrbit{L.nn[k], L.ll[k], L.jj[k]});
  }
  return IMSRG_OK;
}
}  // namespace

extern "C" imsrg_status imsrg_synthetic_me2j_values(imsrg_ctx* ctx, uint64_t seed, double v_scale, double* values,
                                                    int64_t* n) {
  if (!ctx || !n) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  std::vector<IsoOrbit> iso;
  const imsrg_status st = check_pairs(c, iso);
  if (st != IMSRG_OK) return st;
  const int64_t count = record_values(iso);
  if (!values) {
    *n = count;
    return IMSRG_OK;
  }
  if (*n < count) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "values buffer too small");
  const std::vector<double> v = synthetic_values(c->L, iso, seed, v_scale);
  std::memcpy(values, v.data(), sizeof(double) * v.size());
  *n = count;
  return IMSRG_OK;
}

extern "C" imsrg_status imsrg_me2j_to_slab(imsrg_ctx* ctx, const double* values, int64_t n, int32_t emax_file,
                                           int32_t htype, double* host_slab) {
  if (!ctx || !values || !host_slab || emax_file < 0 || htype < 0 || htype > 1) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  std::vector<IsoOrbit> mine;
  const imsrg_status st = check_pairs(c, mine);
  if (st != IMSRG_OK) return st;
  const std::vector<IsoOrbit> iso = file_orbits(emax_file);
  if (record_values(iso) != n)
    return c->fail(IMSRG_ERR_MISMATCH, "value count does not match the me2j records of emax_file");
  me2j_convert(c->L, iso, values, htype, host_slab);
  return IMSRG_OK;
}
