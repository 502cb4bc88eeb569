// EOM-IMSRG on the device: excitation ("ladder") operators, the EOM matrix-vector product and
// the Lanczos eigensolver of calculate_excited_states / LANCZOS_DIAGONALIZE /
// matvec_nonzeroX_prod (src/EOM_IMSRG.f90:13-334, 518-556).
//
// A ladder operator of rank lambda and parity change dpar is a tensor slab whose only amplitudes
// are fph and the pp-hh arrays tgam(3) / tgam(7); its blocks carry lam(1) = 1, so the amplitude
// <pp J1|X|hh J2> with J1 > J2 sits in tgam(7) of block (J2, J1) with phase 1.  The amplitude
// vector is ordered as unwrap_tensor orders it (src/EOM_IMSRG.f90:1039-1132).
//
// The product rewrap([H, X]) of the reference's EOM_TS_commutator_* routines is [H, X] with X an
// excitation operator, read on its particle-hole and pp-hh elements.  It is computed from two
// general scalar-tensor commutators: S(h) is the tensor of herm h whose stored excitation
// elements are X's and whose stored de-excitation elements are h times their images, so that
// X = (S(+1) + S(-1)) / 2 as operators and [H, X] = ([H, S(+1)] + [H, S(-1)]) / 2.  Both
// S(h) are written by one gather kernel from the amplitude vector and both results are read
// back by one kernel.  The commutators run in the tensor engine's excitation mode: only the
// terms with a nonzero (fph, pp-hh) operand of S(h) and only the fph and pp-hh outputs are
// computed (their GEMMs in FP64, or FP32 in the mixed modes, with the 122 / 212 sums), and every
// particle-hole product is recoupled
// (EOM_TS_commutator_222_ph has no 1e-6 cut, and a cut would make the product depend on the
// scale of v).
//
// The eigensolver is a thick-restart Lanczos with full reorthogonalisation on the host
// (ncv = 5 nev basis vectors, the nev Ritz values of smallest magnitude kept, convergence
// |beta s_m| <= tol |theta|), the method ARPACK's dsaupd implements by implicit restarts,
// with the reference's parameters (which = 'SM', tol 1e-10, at most 500 restarts).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "engine.h"
#include "linalg.h"
#include "tensor_state.h"

using namespace imsrg;

struct imsrg_eom {
  Ctx* owner = nullptr;
  TensorState* ts = nullptr;
  int rank = 0, dpar = 0;
  int64_t n = 0, n1b = 0;
  std::vector<int64_t> pos, mirror;  // slab position of each amplitude; J1 == J2 transposed copy or -1
  std::vector<int8_t> kind, phase;   // 0 fph, 1 tgam(3), 2 tgam(7); (-1)^((J1-J2)/2) for kind 2
  int64_t* d_pos = nullptr;
  int64_t* d_mirror = nullptr;
  int8_t* d_kind = nullptr;
  int8_t* d_phase = nullptr;
  double* d_v = nullptr;
  double* d_w = nullptr;
  double* d_S[2] = {nullptr, nullptr};
  double* d_Y[2] = {nullptr, nullptr};
  // the product on d_v -> d_w as one CUDA graph (several hundred launches), for the H it was
  // captured with
  cudaGraphExec_t gexec = nullptr;
  const double* g_H = nullptr;
  int g_prec = -1;  // the context's precision at capture (the kernels differ between modes)
};

namespace {

#define CKE(expr)                  \
  do {                             \
    imsrg_status _s = (expr);      \
    if (_s != IMSRG_OK) return _s; \
  } while (0)

int grid_of(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8)); }

// S(+1) and S(-1) from the amplitudes (only these positions are ever written, so the slabs stay
// zero elsewhere from their allocation on)
__global__ void k_eom_pack(int64_t n, const int64_t* __restrict__ pos, const int8_t* __restrict__ kind,
                           const int8_t* __restrict__ phase, const int64_t* __restrict__ mirror,
                           const double* __restrict__ v, double* __restrict__ Sp, double* __restrict__ Sm) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const double x = v[k];
    const int64_t p = pos[k];
    if (kind[k] == 2) {
      const double y = phase[k] * x;
      Sp[p] = y;
      Sm[p] = -y;
    } else {
      Sp[p] = x;
      Sm[p] = x;
      const int64_t q = mirror[k];
      if (q >= 0) {
        Sp[q] = x;
        Sm[q] = -x;
      }
    }
  }
}

// w = the excitation amplitudes of ([H, S(+1)] + [H, S(-1)]) / 2; Yp has herm -1, Ym herm +1, and
// the excitation element behind a tgam(7) entry is herm (-1)^((J1-J2)/2) times it
__global__ void k_eom_unpack(int64_t n, const int64_t* __restrict__ pos, const int8_t* __restrict__ kind,
                             const int8_t* __restrict__ phase, const double* __restrict__ Yp,
                             const double* __restrict__ Ym, double* __restrict__ w) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = pos[k];
    w[k] = (kind[k] == 2) ? 0.5 * phase[k] * (Ym[p] - Yp[p]) : 0.5 * (Yp[p] + Ym[p]);
  }
}

// unwrap_tensor into a zeroed ladder slab
__global__ void k_eom_unwrap(int64_t n, const int64_t* __restrict__ pos, const int64_t* __restrict__ mirror,
                             const double* __restrict__ v, double* __restrict__ X) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    X[pos[k]] = v[k];
    if (mirror[k] >= 0) X[mirror[k]] = v[k];
  }
}

// rewrap_tensor
__global__ void k_eom_rewrap(int64_t n, const int64_t* __restrict__ pos, const double* __restrict__ X,
                             double* __restrict__ v) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    v[k] = X[pos[k]];
}

// the amplitude order of unwrap_tensor: fph (particles outer, holes inner), then per block the
// tgam(3) elements row by row and, for J1 < J2, the tgam(7) elements row by row; pairs of
// identical orbits are skipped at odd J
void build_map(const Layout& L, const TLayout& T, imsrg_eom& E) {
  auto push = [&](int64_t p, int k, int ph, int64_t mi) {
    E.pos.push_back(p);
    E.kind.push_back((int8_t)k);
    E.phase.push_back((int8_t)ph);
    E.mirror.push_back(mi);
  };
  for (int ix = 0; ix < L.P; ++ix)
    for (int jx = 0; jx < L.A; ++jx) {
      const int p = L.parts[ix], h = L.holes[jx];
      if (std::abs(L.jj[p] - L.jj[h]) > T.rank || L.jj[p] + L.jj[h] < T.rank) continue;
      if (L.tz[p] != L.tz[h]) continue;
      if ((L.ll[p] + L.ll[h] + T.dpar / 2) % 2) continue;
      push(T.off_fph + ix + (int64_t)jx * L.P, 0, 1, -1);
    }
  E.n1b = (int64_t)E.pos.size();
  auto same = [&](int ch, int cls, int i) {
    const int o = L.pair_off[ch * 3 + cls] + i;
    return L.pair_a[o] == L.pair_b[o];
  };
  for (int q = 0; q < T.nblocks; ++q) {
    if (T.q1[q] < 0) continue;
    const int J1 = T.J1[q], J2 = T.J2[q];
    const bool odd1 = ((J1 / 2) % 2) == 1, odd2 = ((J2 / 2) % 2) == 1;
    const int n1 = T.n1[q * 9 + 2], n2 = T.n2[q * 9 + 2];
    int qx = -1;
    if (J1 == J2) qx = T.block(J1, J2, T.T[q], ((T.dpar / 2) % 2) ? 1 - T.P1[q] : T.P1[q], L.JM);
    for (int II = 0; II < n1; ++II)
      for (int JJ = 0; JJ < n2; ++JJ) {
        if (odd1 && same(T.q1[q], 0, II)) continue;
        if (odd2 && same(T.q2[q], 2, JJ)) continue;
        const int64_t mi = (J1 == J2) ? T.goff[qx * 9 + 6] + JJ + (int64_t)II * T.n1[qx * 9 + 6] : -1;
        push(T.goff[q * 9 + 2] + II + (int64_t)JJ * n1, 1, 1, mi);
      }
    if (J1 == J2) continue;
    const int m1 = T.n1[q * 9 + 6], m2 = T.n2[q * 9 + 6];
    for (int II = 0; II < m1; ++II)
      for (int JJ = 0; JJ < m2; ++JJ) {
        if (odd1 && same(T.q1[q], 2, II)) continue;
        if (odd2 && same(T.q2[q], 0, JJ)) continue;
        push(T.goff[q * 9 + 6] + II + (int64_t)JJ * m1, 2, (((J1 - J2) / 2) & 1) ? -1 : 1, -1);
      }
  }
  E.n = (int64_t)E.pos.size();
}

void release(imsrg_eom* E) {
  if (E->gexec) cudaGraphExecDestroy(E->gexec);
  cudaFree(E->d_pos);
  cudaFree(E->d_mirror);
  cudaFree(E->d_kind);
  cudaFree(E->d_phase);
  cudaFree(E->d_v);
  cudaFree(E->d_w);
  for (int s = 0; s < 2; ++s) {
    cudaFree(E->d_S[s]);
    cudaFree(E->d_Y[s]);
  }
}

// 64-bit linear congruential start vector (Knuth's MMIX constants), uniform in [-1, 1)
void start_vector(std::vector<double>& v, uint64_t seed) {
  uint64_t x = seed * 0x9E3779B97F4A7C15ull + 1;
  for (double& e : v) {
    x = x * 6364136223846793005ull + 1442695040888963407ull;
    e = (double)(x >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  }
}

double hdot(const double* a, const double* b, int64_t n) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

// w <- w - V[:, 0:k] (V[:, 0:k]^T w), twice (classical Gram-Schmidt with one reorthogonalisation);
// returns the first pass's coefficients in h
void orthogonalize(const std::vector<double>& V, int64_t n, int k, double* w, std::vector<double>& h) {
  h.assign(k, 0.0);
  std::vector<double> c(k);
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = 0; i < k; ++i) c[i] = hdot(&V[(size_t)i * n], w, n);
    for (int i = 0; i < k; ++i) {
      const double* vi = &V[(size_t)i * n];
      for (int64_t r = 0; r < n; ++r) w[r] -= c[i] * vi[r];
      h[i] += c[i];
    }
  }
}

}  // namespace

// one EOM product on device vectors: w = rewrap([H, unwrap(v)])
imsrg_status Ctx::eom_matvec(imsrg_eom& E, const double* Hd, const double* d_v, double* d_w) {
  const int g = grid_of(E.n);
  k_eom_pack<<<g, 256, 0, stream>>>(E.n, E.d_pos, E.d_kind, E.d_phase, E.d_mirror, d_v, E.d_S[0], E.d_S[1]);
  CKE(launched("k_eom_pack"));
  CKE(tensor_commutator(*E.ts, Hd, 1, E.d_S[0], 1, E.d_Y[0], 127 | kTensorExcitation));
  CKE(tensor_commutator(*E.ts, Hd, 1, E.d_S[1], -1, E.d_Y[1], 127 | kTensorExcitation));
  k_eom_unpack<<<g, 256, 0, stream>>>(E.n, E.d_pos, E.d_kind, E.d_phase, E.d_Y[0], E.d_Y[1], d_w);
  return launched("k_eom_unpack");
}

// the product d_v -> d_w through the CUDA graph captured for Hd and the context's precision
// (captured on first use, after one direct run that also makes the workspaces; the operands are
// read when the graph runs)
imsrg_status Ctx::eom_matvec_graph(imsrg_eom& E, const double* Hd) {
  if (E.gexec && E.g_H == Hd && E.g_prec == (int)precision)
    return cuda(cudaGraphLaunch(E.gexec, stream), "cudaGraphLaunch(eom)");
  CKE(eom_matvec(E, Hd, E.d_v, E.d_w));
  CKE(cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize"));
  if (E.gexec) {
    cudaGraphExecDestroy(E.gexec);
    E.gexec = nullptr;
  }
  cudaGraph_t g = nullptr;
  CKE(cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed), "cudaStreamBeginCapture(eom)"));
  const imsrg_status s = eom_matvec(E, Hd, E.d_v, E.d_w);
  const imsrg_status e = cuda(cudaStreamEndCapture(stream, &g), "cudaStreamEndCapture(eom)");
  imsrg_status r = s != IMSRG_OK ? s : e;
  if (r == IMSRG_OK) r = cuda(cudaGraphInstantiate(&E.gexec, g, 0), "cudaGraphInstantiate(eom)");
  if (g) cudaGraphDestroy(g);
  if (r != IMSRG_OK) {
    E.gexec = nullptr;
    return r;
  }
  E.g_H = Hd;
  E.g_prec = (int)precision;
  return IMSRG_OK;  // d_w already holds the direct run's product
}

// host vectors in and out
imsrg_status Ctx::eom_matvec_host(imsrg_eom& E, const double* Hd, const double* v, double* w) {
  const size_t b = sizeof(double) * (size_t)E.n;
  CKE(cuda(cudaMemcpyAsync(E.d_v, v, b, cudaMemcpyHostToDevice, stream), "H2D eom vector"));
  CKE(eom_matvec_graph(E, Hd));
  CKE(cuda(cudaMemcpyAsync(w, E.d_w, b, cudaMemcpyDeviceToHost, stream), "D2H eom vector"));
  return cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
}

// LANCZOS_DIAGONALIZE (src/EOM_IMSRG.f90:164-334): the nev eigenvalues of smallest magnitude of
// the EOM matrix, ascending, and (optionally) their normalised amplitude vectors
imsrg_status Ctx::eom_lanczos(imsrg_eom& E, const double* Hd, int nev, double tol, int max_restarts,
                              double* energies, double* vectors, int32_t* matvecs, int32_t* restarts) {
  const int64_t n = E.n;
  const int m = (int)std::min<int64_t>(std::max(5 * nev, nev + 2), n);
  if (nev > m) return fail(IMSRG_ERR_INVALID_ARGUMENT, "nev exceeds the number of amplitudes");
  std::vector<double> V((size_t)n * (m + 1), 0.0), T((size_t)m * m, 0.0), w(n), h, theta, S;
  start_vector(w, 1);
  double nrm = std::sqrt(hdot(w.data(), w.data(), n));
  for (int64_t i = 0; i < n; ++i) V[i] = w[i] / nrm;
  int k = 0, nmv = 0, it = 0;
  double beta = 0.0;
  const double eps23 = std::pow(2.220446049250313e-16, 2.0 / 3.0);
  std::vector<int> want;
  bool converged = false;
  for (it = 0; it <= max_restarts; ++it) {
    for (int j = k; j < m; ++j) {
      CKE(eom_matvec_host(E, Hd, &V[(size_t)j * n], w.data()));
      ++nmv;
      orthogonalize(V, n, j + 1, w.data(), h);
      T[j + (size_t)j * m] = h[j];
      beta = std::sqrt(hdot(w.data(), w.data(), n));
      double* next = &V[(size_t)(j + 1) * n];
      if (beta > 1e-13 * std::max(1.0, std::fabs(h[j]))) {
        for (int64_t i = 0; i < n; ++i) next[i] = w[i] / beta;
      } else {  // invariant subspace: continue from a fresh direction orthogonal to the basis
        beta = 0.0;
        std::fill(next, next + n, 0.0);
        if (j + 1 < n) {
          std::vector<double> hh;
          start_vector(w, 2 + j + (uint64_t)it * m);
          orthogonalize(V, n, j + 1, w.data(), hh);
          nrm = std::sqrt(hdot(w.data(), w.data(), n));
          if (nrm > 0.0)
            for (int64_t i = 0; i < n; ++i) next[i] = w[i] / nrm;
        }
      }
      if (j + 1 < m) T[(j + 1) + (size_t)j * m] = T[j + (size_t)(j + 1) * m] = beta;
    }
    imsrg::jacobi_eigen(m, T, theta, S);
    // Ritz values of smallest magnitude first
    std::vector<int> order(m);
    for (int i = 0; i < m; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return std::fabs(theta[a]) < std::fabs(theta[b]); });
    want.assign(order.begin(), order.begin() + nev);
    converged = true;
    for (int i : want)
      if (std::fabs(beta * S[(m - 1) + (size_t)i * m]) > tol * std::max(eps23, std::fabs(theta[i]))) converged = false;
    if (converged || it == max_restarts || m == n) break;
    // thick restart: keep the kn Ritz pairs of smallest magnitude, the residual direction next
    const int kn = std::min(m - 1, nev + (m - nev) / 2);
    std::vector<double> W((size_t)n * kn, 0.0);
    for (int c = 0; c < kn; ++c) {
      const int i = order[c];
      double* wc = &W[(size_t)c * n];
      for (int r = 0; r < m; ++r) {
        const double s = S[r + (size_t)i * m];
        const double* vr = &V[(size_t)r * n];
        for (int64_t x = 0; x < n; ++x) wc[x] += s * vr[x];
      }
    }
    std::memcpy(&V[(size_t)kn * n], &V[(size_t)m * n], sizeof(double) * (size_t)n);
    std::memcpy(V.data(), W.data(), sizeof(double) * W.size());
    std::fill(T.begin(), T.end(), 0.0);
    for (int c = 0; c < kn; ++c) {
      const int i = order[c];
      T[c + (size_t)c * m] = theta[i];
      T[c + (size_t)kn * m] = T[kn + (size_t)c * m] = beta * S[(m - 1) + (size_t)i * m];
    }
    k = kn;
  }
  std::sort(want.begin(), want.end(), [&](int a, int b) { return theta[a] < theta[b]; });
  for (int c = 0; c < nev; ++c) {
    const int i = want[c];
    energies[c] = theta[i];
    if (vectors) {
      double* out = vectors + (size_t)c * n;
      std::fill(out, out + n, 0.0);
      for (int r = 0; r < m; ++r) {
        const double s = S[r + (size_t)i * m];
        const double* vr = &V[(size_t)r * n];
        for (int64_t x = 0; x < n; ++x) out[x] += s * vr[x];
      }
      const double q = std::sqrt(hdot(out, out, n));
      for (int64_t x = 0; x < n; ++x) out[x] /= q;
    }
  }
  if (matvecs) *matvecs = nmv;
  if (restarts) *restarts = it;
  if (!converged && m < n)
    return fail(IMSRG_ERR_NOT_CONVERGED, "EOM Lanczos did not converge within max_restarts");
  return IMSRG_OK;
}

// ====================================================================== C ABI
#define ECTX(ptr)                                                                        \
  if (!(ptr)) return IMSRG_ERR_INVALID_ARGUMENT;                                         \
  Ctx* c = reinterpret_cast<Ctx*>(ptr);                                                  \
  if (c->device < 0) return c->fail(IMSRG_ERR_UNSUPPORTED, "host-only context (device < 0)"); \
  {                                                                                      \
    cudaError_t _e = cudaSetDevice(c->device);                                           \
    if (_e != cudaSuccess) return c->cuda(_e, "cudaSetDevice");                          \
  }

extern "C" {

imsrg_status imsrg_eom_create(imsrg_ctx* ctx, int32_t rank2, int32_t dpar2, imsrg_eom** out) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (c->device >= 0) {
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return c->cuda(e, "cudaSetDevice");
  }
  if (!out || rank2 < 0 || (rank2 & 1) || (dpar2 != 0 && dpar2 != 2))
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_create: rank2 even >= 0, dpar2 0 or 2");
  *out = nullptr;
  TensorState* s = nullptr;
  CKE(c->tensor_state(rank2, dpar2, &s));
  imsrg_eom* E = new (std::nothrow) imsrg_eom();
  if (!E) return IMSRG_ERR_OUT_OF_MEMORY;
  E->owner = c;
  E->ts = s;
  E->rank = rank2;
  E->dpar = dpar2;
  build_map(c->L, s->T, *E);
  if (c->device < 0) {  // host-only context: the amplitude map alone
    *out = E;
    return IMSRG_OK;
  }
  const size_t n = (size_t)std::max<int64_t>(E->n, 1), sb = sizeof(double) * (size_t)s->T.slab;
  imsrg_status st = IMSRG_OK;
  auto alloc = [&](void** p, size_t b, const char* what) {
    if (st == IMSRG_OK) st = c->cuda(cudaMalloc(p, b), what);
  };
  alloc((void**)&E->d_pos, sizeof(int64_t) * n, "cudaMalloc(eom map)");
  alloc((void**)&E->d_mirror, sizeof(int64_t) * n, "cudaMalloc(eom map)");
  alloc((void**)&E->d_kind, n, "cudaMalloc(eom map)");
  alloc((void**)&E->d_phase, n, "cudaMalloc(eom map)");
  alloc((void**)&E->d_v, sizeof(double) * n, "cudaMalloc(eom vector)");
  alloc((void**)&E->d_w, sizeof(double) * n, "cudaMalloc(eom vector)");
  for (int k = 0; k < 2; ++k) {
    alloc((void**)&E->d_S[k], sb, "cudaMalloc(eom slab)");
    alloc((void**)&E->d_Y[k], sb, "cudaMalloc(eom slab)");
  }
  if (st == IMSRG_OK && E->n) {
    st = c->cuda(cudaMemcpy(E->d_pos, E->pos.data(), sizeof(int64_t) * E->n, cudaMemcpyHostToDevice), "H2D eom map");
    if (st == IMSRG_OK)
      st = c->cuda(cudaMemcpy(E->d_mirror, E->mirror.data(), sizeof(int64_t) * E->n, cudaMemcpyHostToDevice),
                   "H2D eom map");
    if (st == IMSRG_OK) st = c->cuda(cudaMemcpy(E->d_kind, E->kind.data(), E->n, cudaMemcpyHostToDevice), "H2D eom map");
    if (st == IMSRG_OK)
      st = c->cuda(cudaMemcpy(E->d_phase, E->phase.data(), E->n, cudaMemcpyHostToDevice), "H2D eom map");
  }
  for (int k = 0; k < 2 && st == IMSRG_OK; ++k) st = c->cuda(cudaMemsetAsync(E->d_S[k], 0, sb, c->stream), "memset(eom slab)");
  if (st == IMSRG_OK) st = c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  if (st != IMSRG_OK) {
    release(E);
    delete E;
    return st;
  }
  *out = E;
  return IMSRG_OK;
}

imsrg_status imsrg_eom_destroy(imsrg_ctx* ctx, imsrg_eom* E) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (!E) return IMSRG_OK;
  if (E->owner != c) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "EOM handle of another context");
  if (c->device >= 0) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    release(E);
  }
  delete E;
  return IMSRG_OK;
}

imsrg_status imsrg_eom_dim(imsrg_ctx* ctx, const imsrg_eom* E, int64_t* n, int64_t* n1b) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (!E || E->owner != c) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_dim");
  if (n) *n = E->n;
  if (n1b) *n1b = E->n1b;
  return IMSRG_OK;
}

imsrg_status imsrg_eom_amplitude_map(imsrg_ctx* ctx, const imsrg_eom* E, int64_t* pos, int8_t* kind, int8_t* phase,
                                     int64_t* mirror) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (!E || E->owner != c) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_amplitude_map");
  for (int64_t k = 0; k < E->n; ++k) {
    if (pos) pos[k] = E->pos[k];
    if (kind) kind[k] = E->kind[k];
    if (phase) phase[k] = E->phase[k];
    if (mirror) mirror[k] = E->mirror[k];
  }
  return IMSRG_OK;
}

imsrg_status imsrg_eom_matvec(imsrg_ctx* ctx, imsrg_eom* E, const imsrg_op* H, const double* v, double* w) {
  ECTX(ctx);
  if (!E || E->owner != c || !H || H->owner != c || !v || !w)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_matvec");
  if (H->herm != 1) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_matvec: H must be hermitian");
  return c->eom_matvec_host(*E, H->d, v, w);
}

imsrg_status imsrg_eom_matvec_device(imsrg_ctx* ctx, imsrg_eom* E, const imsrg_op* H, const double* d_v, double* d_w) {
  ECTX(ctx);
  if (!E || E->owner != c || !H || H->owner != c || !d_v || !d_w)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_matvec_device");
  if (H->herm != 1) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_matvec_device: H must be hermitian");
  return c->eom_matvec(*E, H->d, d_v, d_w);
}

imsrg_status imsrg_eom_unwrap(imsrg_ctx* ctx, imsrg_eom* E, const double* v, imsrg_tensor* X) {
  ECTX(ctx);
  if (!E || E->owner != c || !v || !X || X->owner != c) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_unwrap");
  if (X->ts != E->ts) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_unwrap: tensor of another rank or parity");
  CKE(c->cuda(cudaMemsetAsync(X->d, 0, sizeof(double) * (size_t)E->ts->T.slab, c->stream), "memset(ladder)"));
  CKE(c->cuda(cudaMemcpyAsync(E->d_v, v, sizeof(double) * (size_t)E->n, cudaMemcpyHostToDevice, c->stream),
              "H2D eom vector"));
  k_eom_unwrap<<<grid_of(E->n), 256, 0, c->stream>>>(E->n, E->d_pos, E->d_mirror, E->d_v, X->d);
  CKE(c->launched("k_eom_unwrap"));
  X->herm = 1;
  return c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
}

imsrg_status imsrg_eom_rewrap(imsrg_ctx* ctx, imsrg_eom* E, const imsrg_tensor* X, double* v) {
  ECTX(ctx);
  if (!E || E->owner != c || !v || !X || X->owner != c) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_rewrap");
  if (X->ts != E->ts) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_rewrap: tensor of another rank or parity");
  k_eom_rewrap<<<grid_of(E->n), 256, 0, c->stream>>>(E->n, E->d_pos, X->d, E->d_w);
  CKE(c->launched("k_eom_rewrap"));
  CKE(c->cuda(cudaMemcpyAsync(v, E->d_w, sizeof(double) * (size_t)E->n, cudaMemcpyDeviceToHost, c->stream),
              "D2H eom vector"));
  return c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
}

imsrg_status imsrg_eom_lanczos(imsrg_ctx* ctx, imsrg_eom* E, const imsrg_op* H, int32_t nev, double tol,
                               int32_t max_restarts, double* energies, double* vectors, int32_t* matvecs,
                               int32_t* restarts) {
  ECTX(ctx);
  if (!E || E->owner != c || !H || H->owner != c || !energies || nev < 1 || tol <= 0.0 || max_restarts < 0)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_lanczos");
  if (H->herm != 1) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_lanczos: H must be hermitian");
  if (nev > E->n) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_eom_lanczos: nev exceeds the amplitude count");
  return c->eom_lanczos(*E, H->d, nev, tol, max_restarts, energies, vectors, matvecs, restarts);
}

}  // extern "C"
