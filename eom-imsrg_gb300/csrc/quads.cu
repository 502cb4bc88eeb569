// BCH_EXPAND with quads = 'y' (src/IMSRG_MAGNUS.f90:149-234): each nested commutator first receives
// the correction INT3 of the previous term, then restore_quadrupoles (:908-1070) rebuilds INT3 from
// the operator just commuted.  INT3 is nonzero only in its pp-hh arrays.  restore_quadrupoles:
//   1. the intermediates of build_intermediates_For_intermediates (:1073-1132), per channel
//        W1_hhhh = hX X3^T OM3, W1_pppp = hOM X3 OM3^T, W2_hhhh = hOM OM3^T OM3, W2_pppp = hOM OM3 OM3^T
//      (X3, OM3 the pp-hh arrays), as one grouped FP64 GEMM over all channels;
//   2. their one-body insertions: f1_hh(i,j) = sum_{c hole, J} (J+1) W1(ci,cj)/(j_i+1), the same from
//      W2, and over particles f1_pp(i,j) = hX hOM sum_{c particle, J} (J+1) W1(cj,ci)/(j_i+1)
//      for i <= j only (the reference fills that triangle alone);
//   3. the assignment of every pp-hh element of INT3 from the insertions and the two-body
//      elements of OM and X.
// In the channels step 1 skips (np nh = 0) the reference's w1 / w2 still hold what
// commutator_222_pp_hh(G, AD) left there in the same BCH step (src/commutators.f90:581-640):
// W1_pppp = OM_pppp X_pppp where only pp pairs exist, W2_hhhh = OM_hhhh X_hhhh where only hh pairs
// do, zero otherwise; the insertions read those, so the grouped GEMM forms them as well.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "engine.h"
#include "gemm.h"
#include "kernels.h"

using namespace imsrg;

// workspace of the quadrupole restoration, built on first use
struct QuadState {
  void* tables = nullptr;
  const GemmProb* p = nullptr;
  const GemmTile* t = nullptr;
  const int64_t* pre = nullptr;  // prefix counts of np*nh over the channels
  int nt = 0;
  int64_t n3 = 0;
  double *w1 = nullptr, *w2 = nullptr, *ins = nullptr, *int3 = nullptr;
};

namespace {

#define CKQ(expr)                  \
  do {                             \
    imsrg_status _s = (expr);      \
    if (_s != IMSRG_OK) return _s; \
  } while (0)

// the one-body insertions: ins = [f1_hh A*A][f2_hh A*A][f1_pp P*P][f2_pp P*P]
__global__ void k_quad_insert(DevLayout D, const double* __restrict__ W1, const double* __restrict__ W2, int hX,
                              int hOM, double* __restrict__ ins) {
  const int A = D.A, P = D.P;
  const int64_t nA = (int64_t)A * A, nP = (int64_t)P * P;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nA + nP; e += (int64_t)gridDim.x * blockDim.x) {
    const bool hole = e < nA;
    const int64_t f = hole ? e : e - nA;
    const int n = hole ? A : P;
    const int i = (int)(f % n), j = (int)(f / n);
    const int* orb = hole ? D.holes : D.parts;
    const int ik = orb[i], jk = orb[j], ji = D.jj[ik];
    double sm = 0.0, sm2 = 0.0;
    const bool live = D.jj[jk] == ji && D.ll[jk] == D.ll[ik] && D.tz[jk] == D.tz[ik] && (hole || j >= i);
    if (live)
      for (int c = 0; c < n; ++c) {
        const int ck = orb[c], jc = D.jj[ck];
        for (int JT = abs(jc - ji); JT <= jc + ji; JT += 2) {
          if (hole) {
            sm += d_v_elem(D, W1, 1, ck, ik, ck, jk, JT) * (JT + 1);
            sm2 += d_v_elem(D, W2, 1, ck, ik, ck, jk, JT) * (JT + 1);
          } else {
            sm += hX * hOM * d_v_elem(D, W1, 1, ck, jk, ck, ik, JT) * (JT + 1);
            sm2 += d_v_elem(D, W2, 1, ck, jk, ck, ik, JT) * (JT + 1);
          }
        }
      }
    double* f1 = hole ? ins : ins + 2 * nA;
    double* f2 = hole ? ins + nA : ins + 2 * nA + nP;
    f1[f] = sm / (ji + 1.0);
    f2[f] = sm2 / (ji + 1.0);
  }
}

__device__ __forceinline__ double qsgn(int n) { return (n & 1) ? -1.0 : 1.0; }

// the pp-hh elements of RES (assigned)
__global__ void k_quad_assign(DevLayout D, const int64_t* __restrict__ pre, const double* __restrict__ X, int hX,
                              const double* __restrict__ OM, int hOM, const double* __restrict__ ins,
                              double* __restrict__ RES) {
  const int A = D.A, P = D.P, nb = D.nblocks;
  const int64_t nA = (int64_t)A * A, nP = (int64_t)P * P;
  const double *f1h = ins, *f2h = ins + nA, *f1p = ins + 2 * nA, *f2p = ins + 2 * nA + nP;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < pre[nb]; e += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (pre[mid] <= e) lo = mid;
      else hi = mid - 1;
    }
    const int q = lo, np = D.ncls[q * 3];
    const int64_t f = e - pre[q];
    const int II = (int)(f / np), AA = (int)(f - (int64_t)II * np);
    const int J = D.lamJ[q];
    const int a = D.pair_a[D.pair_off[q * 3] + AA], b = D.pair_b[D.pair_off[q * 3] + AA];
    const int i = D.pair_a[D.pair_off[q * 3 + 2] + II], j = D.pair_b[D.pair_off[q * 3 + 2] + II];
    const double sij = qsgn((D.jj[i] + D.jj[j] - J) / 2), sab = qsgn((D.jj[a] + D.jj[b] - J) / 2);
    const int h1 = D.loc[i], h2 = D.loc[j], p1 = D.loc[a], p2 = D.loc[b];
    double x = 0.0;
    for (int c = 0; c < A; ++c) {
      const int cx = D.holes[c];
      x += -f1h[h1 + (int64_t)c * A] * d_v_elem(D, OM, hOM, a, b, cx, j, J) +
           sij * f1h[h2 + (int64_t)c * A] * d_v_elem(D, OM, hOM, a, b, cx, i, J) +
           f2h[h1 + (int64_t)c * A] * d_v_elem(D, X, hX, a, b, cx, j, J) -
           sij * f2h[h2 + (int64_t)c * A] * d_v_elem(D, X, hX, a, b, cx, i, J);
    }
    for (int c = 0; c < P; ++c) {
      const int cx = D.parts[c];
      x += -f1p[p1 + (int64_t)c * P] * d_v_elem(D, OM, hOM, cx, b, i, j, J) +
           sab * f1p[p2 + (int64_t)c * P] * d_v_elem(D, OM, hOM, cx, a, i, j, J) +
           f2p[p1 + (int64_t)c * P] * d_v_elem(D, X, hX, cx, b, i, j, J) -
           sab * f2p[p2 + (int64_t)c * P] * d_v_elem(D, X, hX, cx, a, i, j, J);
    }
    RES[D.goff[q * 6 + 2] + f] = x;
  }
}

int grid_q(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

}  // namespace

imsrg_status Ctx::quads_prepare() {
  if (qs) return IMSRG_OK;
  QuadState* s = new QuadState();
  std::vector<GemmProb> P;
  std::vector<int64_t> pre{0};
  for (int q = 0; q < L.nblocks; ++q) {
    const int np = L.ncls[q][0], nb = L.ncls[q][1], nh = L.ncls[q][2];
    const bool live = np * nh != 0 && nh + np != 0 && np + nb != 0 && nh + nb != 0;
    pre.push_back(pre.back() + (int64_t)np * nh);
    const int64_t o3 = L.goff[q * 6 + 2], o1 = L.goff[q * 6 + 0], o5 = L.goff[q * 6 + 4];
    if (!live) {
      // what commutator_222_pp_hh(OM, X) leaves in the reference's workspace there
      auto sq = [&](int c_id, int64_t off, int n) {
        GemmProb p{};
        p.c_id = c_id; p.c_off = off; p.M = n; p.N = n; p.ldc = n; p.nterm = 1;
        GemmTerm& t = p.t[0];
        t.a_id = kOpR; t.a_off = off; t.lda = n; t.ta = 0;
        t.b_id = kOpL; t.b_off = off; t.ldb = n; t.tb = 0;
        t.K = n; t.alpha = kAlphaOne;
        P.push_back(p);
      };
      if (np) sq(kOpW1, o1, np);  // W1_pppp = OM_pppp X_pppp
      if (nh) sq(kOpW2, o5, nh);  // W2_hhhh = OM_hhhh X_hhhh
      continue;
    }
    auto prob = [&](int c_id, int64_t c_off, int M, int N, int a_id, int ta, int b_id, int tb, int K, int alpha) {
      GemmProb p{};
      p.c_id = c_id; p.c_off = c_off; p.M = M; p.N = N; p.ldc = M; p.nterm = 1;
      GemmTerm& t = p.t[0];
      t.a_id = a_id; t.a_off = o3; t.lda = np; t.ta = ta;
      t.b_id = b_id; t.b_off = o3; t.ldb = np; t.tb = tb;
      t.K = K; t.alpha = alpha;
      P.push_back(p);
    };
    prob(kOpW1, o5, nh, nh, kOpL, 1, kOpR, 0, np, kAlphaHL);  // W1_hhhh = hX X3^T OM3
    prob(kOpW1, o1, np, np, kOpL, 0, kOpR, 1, nh, kAlphaHR);  // W1_pppp = hOM X3 OM3^T
    prob(kOpW2, o5, nh, nh, kOpR, 1, kOpR, 0, np, kAlphaHR);  // W2_hhhh = hOM OM3^T OM3
    prob(kOpW2, o1, np, np, kOpR, 0, kOpR, 1, nh, kAlphaHR);  // W2_pppp = hOM OM3 OM3^T
  }
  const auto tiles = build_tiles(P, 64, 64);
  const size_t bp = (sizeof(GemmProb) * std::max<size_t>(P.size(), 1) + 255) & ~size_t(255);
  const size_t bt = (sizeof(GemmTile) * std::max<size_t>(tiles.size(), 1) + 255) & ~size_t(255);
  const size_t br = sizeof(int64_t) * pre.size();
  imsrg_status st = cuda(cudaMalloc(&s->tables, bp + bt + br), "cudaMalloc(quadrupole tables)");
  if (st == IMSRG_OK && !P.empty())
    st = cuda(cudaMemcpy(s->tables, P.data(), sizeof(GemmProb) * P.size(), cudaMemcpyHostToDevice), "H2D quads");
  if (st == IMSRG_OK && !tiles.empty())
    st = cuda(cudaMemcpy((char*)s->tables + bp, tiles.data(), sizeof(GemmTile) * tiles.size(), cudaMemcpyHostToDevice),
              "H2D quads");
  if (st == IMSRG_OK)
    st = cuda(cudaMemcpy((char*)s->tables + bp + bt, pre.data(), br, cudaMemcpyHostToDevice), "H2D quads");
  s->p = reinterpret_cast<const GemmProb*>(s->tables);
  s->t = reinterpret_cast<const GemmTile*>((char*)s->tables + bp);
  s->pre = reinterpret_cast<const int64_t*>((char*)s->tables + bp + bt);
  s->nt = (int)tiles.size();
  s->n3 = pre.back();
  const size_t sb = sizeof(double) * (size_t)L.slab;
  const size_t ib = sizeof(double) * (2 * (size_t)L.A * L.A + 2 * (size_t)L.P * L.P);
  for (double** p : {&s->w1, &s->w2, &s->int3})
    if (st == IMSRG_OK) st = cuda(cudaMalloc(p, sb), "cudaMalloc(quadrupole workspace)");
  if (st == IMSRG_OK) st = cuda(cudaMalloc(&s->ins, std::max<size_t>(ib, 8)), "cudaMalloc(quadrupole insertions)");
  for (double* p : {s->w1, s->w2})
    if (st == IMSRG_OK) st = cuda(cudaMemset(p, 0, sb), "memset(quadrupole workspace)");
  if (st != IMSRG_OK) {
    for (void* p : {s->tables, (void*)s->w1, (void*)s->w2, (void*)s->int3, (void*)s->ins})
      if (p) cudaFree(p);
    delete s;
    return st;
  }
  qs = s;
  return IMSRG_OK;
}

double* Ctx::quads_int3() { return qs ? qs->int3 : nullptr; }

void Ctx::quads_release() {
  if (!qs) return;
  for (void* p : {qs->tables, (void*)qs->w1, (void*)qs->w2, (void*)qs->int3, (void*)qs->ins})
    if (p) cudaFree(p);
  delete qs;
  qs = nullptr;
}

// restore_quadrupoles(X, OM) -> the pp-hh arrays of RES (the rest of RES untouched)
imsrg_status Ctx::restore_quadrupoles(const double* X, int hX, const double* OM, int hOM, double* RES) {
  CKQ(quads_prepare());
  if (qs->nt) {
    GemmOperands ops{};
    ops.in[kOpL] = X; ops.in[kOpR] = OM;
    ops.out[kOpW1] = qs->w1; ops.out[kOpW2] = qs->w2;
    ops.hL = hX; ops.hR = hOM;
    k_gemm_fp64<<<qs->nt, 256, 0, stream>>>(qs->p, qs->t, ops);
    CKQ(launched("k_gemm_fp64(quadrupole intermediates)"));
  }
  const int64_t ni = (int64_t)L.A * L.A + (int64_t)L.P * L.P;
  k_quad_insert<<<grid_q(ni), 256, 0, stream>>>(D, qs->w1, qs->w2, hX, hOM, qs->ins);
  CKQ(launched("k_quad_insert"));
  if (qs->n3) {
    k_quad_assign<<<grid_q(qs->n3), 256, 0, stream>>>(D, qs->pre, X, hX, OM, hOM, qs->ins, RES);
    CKQ(launched("k_quad_assign"));
  }
  return IMSRG_OK;
}

// ====================================================================== C ABI
#define QCTX(ptr)                                                                        \
  if (!(ptr)) return IMSRG_ERR_INVALID_ARGUMENT;                                         \
  Ctx* c = reinterpret_cast<Ctx*>(ptr);                                                  \
  if (c->device < 0) return c->fail(IMSRG_ERR_UNSUPPORTED, "host-only context (device < 0)"); \
  {                                                                                      \
    cudaError_t _e = cudaSetDevice(c->device);                                           \
    if (_e != cudaSuccess) return c->cuda(_e, "cudaSetDevice");                          \
  }

extern "C" {

imsrg_status imsrg_restore_quadrupoles(imsrg_ctx* ctx, const imsrg_op* X, const imsrg_op* OM, imsrg_op* RES) {
  QCTX(ctx);
  if (!X || X->owner != c || !OM || OM->owner != c || !RES || RES->owner != c || RES == X || RES == OM)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_restore_quadrupoles");
  CKQ(c->cuda(cudaMemsetAsync(RES->d, 0, sizeof(double) * (size_t)c->L.slab, c->stream), "memset(RES)"));
  RES->herm = 1;
  CKQ(c->restore_quadrupoles(X->d, X->herm, OM->d, OM->herm, RES->d));
  return c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
}

}  // extern "C"
