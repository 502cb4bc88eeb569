// Reverse mode of the FP64 commutator and of the White generator on the device: the
// building blocks of the adjoint dE0/dtheta of a Magnus flow (the flow-level reverse
// sweep over checkpointed Omega(s) is driven from the host, imsrg_gb300/adjoint.py).
//
// Ctx::commutator_vjp reverses Ctx::commutator's FP64 sequence (pandya, 110/220, 111,
// 121, 122, 222_pp_hh, 221, 222_ph) piece by piece in the opposite order, carrying the
// cotangent of RES through the pieces' assign / accumulate / mirror writes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "../../include/imsrg_gb300.h"
#include "engine.h"
#include "kernels.h"

using namespace imsrg;

namespace imsrg {
__global__ void k_vjp_222ph(DevLayout D, double* cb, int hL, int hR, int hRES, double* Wb);
__global__ void k_vjp_221(DevLayout D, int pm, double* cb, int hRES, double* w1b, double* w2b);
__global__ void k_vjp_pphh_wbar(DevLayout D, const double* cb, double* w1b, double* w2b, double pm);
__global__ void k_vjp_122(DevLayout D, const double* L, int hL, const double* R, int hR, double* cb, int hRES,
                          double* Lb, double* Rb);
__global__ void k_vjp_121(DevLayout D, const double* L, int hL, const double* R, int hR, double* cb, int hRES,
                          double* Lb, double* Rb);
__global__ void k_vjp_111(DevLayout D, const double* L, int hL, const double* R, int hR, const double* cb,
                          double* Lb, double* Rb);
__global__ void k_vjp_e0(DevLayout D, const double* L, int hL, const double* R, int hR, const double* cb, double* Lb,
                         double* Rb);
__global__ void k_pandya_vjp(DevLayout D, int herm, const double* ccb, double* opb);
__global__ void k_white_vjp_1b(DevLayout D, const double* H, int hH, const double* ETAb, double* Hb);
__global__ void k_white_vjp_2b(DevLayout D, const double* H, int hH, const double* mono, const double* ETAb,
                               double* Hb, double* monob);
__global__ void k_monopole_vjp(DevLayout D, int hH, const double* monob, double* Hb);
__global__ void k_dot_partial(const double* x, const double* y, int64_t n, double* partial);
}  // namespace imsrg

struct AdjointState {
  double* cb = nullptr;     // running cotangent of RES (slab)
  double* lccb = nullptr;   // cotangents of LCC / RCC
  double* rccb = nullptr;
  double* wccb = nullptr;   // cotangent of WCC (FP64, wcc_size)
  double* monob = nullptr;  // N x N monopole cotangents
  double* partial = nullptr;
  void* tables = nullptr;
  const GemmProb* pphh_p = nullptr;
  const GemmTile* pphh_t = nullptr;
  const GemmProb* wcc_p = nullptr;
  const GemmTile* wcc_t = nullptr;
  int n_pphh_t = 0, n_wcc_t = 0;
};

namespace {
constexpr int kDotBlocks = 1024;
int grid_of(int64_t n, int threads = 256, int cap = 152 * 16) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, cap));
}
}  // namespace

#define CKA(expr)                 \
  do {                            \
    imsrg_status _s = (expr);     \
    if (_s != IMSRG_OK) return _s; \
  } while (0)

imsrg_status Ctx::adjoint_prepare() {
  if (adj) return IMSRG_OK;
  CKA(ensure_workspace());
  adj = new AdjointState();
  const Layout& l = L;
  CKA(cuda(cudaMalloc(&adj->cb, sizeof(double) * (size_t)l.slab), "cudaMalloc(adjoint cb)"));
  CKA(cuda(cudaMalloc(&adj->lccb, sizeof(double) * std::max<int64_t>(l.cc_size, 1)), "cudaMalloc(LCCb)"));
  CKA(cuda(cudaMalloc(&adj->rccb, sizeof(double) * std::max<int64_t>(l.cc_size, 1)), "cudaMalloc(RCCb)"));
  CKA(cuda(cudaMalloc(&adj->wccb, sizeof(double) * std::max<int64_t>(l.wcc_size, 1)), "cudaMalloc(WCCb)"));
  CKA(cuda(cudaMalloc(&adj->monob, sizeof(double) * (size_t)l.N * l.N), "cudaMalloc(monopole cotangents)"));
  CKA(cuda(cudaMalloc(&adj->partial, sizeof(double) * kDotBlocks), "cudaMalloc(dot partials)"));
  const auto pp = build_pphh_vjp_problems(l.nblocks, l.ncls, l.goff);
  const auto pt = build_tiles(pp, 64, 64);
  const auto wp = build_wcc_vjp_problems(l.ncc, l.cc_rlen, l.cc_nph, l.cc_off, l.wcc_off);
  const auto wt = build_tiles(wp, 64, 64);
  size_t o[5] = {0};
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  o[1] = al(o[0] + sizeof(GemmProb) * pp.size());
  o[2] = al(o[1] + sizeof(GemmTile) * pt.size());
  o[3] = al(o[2] + sizeof(GemmProb) * wp.size());
  o[4] = al(o[3] + sizeof(GemmTile) * wt.size());
  std::vector<char> buf(std::max<size_t>(o[4], 256));
  if (!pp.empty()) std::memcpy(buf.data() + o[0], pp.data(), sizeof(GemmProb) * pp.size());
  if (!pt.empty()) std::memcpy(buf.data() + o[1], pt.data(), sizeof(GemmTile) * pt.size());
  if (!wp.empty()) std::memcpy(buf.data() + o[2], wp.data(), sizeof(GemmProb) * wp.size());
  if (!wt.empty()) std::memcpy(buf.data() + o[3], wt.data(), sizeof(GemmTile) * wt.size());
  CKA(cuda(cudaMalloc(&adj->tables, buf.size()), "cudaMalloc(adjoint tables)"));
  CKA(cuda(cudaMemcpy(adj->tables, buf.data(), buf.size(), cudaMemcpyHostToDevice), "cudaMemcpy(adjoint tables)"));
  const char* base = static_cast<const char*>(adj->tables);
  adj->pphh_p = reinterpret_cast<const GemmProb*>(base + o[0]);
  adj->pphh_t = reinterpret_cast<const GemmTile*>(base + o[1]);
  adj->wcc_p = reinterpret_cast<const GemmProb*>(base + o[2]);
  adj->wcc_t = reinterpret_cast<const GemmTile*>(base + o[3]);
  adj->n_pphh_t = (int)pt.size();
  adj->n_wcc_t = (int)wt.size();
  return IMSRG_OK;
}

void Ctx::adjoint_release() {
  if (!adj) return;
  for (void* p : {(void*)adj->cb, (void*)adj->lccb, (void*)adj->rccb, (void*)adj->wccb, (void*)adj->monob,
                  (void*)adj->partial, adj->tables})
    if (p) cudaFree(p);
  delete adj;
  adj = nullptr;
}

imsrg_status Ctx::commutator_vjp(const double* Lp, int hL, const double* Rp, int hR, int hRES, bool with_e0,
                                 const double* Cb, double* Lb, double* Rb) {
  CKA(adjoint_prepare());
  const Layout& l = L;
  const size_t sb = sizeof(double) * (size_t)l.slab;
  AdjointState& a = *adj;
  CKA(cuda(cudaMemcpyAsync(a.cb, Cb, sb, cudaMemcpyDeviceToDevice, stream), "copy cotangent"));
  CKA(cuda(cudaMemsetAsync(d_w1, 0, sb, stream), "memset(w1b)"));
  CKA(cuda(cudaMemsetAsync(d_w2, 0, sb, stream), "memset(w2b)"));
  if (l.cc_size) {
    CKA(cuda(cudaMemsetAsync(a.lccb, 0, sizeof(double) * l.cc_size, stream), "memset(LCCb)"));
    CKA(cuda(cudaMemsetAsync(a.rccb, 0, sizeof(double) * l.cc_size, stream), "memset(RCCb)"));
    CKA(cuda(cudaMemsetAsync(a.wccb, 0, sizeof(double) * l.wcc_size, stream), "memset(WCCb)"));
    // forward Pandya transforms (inputs of the WCC transposes)
    CKA(pandya(Lp, hL, d_lcc));
    CKA(pandya(Rp, hR, d_rcc));
  }
  const int pm = hL * hR;
  if (l.n_unique) {  // 222_ph: RES cotangent -> WCC cotangent -> LCC / RCC cotangents
    k_vjp_222ph<<<grid_of(l.n_unique), 256, 0, stream>>>(D, a.cb, hL, hR, hRES, a.wccb);
    CKA(launched("k_vjp_222ph"));
  }
  if (a.n_wcc_t) {
    GemmOperands ops{};
    ops.in[kOpWCC] = a.wccb; ops.in[kOpLCC] = d_lcc; ops.in[kOpRCC] = d_rcc;
    ops.out[kOpLCC] = a.lccb; ops.out[kOpRCC] = a.rccb;
    ops.hL = hL; ops.hR = hR;
    k_gemm_fp64<<<a.n_wcc_t, 256, 0, stream>>>(a.wcc_p, a.wcc_t, ops);
    CKA(launched("k_gemm_fp64(wcc vjp)"));
  }
  if (D.n_ob) {  // 221: one-body cotangent -> w1 / w2 cotangents
    k_vjp_221<<<(D.n_ob * 32 + 255) / 256, 256, 0, stream>>>(D, pm, a.cb, hRES, d_w1, d_w2);
    CKA(launched("k_vjp_221"));
  }
  // 222_pp_hh: RES accumulation -> W cotangents -> L / R cotangents
  k_vjp_pphh_wbar<<<grid_of(l.slab - l.goff[0]), 256, 0, stream>>>(D, a.cb, d_w1, d_w2, (double)pm);
  CKA(launched("k_vjp_pphh_wbar"));
  if (a.n_pphh_t) {
    GemmOperands ops{};
    ops.in[kOpL] = Lp; ops.in[kOpR] = Rp; ops.in[kOpW1] = d_w1; ops.in[kOpW2] = d_w2;
    ops.out[kOpL] = Lb; ops.out[kOpR] = Rb;
    ops.hL = hL; ops.hR = hR;
    k_gemm_fp64<<<a.n_pphh_t, 256, 0, stream>>>(a.pphh_p, a.pphh_t, ops);
    CKA(launched("k_gemm_fp64(pphh vjp)"));
  }
  if (l.n_unique) {
    k_vjp_122<<<grid_of(l.n_unique), 256, 0, stream>>>(D, Lp, hL, Rp, hR, a.cb, hRES, Lb, Rb);
    CKA(launched("k_vjp_122"));
  }
  if (D.n_ob) {
    k_vjp_121<<<(D.n_ob * 32 + 255) / 256, 256, 0, stream>>>(D, Lp, hL, Rp, hR, a.cb, hRES, Lb, Rb);
    CKA(launched("k_vjp_121"));
  }
  {
    const int64_t n1 = (int64_t)l.A * l.A + (int64_t)l.P * l.A + (int64_t)l.P * l.P;
    k_vjp_111<<<grid_of(2 * n1 * 32), 256, 0, stream>>>(D, Lp, hL, Rp, hR, a.cb, Lb, Rb);
    CKA(launched("k_vjp_111"));
  }
  if (with_e0) {
    dim3 grid(16, l.nblocks + 1);
    k_vjp_e0<<<grid, 256, 0, stream>>>(D, Lp, hL, Rp, hR, a.cb, Lb, Rb);
    CKA(launched("k_vjp_e0"));
  }
  if (l.cc_size) {
    k_pandya_vjp<<<grid_of(l.cc_size), 256, 0, stream>>>(D, hL, a.lccb, Lb);
    CKA(launched("k_pandya_vjp"));
    k_pandya_vjp<<<grid_of(l.cc_size), 256, 0, stream>>>(D, hR, a.rccb, Rb);
    CKA(launched("k_pandya_vjp"));
  }
  return IMSRG_OK;
}

imsrg_status Ctx::white_vjp(const double* H, int hH, const double* ETAb, double* Hb) {
  CKA(adjoint_prepare());
  CKA(cuda(cudaMemsetAsync(adj->monob, 0, sizeof(double) * (size_t)L.N * L.N, stream), "memset(monopole cotangents)"));
  k_monopole<<<(L.N * L.N + 255) / 256, 256, 0, stream>>>(D, H, hH, d_mono);
  CKA(launched("k_monopole"));
  if (D.n_ai) {
    k_white_vjp_1b<<<(D.n_ai + 255) / 256, 256, 0, stream>>>(D, H, hH, ETAb, Hb);
    CKA(launched("k_white_vjp_1b"));
  }
  dim3 grid(16, L.nblocks);
  k_white_vjp_2b<<<grid, 256, 0, stream>>>(D, H, hH, d_mono, ETAb, Hb, adj->monob);
  CKA(launched("k_white_vjp_2b"));
  k_monopole_vjp<<<(L.N * L.N + 255) / 256, 256, 0, stream>>>(D, hH, adj->monob, Hb);
  return launched("k_monopole_vjp");
}

imsrg_status Ctx::dot(const double* A, const double* B, double* out) {
  CKA(adjoint_prepare());
  k_dot_partial<<<kDotBlocks, 256, 0, stream>>>(A, B, L.slab, adj->partial);
  CKA(launched("k_dot_partial"));
  k_sum<<<1, 1024, 0, stream>>>(adj->partial, kDotBlocks, d_scalars);
  CKA(launched("k_sum"));
  CKA(read_scalars(1));
  *out = h_scalars[0];
  return IMSRG_OK;
}

// ====================================================================== C ABI
#define ACTX(ptr)                                                                        \
  if (!(ptr)) return IMSRG_ERR_INVALID_ARGUMENT;                                         \
  Ctx* c = reinterpret_cast<Ctx*>(ptr);                                                  \
  if (c->device < 0) return c->fail(IMSRG_ERR_UNSUPPORTED, "host-only context (device < 0)"); \
  {                                                                                      \
    cudaError_t _e = cudaSetDevice(c->device);                                           \
    if (_e != cudaSuccess) return c->cuda(_e, "cudaSetDevice");                          \
  }

namespace {
bool mine(Ctx* c, const imsrg_op* op) { return op && op->owner == c; }
}  // namespace

extern "C" {

imsrg_status imsrg_commutator_vjp(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, const imsrg_op* RESb,
                                  imsrg_op* Lb, imsrg_op* Rb, int32_t flags) {
  ACTX(ctx);
  if (!mine(c, L) || !mine(c, R) || !mine(c, RESb) || !mine(c, Lb) || !mine(c, Rb))
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_commutator_vjp: operator of another context or NULL");
  if (Lb == Rb || Lb == L || Lb == R || Lb == RESb || Rb == L || Rb == R || Rb == RESb)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_commutator_vjp: Lb and Rb must be distinct from the inputs");
  Lb->herm = L->herm;
  Rb->herm = R->herm;
  return c->commutator_vjp(L->d, L->herm, R->d, R->herm, RESb->herm, (flags & IMSRG_COMM_E0) != 0, RESb->d, Lb->d,
                           Rb->d);
}

imsrg_status imsrg_white_vjp(imsrg_ctx* ctx, const imsrg_op* H, const imsrg_op* ETAb, imsrg_op* Hb) {
  ACTX(ctx);
  if (!mine(c, H) || !mine(c, ETAb) || !mine(c, Hb))
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_white_vjp: operator of another context or NULL");
  if (Hb == H || Hb == ETAb) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_white_vjp: Hb must not alias H or ETAb");
  Hb->herm = H->herm;
  return c->white_vjp(H->d, H->herm, ETAb->d, Hb->d);
}

imsrg_status imsrg_dot_sq_op(imsrg_ctx* ctx, const imsrg_op* A, const imsrg_op* B, double* out) {
  ACTX(ctx);
  if (!mine(c, A) || !mine(c, B) || !out)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_dot_sq_op: operator of another context or NULL");
  return c->dot(A->d, B->d, out);
}

}  // extern "C"
