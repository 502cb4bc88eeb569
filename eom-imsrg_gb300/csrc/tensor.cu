// Rank-lambda tensor operators on the device: layout tables, the scalar-tensor commutator
// [L, R] of src/TS_commutators.f90 in the call order of BCH_TENSOR (src/IMSRG_MAGNUS.f90:418-455),
// BCH_TENSOR itself, norms, and their C ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <tuple>

#include "../../include/imsrg_gb300.h"
#include "engine.h"
#include "kernels.h"
#include "tensor.h"
#include "tensor_state.h"

using namespace imsrg;

namespace imsrg {
__global__ void k_ts111(DevLayout D, DevTLayout T, const double* L, int hL, const double* R, int hR, double* RES);
__global__ void k_ts121(DevLayout D, DevTLayout T, const double* L, int hL, const double* R, int hR, double* RES,
                        int hRES);
__global__ void k_ts211(DevLayout D, DevTLayout T, const double* LCC, int hL, const double* R, int hR, double* RES,
                        int hRES);
__global__ void k_ts221(DevLayout D, DevTLayout T, const double* w1, const double* w2, int pm, double* RES, int hRES);
__global__ void k_ts122(DevLayout D, DevTLayout T, const double* L, int hL, const double* R, int hR, double* RES,
                        ElemSegs sg);
__global__ void k_ts212(DevLayout D, DevTLayout T, const double* L, int hL, const double* R, int hR, double* RES,
                        ElemSegs sg);
__global__ void k_ts122f(DevLayout D, DevTLayout T, const double* L, int hL, const double* R, int hR, double* RES,
                         ElemSegs sg);
__global__ void k_ts212f(DevLayout D, DevTLayout T, const double* L, int hL, const double* R, int hR, double* RES,
                         ElemSegs sg);
__global__ void k_ts_pphh_update(int64_t n, int64_t off, double* RES, const double* w1, const double* w2);
__global__ void k_tpandya(DevLayout D, DevTLayout T, const double* R, int hR, int J3, int J4, int qa, int qb, int term,
                          double scale, double* out);
// FP32 SIMT form of k_gemm_fp64 (FP64 operands and results), gemm_tc.cu
__global__ void k_gemm_f32(const GemmProb* probs, const GemmTile* tiles, GemmOperands ops);
__global__ void k_tpandya_exc(DevLayout D, DevTLayout T, const double* R, int hR, const ExcBlock* blk,
                              const int64_t* pre, int nblk, const int* pe, const int* hp, double* ccr, double* ccx);
__global__ void k_ts222ph_scatter_exc(DevLayout D, DevTLayout T, const ExcBlock* blk, const int64_t* pre, int nblk,
                                      const int* pe, const int* hp, const double* Wx, const double* Wy, int hL, int hR,
                                      double* RES);
__global__ void k_ts222ph_scatter(DevLayout D, DevTLayout T, const double* Wx, const double* Wy, int J3, int J4,
                                  int qa, int qb, int hL, int hR, double thresh, int exc, double* RES);
}  // namespace imsrg

namespace {

int grid_n(int64_t n, int threads = 256, int cap = 152 * 16) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, cap));
}

std::map<std::pair<Ctx*, int>, std::unique_ptr<TensorState>>& registry() {
  static std::map<std::pair<Ctx*, int>, std::unique_ptr<TensorState>> r;
  return r;
}

struct Pack {
  std::vector<char> buf;
  std::vector<std::pair<size_t, const void**>> fix;
  template <class V>
  void add(const std::vector<V>& v, const V** dst) {
    const size_t o = (buf.size() + 255) & ~size_t(255);
    buf.resize(o + std::max<size_t>(v.size() * sizeof(V), 1));
    if (!v.empty()) std::memcpy(buf.data() + o, v.data(), v.size() * sizeof(V));
    fix.push_back({o, reinterpret_cast<const void**>(dst)});
  }
};

}  // namespace

#define CKT(expr)                 \
  do {                            \
    imsrg_status _s = (expr);     \
    if (_s != IMSRG_OK) return _s; \
  } while (0)

// layout, device tables and workspaces of a (rank, dpar) pair, built on first use
imsrg_status Ctx::tensor_state(int rank, int dpar, TensorState** out) {
  auto& reg = registry();
  const auto key = std::make_pair(this, rank * 4 + dpar);
  auto it = reg.find(key);
  if (it != reg.end()) {
    *out = it->second.get();
    return IMSRG_OK;
  }
  auto st = std::make_unique<TensorState>();
  TLayout& T = st->T;
  const std::string e = build_tlayout(T, L, rank, dpar);
  if (!e.empty()) return fail(IMSRG_ERR_INVALID_ARGUMENT, e);
  if (device < 0) {  // host-only context: layout queries only
    *out = st.get();
    reg[key] = std::move(st);
    return IMSRG_OK;
  }
  CKT(ensure_workspace());
  const auto pphh = build_tensor_pphh_problems(T, L);
  const auto pphh_tiles = build_tiles(pphh, 64, 64);
  const auto exc = build_tensor_pphh_problems(T, L, true);
  const auto exc_tiles = build_tiles(exc, 64, 64);
  // per cross-coupled channel, its rows (i, j) with i a particle and j a hole, and with i a hole
  // and j a particle: the only columns of CCR and rows of CCX an excitation operator fills
  std::vector<int> pe_off{0}, pe, hp_off{0}, hp;
  for (int q = 0; q < L.ncc; ++q) {
    for (int r = 0; r < L.cc_rlen[q]; ++r) {
      const int i = L.cc_ra[L.cc_row_off[q] + r], j = L.cc_rb[L.cc_row_off[q] + r];
      if (L.con[i] == 0 && L.con[j] == 1) pe.push_back(r);
      if (L.con[i] == 1 && L.con[j] == 0) hp.push_back(r);
    }
    pe_off.push_back((int)pe.size());
    hp_off.push_back((int)hp.size());
  }
  // excitation-mode particle-hole products of all cross-coupled tensor blocks, batched: the
  // packed CCR / CCX of every block, Wx (r1 x npe(qb)) = -LCC(qa) CCR and Wy (nhp(qa) x r2) =
  // CCX LCC(qb)^T as one grouped GEMM, each in its own region of four buffers
  std::vector<ExcBlock> xblk;
  std::vector<int64_t> xpre_p{0}, xpre_s{0};
  std::vector<GemmProb> xbp;
  int64_t o_ccr = 0, o_ccx = 0, o_wx = 0, o_wy = 0;
  for (size_t b = 0; b < T.cb_J3.size(); ++b) {
    const int qa = T.cb_qa[b], qb = T.cb_qb[b];
    const int r1 = L.cc_rlen[qa], r2 = L.cc_rlen[qb], nb1 = L.cc_nph[qa], nb2 = L.cc_nph[qb];
    const int nx = nb1 ? pe_off[qb + 1] - pe_off[qb] : 0;
    const int ny = (nb2 && T.cb_J3[b] != T.cb_J4[b]) ? hp_off[qa + 1] - hp_off[qa] : 0;
    if (!nx && !ny) continue;
    ExcBlock B{T.cb_J3[b], T.cb_J4[b], qa, qb, nx, ny, pe_off[qb], hp_off[qa], o_ccr, o_ccx, o_wx, o_wy};
    if (nx) {
      GemmProb p{};
      p.c_id = kOpW1; p.c_off = o_wx; p.M = r1; p.N = nx; p.ldc = r1; p.nterm = 1;
      GemmTerm& t = p.t[0];
      t.a_id = kOpLCC; t.a_off = L.cc_off[qa]; t.lda = r1; t.ta = 0;
      t.b_id = kOpRCC; t.b_off = o_ccr; t.ldb = nb1; t.tb = 0;
      t.K = nb1; t.alpha = kAlphaNeg | kAlphaOne;
      xbp.push_back(p);
    }
    if (ny) {
      GemmProb p{};
      p.c_id = kOpW2; p.c_off = o_wy; p.M = ny; p.N = r2; p.ldc = ny; p.nterm = 1;
      GemmTerm& t = p.t[0];
      t.a_id = kOpWCC; t.a_off = o_ccx; t.lda = ny; t.ta = 0;
      t.b_id = kOpLCC; t.b_off = L.cc_off[qb]; t.ldb = r2; t.tb = 1;
      t.K = nb2; t.alpha = kAlphaOne;
      xbp.push_back(p);
    }
    o_ccr += (int64_t)nb1 * nx; o_ccx += (int64_t)ny * nb2; o_wx += (int64_t)r1 * nx; o_wy += (int64_t)ny * r2;
    xblk.push_back(B);
    xpre_p.push_back(xpre_p.back() + (int64_t)nb1 * nx + (int64_t)ny * nb2);
    xpre_s.push_back(xpre_s.back() + (int64_t)r1 * nx + (int64_t)ny * r2);
  }
  const auto xbt = build_tiles(xbp, 64, 64);
  st->x_nblk = (int)xblk.size();
  st->x_np = xpre_p.back();
  st->x_ns = xpre_s.back();
  st->x_n_t = (int)xbt.size();
  st->x_sizes[0] = o_ccr; st->x_sizes[1] = o_ccx; st->x_sizes[2] = o_wx; st->x_sizes[3] = o_wy;
  st->pe_off = pe_off;
  st->hp_off = hp_off;
  // the (pp,hh) and (hh,pp) arrays of every block, relative to goff[0]
  std::vector<int64_t> seg_off, seg_pre{0};
  for (int q = 0; q < T.nblocks; ++q)
    for (int g : {2, 6}) {
      const int64_t n = (int64_t)T.n1[(size_t)q * 9 + g] * T.n2[(size_t)q * 9 + g];
      if (!n) continue;
      seg_off.push_back(T.goff[(size_t)q * 9 + g] - T.goff[0]);
      seg_pre.push_back(seg_pre.back() + n);
    }
  // per cross-coupled block: Wx = -LCC(qa) CCR and Wy = CCX LCC(qb)^T
  std::vector<GemmProb> cbp;
  std::vector<GemmTile> cbt;
  for (size_t b = 0; b < T.cb_J3.size(); ++b) {
    const int qa = T.cb_qa[b], qb = T.cb_qb[b];
    const int r1 = L.cc_rlen[qa], r2 = L.cc_rlen[qb], nb1 = L.cc_nph[qa], nb2 = L.cc_nph[qb];
    std::vector<GemmProb> ps;
    if (nb1) {
      GemmProb p{};
      p.c_id = kOpW1; p.M = r1; p.N = r2; p.ldc = r1; p.nterm = 1;
      GemmTerm& t = p.t[0];
      t.a_id = kOpLCC; t.a_off = L.cc_off[qa]; t.lda = r1; t.ta = 0;
      t.b_id = kOpRCC; t.b_off = 0; t.ldb = nb1; t.tb = 0;
      t.K = nb1; t.alpha = kAlphaNeg | kAlphaOne;
      ps.push_back(p);
    }
    if (nb2 && T.cb_J3[b] != T.cb_J4[b]) {
      GemmProb p{};
      p.c_id = kOpW2; p.M = r1; p.N = r2; p.ldc = r1; p.nterm = 1;
      GemmTerm& t = p.t[0];
      t.a_id = kOpWCC; t.a_off = 0; t.lda = r1; t.ta = 0;
      t.b_id = kOpLCC; t.b_off = L.cc_off[qb]; t.ldb = r2; t.tb = 1;
      t.K = nb2; t.alpha = kAlphaOne;
      ps.push_back(p);
    }
    const int base = (int)cbp.size();
    auto tiles = build_tiles(ps, 64, 64);
    st->cb_tile_start.push_back((int)cbt.size());
    st->cb_tile_n.push_back((int)tiles.size());
    for (auto& t : tiles) {
      t.prob += base;
      cbt.push_back(t);
    }
    for (auto& p : ps) cbp.push_back(p);
  }
  Pack pk;
  DevTLayout& d = st->DT;
  d.rank = T.rank; d.dpar = T.dpar; d.nblocks = T.nblocks; d.n_ob = (int)T.ob_kind.size();
  d.six_nJ = T.six_nJ; d.six_nh = T.six_nh; d.six_nhx = T.six_nhx;
  d.off_fhh = T.off_fhh; d.off_fpp = T.off_fpp; d.off_fph = T.off_fph; d.slab = T.slab; d.n2b = T.n2b;
  pk.add(T.J1, &d.J1); pk.add(T.J2, &d.J2); pk.add(T.q1, &d.q1); pk.add(T.q2, &d.q2); pk.add(T.lut, &d.lut);
  pk.add(T.goff, &d.goff); pk.add(T.n1, &d.n1); pk.add(T.n2, &d.n2);
  pk.add(T.ob_kind, &d.ob_kind); pk.add(T.ob_p, &d.ob_p); pk.add(T.ob_q, &d.ob_q); pk.add(T.ob_pk, &d.ob_pk);
  pk.add(T.ob_qk, &d.ob_qk);
  pk.add(T.six, &d.six); pk.add(T.six_m, &d.six_m); pk.add(T.ccnb, &d.ccnb);
  const std::vector<float> six_f(T.six.begin(), T.six.end());
  pk.add(six_f, &d.six_f);
  pk.add(T.tnb_start, &d.tnb_start); pk.add(T.tnb_count, &d.tnb_count); pk.add(T.tnb_list, &d.tnb_list);
  pk.add(pphh, &st->pphh_p); pk.add(pphh_tiles, &st->pphh_t);
  pk.add(exc, &st->exc_p); pk.add(exc_tiles, &st->exc_t);
  pk.add(seg_off, &st->exc_segs.off); pk.add(seg_pre, &st->exc_segs.pre);
  pk.add(pe, &st->d_pe); pk.add(hp, &st->d_hp);
  pk.add(xbp, &st->x_p); pk.add(xbt, &st->x_t);
  pk.add(xblk, &st->x_blk); pk.add(xpre_p, &st->x_pre_p); pk.add(xpre_s, &st->x_pre_s);
  pk.add(cbp, &st->cb_p); pk.add(cbt, &st->cb_t);
  pk.add(T.seg_start, &st->seg_start); pk.add(T.seg_len, &st->seg_len); pk.add(T.seg_w, &st->seg_w);
  CKT(cuda(cudaMalloc(&st->tables, pk.buf.size()), "cudaMalloc(tensor tables)"));
  CKT(cuda(cudaMemcpy(st->tables, pk.buf.data(), pk.buf.size(), cudaMemcpyHostToDevice), "cudaMemcpy(tensor tables)"));
  for (auto& f : pk.fix) *f.second = static_cast<const char*>(st->tables) + f.first;
  st->n_pphh_t = (int)pphh_tiles.size();
  st->n_exc_t = (int)exc_tiles.size();
  st->exc_segs.n = (int)seg_off.size();
  st->exc_n2 = seg_pre.back();
  st->nseg = (int)T.seg_start.size();
  const size_t tb = sizeof(double) * (size_t)T.slab;
  for (double** p : {&st->w1, &st->w2, &st->bch_a, &st->bch_b}) {
    CKT(cuda(cudaMalloc(p, tb), "cudaMalloc(tensor workspace)"));
    CKT(cuda(cudaMemsetAsync(*p, 0, tb, stream), "memset(tensor workspace)"));
  }
  const size_t xb = sizeof(double) * (size_t)std::max<int64_t>(T.cb_max_x, 1);
  const size_t wb = sizeof(double) * (size_t)std::max<int64_t>(T.cb_max_w, 1);
  CKT(cuda(cudaMalloc(&st->ccx, xb), "cudaMalloc(CCX tensor)"));
  CKT(cuda(cudaMalloc(&st->ccr, xb), "cudaMalloc(CCR tensor)"));
  CKT(cuda(cudaMalloc(&st->wx, wb), "cudaMalloc(Wx)"));
  CKT(cuda(cudaMalloc(&st->wy, wb), "cudaMalloc(Wy)"));
  *out = st.get();
  reg[key] = std::move(st);
  return IMSRG_OK;
}

void Ctx::tensor_release() {
  auto& reg = registry();
  for (auto it = reg.begin(); it != reg.end();) {
    if (it->first.first != this) {
      ++it;
      continue;
    }
    TensorState* s = it->second.get();
    for (void* p : {(void*)s->w1, (void*)s->w2, (void*)s->ccx, (void*)s->ccr, (void*)s->wx, (void*)s->wy,
                    (void*)s->bch_a, (void*)s->bch_b, s->tables, (void*)s->tc_buf, s->tc_tables, (void*)s->w3,
                    (void*)s->x_buf[0], (void*)s->x_buf[1], (void*)s->x_buf[2], (void*)s->x_buf[3]})
      if (p) cudaFree(p);
    it = reg.erase(it);
  }
}

// [L (scalar, hL), R (tensor, hR)] -> RES (tensor, herm -hL hR); pieces as imsrg_tensor_commutator
// Split-BF16 plan of the tensor ladder for the context's slice count: every product through
// pp pairs of the FP64 problem list becomes a single-term tensor-core problem over K-major
// operand tiles (columns of a stored array, or its rows through the transposed split); the
// products through hh pairs keep their FP64 problems.
imsrg_status Ctx::tensor_tc_prepare(TensorState& S) {
  if (!tc_slices()) return fail(IMSRG_ERR_UNSUPPORTED, "tensor-core ladder needs a mixed-precision context");
  if (S.tc_S == tc_slices() && S.tc_kind == tc_kind()) return IMSRG_OK;
  for (void* p : {(void*)S.tc_buf, S.tc_tables, (void*)S.w3})
    if (p) cudaFree(p);
  S.tc_buf = nullptr; S.tc_tables = nullptr; S.w3 = nullptr; S.tc_S = 0;
  const int BMr = kTcTileRows, BKk = tc_tile_k();
  const auto P = build_tensor_pphh_problems(S.T, L);
  std::vector<TcSplitOp> ops;
  std::map<std::tuple<int, int64_t, int, int, int, int>, int> seen;  // operand -> tile base
  int tiles = 0;
  auto split = [&](int src, int64_t off, int rows, int K, int trans, int ld) {
    const auto key = std::make_tuple(src, off, rows, K, trans, ld);
    auto it = seen.find(key);
    if (it != seen.end()) return it->second;
    TcSplitOp o{};
    o.src = src; o.src_off = off; o.rows = rows; o.K = K; o.nkb = (K + BKk - 1) / BKk;
    o.tile_base = tiles; o.trans = trans; o.ld = ld;
    tiles += ((rows + BMr - 1) / BMr) * o.nkb;
    ops.push_back(o);
    seen[key] = o.tile_base;
    return o.tile_base;
  };
  std::vector<TcProb> probs;
  std::vector<GemmProb> hh;
  for (const GemmProb& p : P) {
    if (p.c_id == kOpW2) { hh.push_back(p); continue; }
    for (int ti = 0; ti < p.nterm; ++ti) {
      const GemmTerm& t = p.t[ti];
      if ((t.ta == 1 && t.lda != t.K) || (t.tb == 0 && t.ldb != t.K))
        return fail(IMSRG_ERR_MISMATCH, "tensor ladder operand with padded leading dimension");
      const int sa = t.a_id == kOpL ? 0 : 1, sb = t.b_id == kOpL ? 0 : 1;
      const int a_tile = t.ta == 1 ? split(sa, t.a_off, p.M, t.K, 0, 0) : split(sa, t.a_off, p.M, t.K, 1, t.lda);
      const int b_tile = t.tb == 0 ? split(sb, t.b_off, p.N, t.K, 0, 0) : split(sb, t.b_off, p.N, t.K, 1, t.ldb);
      TcProb q{};
      q.M = p.M; q.N = p.N; q.nkb = (t.K + BKk - 1) / BKk; q.nterm = 1;
      q.t[0] = TcTermDesc{a_tile, b_tile, t.alpha};  // the alpha bits are the TcSign bits
      q.out_f32 = 0; q.c_id = ti == 0 ? kOpW1 : kTensorOpW3; q.c_off = p.c_off; q.ldc = p.ldc;
      probs.push_back(q);
    }
  }
  std::vector<TcTile> tl;
  for (int i = 0; i < (int)probs.size(); ++i)
    for (int m0 = 0; m0 < probs[i].M; m0 += BMr)
      for (int n0 = 0; n0 < probs[i].N; n0 += BMr) tl.push_back(TcTile{i, m0, n0, BMr});
  std::stable_sort(tl.begin(), tl.end(), [&](const TcTile& a, const TcTile& b) { return probs[a.prob].nkb > probs[b.prob].nkb; });
  std::vector<SplitChunk> chunks;
  auto add_chunks = [&](int op) {
    const int rows_per = std::max(1, 4096 / std::max(ops[op].K, 1));
    for (int r0 = 0; r0 < ops[op].rows; r0 += rows_per)
      chunks.push_back(SplitChunk{op, r0, std::min(ops[op].rows, r0 + rows_per)});
  };
  for (int op = 0; op < (int)ops.size(); ++op) add_chunks(op);
  const int ladder_nchunks = (int)chunks.size();
  // ---- particle-hole: LCC rows of every channel (src 0 = d_lcc), split once per commutator
  std::vector<int> lcc_tile(L.ncc, -1);
  const size_t lcc_op0 = ops.size();
  for (int q = 0; q < L.ncc; ++q) {
    const int r = L.cc_rlen[q], nb = L.cc_nph[q];
    if (r == 0 || nb == 0) continue;
    lcc_tile[q] = split(0, L.cc_off[q], r, nb, 1, r);
  }
  for (size_t op = lcc_op0; op < ops.size(); ++op) add_chunks((int)op);
  S.ph_lcc_nchunks = (int)chunks.size() - ladder_nchunks;
  // per block: CCR (src 0, its columns, K = nb1) and CCX (src 1, its rows, K = nb2) into two
  // regions shared by all blocks, then Wx = -LCC(qa) CCR and Wy = CCX LCC(qb)^T
  const TLayout& TT = S.T;
  int ccr_tiles_max = 0, ccx_tiles_max = 0;
  for (size_t b = 0; b < TT.cb_J3.size(); ++b) {
    const int qa = TT.cb_qa[b], qb = TT.cb_qb[b];
    const int r1 = L.cc_rlen[qa], r2 = L.cc_rlen[qb], nb1 = L.cc_nph[qa], nb2 = L.cc_nph[qb];
    ccr_tiles_max = std::max(ccr_tiles_max, ((r2 + BMr - 1) / BMr) * ((nb1 + BKk - 1) / BKk));
    ccx_tiles_max = std::max(ccx_tiles_max, ((r1 + BMr - 1) / BMr) * ((nb2 + BKk - 1) / BKk));
  }
  const int ccr_base = tiles, ccx_base = tiles + ccr_tiles_max;
  tiles += ccr_tiles_max + ccx_tiles_max;
  std::vector<TcTile> tph;
  S.ph_chunk_start.clear(); S.ph_chunk_n.clear(); S.ph_tile_start.clear(); S.ph_tile_n.clear();
  for (size_t b = 0; b < TT.cb_J3.size(); ++b) {
    const int qa = TT.cb_qa[b], qb = TT.cb_qb[b];
    const int r1 = L.cc_rlen[qa], r2 = L.cc_rlen[qb], nb1 = L.cc_nph[qa], nb2 = L.cc_nph[qb];
    const bool dox = nb1 > 0, doy = nb2 > 0 && TT.cb_J3[b] != TT.cb_J4[b];
    S.ph_chunk_start.push_back((int)chunks.size());
    S.ph_tile_start.push_back((int)(tl.size() + tph.size()));
    auto add_prob = [&](int K, TcTermDesc t, int c_id) {
      TcProb q{};
      q.M = r1; q.N = r2; q.nkb = (K + BKk - 1) / BKk; q.nterm = 1; q.t[0] = t;
      q.out_f32 = 0; q.c_id = c_id; q.c_off = 0; q.ldc = r1;
      probs.push_back(q);
      const int pi = (int)probs.size() - 1;
      for (int m0 = 0; m0 < r1; m0 += BMr)
        for (int n0 = 0; n0 < r2; n0 += BMr) tph.push_back(TcTile{pi, m0, n0, BMr});
    };
    if (dox && r1 && r2) {
      TcSplitOp o{};
      o.src = 0; o.src_off = 0; o.rows = r2; o.K = nb1; o.nkb = (nb1 + BKk - 1) / BKk; o.tile_base = ccr_base;
      ops.push_back(o);
      add_chunks((int)ops.size() - 1);
      add_prob(nb1, TcTermDesc{lcc_tile[qa], ccr_base, kSignNeg}, kOpW1);
    }
    if (doy && r1 && r2) {
      TcSplitOp o{};
      o.src = 1; o.src_off = 0; o.rows = r1; o.K = nb2; o.nkb = (nb2 + BKk - 1) / BKk; o.tile_base = ccx_base;
      o.trans = 1; o.ld = r1;
      ops.push_back(o);
      add_chunks((int)ops.size() - 1);
      add_prob(nb2, TcTermDesc{ccx_base, lcc_tile[qb], 0}, kOpW2);
    }
    S.ph_chunk_n.push_back((int)chunks.size() - S.ph_chunk_start.back());
    S.ph_tile_n.push_back((int)(tl.size() + tph.size()) - S.ph_tile_start.back());
  }
  tl.insert(tl.end(), tph.begin(), tph.end());
  S.tc_ntiles = 0;  // set below: the ladder's tiles come first
  const int ladder_ntiles = (int)(tl.size() - tph.size());
  const auto hh_tiles = build_tiles(hh, 64, 64);
  const int Sl = tc_slices();
  S.tc_slice_rows = (int64_t)tiles * BMr;
  S.tc_slice_elems = S.tc_slice_rows * BKk;
  if ((int64_t)Sl * S.tc_slice_rows >= (int64_t)1 << 31)
    return fail(IMSRG_ERR_UNSUPPORTED, "tensor ladder operands too large for 32-bit TMA rows");
  const size_t bytes = (size_t)tc_elem_bytes() * (size_t)Sl * (size_t)S.tc_slice_elems;
  CKT(cuda(cudaMalloc(&S.tc_buf, std::max<size_t>(bytes, 256)), "cudaMalloc(tensor ladder operands)"));
  CKT(cuda(cudaMemset(S.tc_buf, 0, std::max<size_t>(bytes, 256)), "memset(tensor ladder operands)"));
  CKT(tc_encode_map(&S.tc_map, S.tc_buf, (int64_t)Sl * S.tc_slice_rows));
  Pack pk;
  pk.add(ops, &S.tc_ops); pk.add(chunks, &S.tc_chunks); pk.add(probs, &S.tc_probs); pk.add(tl, &S.tc_tiles);
  pk.add(hh, &S.hh_p); pk.add(hh_tiles, &S.hh_t);
  CKT(cuda(cudaMalloc(&S.tc_tables, pk.buf.size()), "cudaMalloc(tensor ladder tables)"));
  CKT(cuda(cudaMemcpy(S.tc_tables, pk.buf.data(), pk.buf.size(), cudaMemcpyHostToDevice), "cudaMemcpy(tensor ladder)"));
  for (auto& f : pk.fix) *f.second = static_cast<const char*>(S.tc_tables) + f.first;
  S.tc_nchunks = ladder_nchunks;
  S.tc_ntiles = ladder_ntiles;
  S.n_hh_t = (int)hh_tiles.size();
  CKT(cuda(cudaMalloc(&S.w3, sizeof(double) * (size_t)S.T.slab), "cudaMalloc(tensor w3)"));
  S.tc_S = Sl;
  S.tc_kind = tc_kind();
  return IMSRG_OK;
}

imsrg_status Ctx::tensor_commutator(TensorState& S, const double* Lp, int hL, const double* R, int hR, double* RES,
                                    int pieces) {
  CKT(ensure_workspace());
  const DevTLayout& T = S.DT;
  const int hRES = -hL * hR;
  const double thresh = (pieces & (kTensorExactPh | kTensorExcitation)) ? 0.0 : 1e-6;
  // excitation mode: R has only fph and (pp,hh) / (hh,pp) elements and only the fph and
  // (pp,hh) / (hh,pp) elements of RES are wanted (the EOM product)
  const int exc = (pieces & kTensorExcitation) ? 1 : 0;
  const ElemSegs segs = exc ? S.exc_segs : ElemSegs{};
  const int64_t n2out = exc ? S.exc_n2 : (int64_t)T.n2b;
  if (L.cc_size) CKT(pandya(Lp, hL, d_lcc));
  const int nob = T.n_ob;
  if (pieces & 1) {
    const int64_t n1 = (int64_t)L.A * L.A + (int64_t)L.P * L.A + (int64_t)L.P * L.P;
    k_ts111<<<grid_n(n1 * 32), 256, 0, stream>>>(D, T, Lp, hL, R, hR, RES);
    CKT(launched("k_ts111"));
  }
  if ((pieces & 2) && nob) {
    k_ts121<<<(nob * 32 + 255) / 256, 256, 0, stream>>>(D, T, Lp, hL, R, hR, RES, hRES);
    CKT(launched("k_ts121"));
  }
  if ((pieces & 4) && nob) {
    k_ts211<<<(nob * 32 + 255) / 256, 256, 0, stream>>>(D, T, d_lcc, hL, R, hR, RES, hRES);
    CKT(launched("k_ts211"));
  }
  if ((pieces & 8) && n2out) {
    if (precision != IMSRG_PREC_FP64)
      k_ts122f<<<grid_n(n2out), 256, 0, stream>>>(D, T, Lp, hL, R, hR, RES, segs);
    else
      k_ts122<<<grid_n(n2out), 256, 0, stream>>>(D, T, Lp, hL, R, hR, RES, segs);
    CKT(launched("k_ts122"));
  }
  if ((pieces & 16) && n2out) {
    if (precision != IMSRG_PREC_FP64)
      k_ts212f<<<grid_n(n2out), 256, 0, stream>>>(D, T, Lp, hL, R, hR, RES, segs);
    else
      k_ts212<<<grid_n(n2out), 256, 0, stream>>>(D, T, Lp, hL, R, hR, RES, segs);
    CKT(launched("k_ts212"));
  }
  if ((pieces & 32) && precision != IMSRG_PREC_FP64 && !exc) {  // split-BF16 products through pp pairs
    CKT(tensor_tc_prepare(S));
    const size_t tb = sizeof(double) * (size_t)T.slab;
    CKT(cuda(cudaMemsetAsync(S.w1, 0, tb, stream), "memset(tensor w1)"));
    CKT(cuda(cudaMemsetAsync(S.w2, 0, tb, stream), "memset(tensor w2)"));
    CKT(cuda(cudaMemsetAsync(S.w3, 0, tb, stream), "memset(tensor w3)"));
    CKT(tc_split_on(S.tc_ops, S.tc_chunks, S.tc_nchunks, Lp, R, S.tc_buf, S.tc_slice_elems));
    TcOut out{};
    out.f64[kOpW1] = S.w1;
    out.f64[kTensorOpW3] = S.w3;
    CKT(tc_gemm_on(S.tc_map, S.tc_slice_rows, S.tc_probs, S.tc_tiles, S.tc_ntiles, out, hL, hR));
    if (S.n_hh_t) {
      GemmOperands ops{};
      ops.in[kOpL] = Lp; ops.in[kOpR] = R;
      ops.out[kOpW1] = S.w1; ops.out[kOpW2] = S.w2;
      ops.hL = hL; ops.hR = hR;
      k_gemm_fp64<<<S.n_hh_t, 256, 0, stream>>>(S.hh_p, S.hh_t, ops);
      CKT(launched("k_gemm_fp64(tensor hh ladder)"));
    }
    k_axpby<<<grid_n(T.slab), 256, 0, stream>>>(T.slab, S.w1, 1.0, S.w3, 1.0, S.w1);
    CKT(launched("k_axpby"));
    if (T.n2b) {
      k_ts_pphh_update<<<grid_n(T.n2b), 256, 0, stream>>>(T.n2b, S.T.goff.empty() ? 0 : S.T.goff[0], RES, S.w1, S.w2);
      CKT(launched("k_ts_pphh_update"));
    }
    if (nob) {
      k_ts221<<<(nob * 32 + 255) / 256, 256, 0, stream>>>(D, T, S.w1, S.w2, hL * hR, RES, hRES);
      CKT(launched("k_ts221"));
    }
  } else if (pieces & 32) {
    const size_t tb = sizeof(double) * (size_t)T.slab;
    CKT(cuda(cudaMemsetAsync(S.w1, 0, tb, stream), "memset(tensor w1)"));
    CKT(cuda(cudaMemsetAsync(S.w2, 0, tb, stream), "memset(tensor w2)"));
    const int nt = exc ? S.n_exc_t : S.n_pphh_t;
    if (nt) {
      GemmOperands ops{};
      ops.in[kOpL] = Lp; ops.in[kOpR] = R;
      ops.out[kOpW1] = S.w1; ops.out[kOpW2] = S.w2;
      ops.hL = hL; ops.hR = hR;
      if (exc && precision != IMSRG_PREC_FP64) {  // mixed modes: the excitation ladder in FP32
        k_gemm_f32<<<nt, 256, 0, stream>>>(S.exc_p, S.exc_t, ops);
        CKT(launched("k_gemm_f32(tensor pphh, excitation)"));
      } else {
        k_gemm_fp64<<<nt, 256, 0, stream>>>(exc ? S.exc_p : S.pphh_p, exc ? S.exc_t : S.pphh_t, ops);
        CKT(launched("k_gemm_fp64(tensor pphh)"));
      }
    }
    if (T.n2b) {
      k_ts_pphh_update<<<grid_n(T.n2b), 256, 0, stream>>>(T.n2b, S.T.goff.empty() ? 0 : S.T.goff[0], RES, S.w1, S.w2);
      CKT(launched("k_ts_pphh_update"));
    }
    if (nob) {
      k_ts221<<<(nob * 32 + 255) / 256, 256, 0, stream>>>(D, T, S.w1, S.w2, hL * hR, RES, hRES);
      CKT(launched("k_ts221"));
    }
  }
  if ((pieces & 64) && exc) {  // excitation mode: packed CCR / CCX of all blocks (FP32 products in mixed modes)
    if (S.x_nblk) {
      if (!S.x_buf[0])
        for (int k = 0; k < 4; ++k)
          CKT(cuda(cudaMalloc(&S.x_buf[k], sizeof(double) * (size_t)std::max<int64_t>(S.x_sizes[k], 1)),
                   "cudaMalloc(excitation ph buffers)"));
      k_tpandya_exc<<<grid_n(S.x_np), 256, 0, stream>>>(D, T, R, hR, S.x_blk, S.x_pre_p, S.x_nblk, S.d_pe, S.d_hp,
                                                         S.x_buf[0], S.x_buf[1]);
      CKT(launched("k_tpandya_exc"));
      if (S.x_n_t) {
        GemmOperands ops{};
        ops.in[kOpLCC] = d_lcc; ops.in[kOpRCC] = S.x_buf[0]; ops.in[kOpWCC] = S.x_buf[1];
        ops.out[kOpW1] = S.x_buf[2]; ops.out[kOpW2] = S.x_buf[3];
        ops.hL = hL; ops.hR = hR;
        if (precision != IMSRG_PREC_FP64) {  // mixed modes: FP32 products
          k_gemm_f32<<<S.x_n_t, 256, 0, stream>>>(S.x_p, S.x_t, ops);
          CKT(launched("k_gemm_f32(tensor ph, excitation)"));
        } else {
          k_gemm_fp64<<<S.x_n_t, 256, 0, stream>>>(S.x_p, S.x_t, ops);
          CKT(launched("k_gemm_fp64(tensor ph, excitation)"));
        }
      }
      k_ts222ph_scatter_exc<<<grid_n(S.x_ns), 256, 0, stream>>>(D, T, S.x_blk, S.x_pre_s, S.x_nblk, S.d_pe, S.d_hp,
                                                                 S.x_buf[2], S.x_buf[3], hL, hR, RES);
      CKT(launched("k_ts222ph_scatter_exc"));
    }
  } else if ((pieces & 64) && precision != IMSRG_PREC_FP64) {  // split-BF16 cross-coupled products
    CKT(tensor_tc_prepare(S));
    const TLayout& H = S.T;
    CKT(tc_split_on(S.tc_ops, S.tc_chunks + S.tc_nchunks, S.ph_lcc_nchunks, d_lcc, nullptr, S.tc_buf,
                    S.tc_slice_elems));
    for (size_t b = 0; b < H.cb_J3.size(); ++b) {
      const int J3 = H.cb_J3[b], J4 = H.cb_J4[b], qa = H.cb_qa[b], qb = H.cb_qb[b];
      const int r1 = L.cc_rlen[qa], r2 = L.cc_rlen[qb], nb1 = L.cc_nph[qa], nb2 = L.cc_nph[qb];
      const bool dox = nb1 > 0, doy = nb2 > 0 && J3 != J4;
      if (!dox && !doy) continue;
      if (dox) {
        k_tpandya<<<grid_n((int64_t)nb1 * r2), 256, 0, stream>>>(D, T, R, hR, J3, J4, qa, qb, 2,
                                                                 1.0 / std::sqrt(J3 + 1.0), S.ccr);
        CKT(launched("k_tpandya"));
      } else {
        CKT(cuda(cudaMemsetAsync(S.wx, 0, sizeof(double) * (size_t)r1 * r2, stream), "memset(Wx)"));
      }
      if (doy) {
        k_tpandya<<<grid_n((int64_t)r1 * nb2), 256, 0, stream>>>(D, T, R, hR, J3, J4, qa, qb, 1,
                                                                 1.0 / std::sqrt(J4 + 1.0), S.ccx);
        CKT(launched("k_tpandya"));
      }
      CKT(tc_split_on(S.tc_ops, S.tc_chunks + S.ph_chunk_start[b], S.ph_chunk_n[b], S.ccr, S.ccx, S.tc_buf,
                      S.tc_slice_elems));
      TcOut out{};
      out.f64[kOpW1] = S.wx;
      out.f64[kOpW2] = S.wy;
      CKT(tc_gemm_on(S.tc_map, S.tc_slice_rows, S.tc_probs, S.tc_tiles + S.ph_tile_start[b], S.ph_tile_n[b], out, hL,
                     hR));
      k_ts222ph_scatter<<<grid_n((int64_t)r1 * r2), 256, 0, stream>>>(D, T, S.wx, doy ? S.wy : nullptr, J3, J4, qa,
                                                                      qb, hL, hR, thresh, exc, RES);
      CKT(launched("k_ts222ph_scatter"));
    }
  } else if (pieces & 64) {
    const TLayout& H = S.T;
    for (size_t b = 0; b < H.cb_J3.size(); ++b) {
      const int J3 = H.cb_J3[b], J4 = H.cb_J4[b], qa = H.cb_qa[b], qb = H.cb_qb[b];
      const int r1 = L.cc_rlen[qa], r2 = L.cc_rlen[qb], nb1 = L.cc_nph[qa], nb2 = L.cc_nph[qb];
      const bool dox = nb1 > 0, doy = nb2 > 0 && J3 != J4;
      if (!dox && !doy) continue;
      if (dox) {
        k_tpandya<<<grid_n((int64_t)nb1 * r2), 256, 0, stream>>>(D, T, R, hR, J3, J4, qa, qb, 2,
                                                                 1.0 / std::sqrt(J3 + 1.0), S.ccr);
        CKT(launched("k_tpandya"));
      } else {
        CKT(cuda(cudaMemsetAsync(S.wx, 0, sizeof(double) * (size_t)r1 * r2, stream), "memset(Wx)"));
      }
      if (doy) {
        k_tpandya<<<grid_n((int64_t)r1 * nb2), 256, 0, stream>>>(D, T, R, hR, J3, J4, qa, qb, 1,
                                                                 1.0 / std::sqrt(J4 + 1.0), S.ccx);
        CKT(launched("k_tpandya"));
      }
      if (S.cb_tile_n[b]) {
        GemmOperands ops{};
        ops.in[kOpLCC] = d_lcc; ops.in[kOpRCC] = S.ccr; ops.in[kOpWCC] = S.ccx;
        ops.out[kOpW1] = S.wx; ops.out[kOpW2] = S.wy;
        ops.hL = hL; ops.hR = hR;
        k_gemm_fp64<<<S.cb_tile_n[b], 256, 0, stream>>>(S.cb_p, S.cb_t + S.cb_tile_start[b], ops);
        CKT(launched("k_gemm_fp64(tensor ph)"));
      }
      k_ts222ph_scatter<<<grid_n((int64_t)r1 * r2), 256, 0, stream>>>(D, T, S.wx, doy ? S.wy : nullptr, J3, J4, qa,
                                                                      qb, hL, hR, thresh, exc, RES);
      CKT(launched("k_ts222ph_scatter"));
    }
  }
  return IMSRG_OK;
}

imsrg_status Ctx::tensor_frob(TensorState& S, const double* op, double scale, int slot) {
  if (S.nseg == 0) return cuda(cudaMemsetAsync(d_scalars + slot, 0, sizeof(double), stream), "memset(norm)");
  if ((int64_t)S.nseg > partial_capacity) {  // one partial per segment: grow the buffer
    double* p = nullptr;
    CKT(cuda(cudaMalloc(&p, sizeof(double) * (size_t)S.nseg), "cudaMalloc(partials)"));
    CKT(cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize"));
    cudaFree(d_partial);
    d_partial = p;
    partial_capacity = S.nseg;
  }
  k_frob_partial<<<S.nseg, 256, 0, stream>>>(op, S.seg_start, S.seg_len, S.seg_w, d_partial);
  CKT(launched("k_frob_partial"));
  k_sum_sqrt<<<1, 1024, 0, stream>>>(d_partial, S.nseg, scale, d_scalars + slot);
  return launched("k_sum_sqrt");
}

// BCH_TENSOR (src/IMSRG_MAGNUS.f90:389-464): HS <- e^G HS e^-G, HS a hermitian tensor, G an
// anti-hermitian scalar; stops when coef * ||ad^n(HS)|| < conv (the reference uses 1e-6, up to 30 terms)
imsrg_status Ctx::bch_tensor(TensorState& S, const double* G, int hG, double* HS, int max_terms, double conv,
                             int* terms) {
  const size_t tb = sizeof(double) * (size_t)S.T.slab;
  double coef = 1.0;
  int iw;
  for (iw = 2; iw <= max_terms; ++iw) {
    coef = coef / (iw - 1.0);
    const double* ad = (iw == 2) ? HS : ((iw & 1) ? S.bch_a : S.bch_b);
    double* out = (iw & 1) ? S.bch_b : S.bch_a;
    CKT(cuda(cudaMemsetAsync(out, 0, tb, stream), "memset(BCH term)"));
    CKT(tensor_commutator(S, G, hG, ad, 1, out, 127));
    k_axpby<<<grid_n(S.T.slab), 256, 0, stream>>>(S.T.slab, HS, 1.0, out, coef, HS);
    CKT(launched("k_axpby"));
    CKT(tensor_frob(S, out, coef, 0));
    CKT(read_scalars(1));
    if (h_scalars[0] < conv) break;
  }
  *terms = (iw > max_terms) ? max_terms - 1 : iw - 1;
  if (iw > max_terms) return fail(IMSRG_ERR_NOT_CONVERGED, "tensor BCH series did not converge within max_terms");
  return IMSRG_OK;
}

// ====================================================================== C ABI
#define TCTX(ptr)                                                                        \
  if (!(ptr)) return IMSRG_ERR_INVALID_ARGUMENT;                                         \
  Ctx* c = reinterpret_cast<Ctx*>(ptr);                                                  \
  if (c->device < 0) return c->fail(IMSRG_ERR_UNSUPPORTED, "host-only context (device < 0)"); \
  {                                                                                      \
    cudaError_t _e = cudaSetDevice(c->device);                                           \
    if (_e != cudaSuccess) return c->cuda(_e, "cudaSetDevice");                          \
  }

extern "C" {

imsrg_status imsrg_tensor_sizes(imsrg_ctx* ctx, int32_t rank2, int32_t dpar2, int64_t* slab, int32_t* nblocks) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  TensorState* s = nullptr;
  CKT(c->tensor_state(rank2, dpar2, &s));
  if (slab) *slab = s->T.slab;
  if (nblocks) *nblocks = s->T.nblocks;
  return IMSRG_OK;
}

imsrg_status imsrg_tensor_block_info(imsrg_ctx* ctx, int32_t rank2, int32_t dpar2, int32_t* J1, int32_t* J2,
                                     int32_t* Tz, int32_t* P1) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  TensorState* s = nullptr;
  CKT(c->tensor_state(rank2, dpar2, &s));
  for (int q = 0; q < s->T.nblocks; ++q) {
    if (J1) J1[q] = s->T.J1[q];
    if (J2) J2[q] = s->T.J2[q];
    if (Tz) Tz[q] = s->T.T[q];
    if (P1) P1[q] = s->T.P1[q];
  }
  return IMSRG_OK;
}

imsrg_status imsrg_tensor_create(imsrg_ctx* ctx, int32_t rank2, int32_t dpar2, int32_t herm, imsrg_tensor** out) {
  TCTX(ctx);
  if (!out || (herm != 1 && herm != -1)) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "herm must be +1 or -1");
  *out = nullptr;
  TensorState* s = nullptr;
  CKT(c->tensor_state(rank2, dpar2, &s));
  imsrg_tensor* t = new (std::nothrow) imsrg_tensor();
  if (!t) return IMSRG_ERR_OUT_OF_MEMORY;
  const size_t tb = sizeof(double) * (size_t)s->T.slab;
  imsrg_status st = c->cuda(cudaMalloc(&t->d, tb), "cudaMalloc(tensor operator)");
  if (st == IMSRG_OK) st = c->cuda(cudaMemsetAsync(t->d, 0, tb, c->stream), "memset(tensor operator)");
  if (st != IMSRG_OK) {
    if (t->d) cudaFree(t->d);
    delete t;
    return st;
  }
  t->herm = herm;
  t->ts = s;
  t->owner = c;
  *out = t;
  return IMSRG_OK;
}

imsrg_status imsrg_tensor_destroy(imsrg_ctx* ctx, imsrg_tensor* t) {
  TCTX(ctx);
  if (!t) return IMSRG_OK;
  if (t->owner != c) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "tensor of another context");
  cudaStreamSynchronize(c->stream);
  cudaFree(t->d);
  delete t;
  return IMSRG_OK;
}

imsrg_status imsrg_tensor_upload_slab(imsrg_ctx* ctx, imsrg_tensor* t, const double* host) {
  TCTX(ctx);
  if (!t || t->owner != c || !host) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_tensor_upload_slab");
  CKT(c->cuda(cudaMemcpyAsync(t->d, host, sizeof(double) * (size_t)t->ts->T.slab, cudaMemcpyHostToDevice, c->stream),
              "H2D tensor"));
  return c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
}

imsrg_status imsrg_tensor_download_slab(imsrg_ctx* ctx, const imsrg_tensor* t, double* host) {
  TCTX(ctx);
  if (!t || t->owner != c || !host) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_tensor_download_slab");
  CKT(c->cuda(cudaMemcpyAsync(host, t->d, sizeof(double) * (size_t)t->ts->T.slab, cudaMemcpyDeviceToHost, c->stream),
              "D2H tensor"));
  return c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
}

imsrg_status imsrg_tensor_commutator(imsrg_ctx* ctx, const imsrg_op* Lop, const imsrg_tensor* R, imsrg_tensor* RES,
                                     int32_t pieces) {
  TCTX(ctx);
  if (!Lop || Lop->owner != c || !R || R->owner != c || !RES || RES->owner != c)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_tensor_commutator: operand of another context or NULL");
  if (R->ts != RES->ts) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "R and RES must have the same rank and parity");
  if (R == RES) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "RES must not alias R");
  RES->herm = -Lop->herm * R->herm;
  return c->tensor_commutator(*R->ts, Lop->d, Lop->herm, R->d, R->herm, RES->d, pieces);
}

imsrg_status imsrg_bch_tensor(imsrg_ctx* ctx, const imsrg_op* G, imsrg_tensor* HS, int32_t max_terms, double conv,
                              int32_t* terms_used) {
  TCTX(ctx);
  if (!G || G->owner != c || !HS || HS->owner != c)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_bch_tensor: operand of another context or NULL");
  if (max_terms < 2) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "max_terms must be >= 2");
  int t = 0;
  imsrg_status s = c->bch_tensor(*HS->ts, G->d, G->herm, HS->d, max_terms, conv, &t);
  if (terms_used) *terms_used = t;
  return s;
}

imsrg_status imsrg_tensor_frob_norm(imsrg_ctx* ctx, const imsrg_tensor* t, double* out) {
  TCTX(ctx);
  if (!t || t->owner != c || !out) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_tensor_frob_norm");
  CKT(c->tensor_frob(*t->ts, t->d, 1.0, 0));
  CKT(c->read_scalars(1));
  *out = c->h_scalars[0];
  return IMSRG_OK;
}

}  // extern "C"
