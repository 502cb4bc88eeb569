// C-ABI implementation: contexts, device operators, orchestration of the commutator
// pieces, the White generator and the Magnus / BCH drivers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "engine.h"
#include "kernels.h"
#include "layout.h"

using namespace imsrg;

namespace {

constexpr int kThreads = 256;

int grid_for(int64_t n, int max_blocks = 152 * 16) {
  int64_t b = (n + kThreads - 1) / kThreads;
  if (b < 1) b = 1;
  return (int)std::min<int64_t>(b, max_blocks);
}

}  // namespace

// ---------------------------------------------------------------- error helpers
imsrg_status Ctx::fail(imsrg_status code, const std::string& msg) {
  err = msg;
  return code;
}
imsrg_status Ctx::cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return IMSRG_OK;
  err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? IMSRG_ERR_OUT_OF_MEMORY : IMSRG_ERR_CUDA;
}
imsrg_status Ctx::launched(const char* what) {
  ++launches;
  return cuda(cudaGetLastError(), what);
}

// Records the end of a phase on the stream when per-phase timing is enabled.
void Ctx::mark(int phase) {
  if (!prof) return;
  cudaEvent_t e;
  if (!prof_pool.empty()) {
    e = prof_pool.back();
    prof_pool.pop_back();
  } else if (cudaEventCreate(&e) != cudaSuccess) {
    return;
  }
  cudaEventRecord(e, stream);
  prof_marks.push_back({phase, e});
}

#define CK(expr)                                 \
  do {                                           \
    imsrg_status _s = (expr);                    \
    if (_s != IMSRG_OK) return _s;               \
  } while (0)

// ---------------------------------------------------------------- device tables
namespace {

struct Packer {
  std::vector<char> buf;
  std::vector<std::pair<size_t, const void**>> fix;
  template <class T>
  void add(const std::vector<T>& v, const T** dst) {
    size_t o = (buf.size() + 255) & ~size_t(255);
    buf.resize(o + std::max<size_t>(v.size() * sizeof(T), 1));
    if (!v.empty()) std::memcpy(buf.data() + o, v.data(), v.size() * sizeof(T));
    fix.push_back({o, reinterpret_cast<const void**>(dst)});
  }
};

}  // namespace

imsrg_status Ctx::upload_tables() {
  Packer pk;
  DevLayout& d = D;
  const Layout& l = L;
  d.N = l.N; d.A = l.A; d.P = l.P; d.JM = l.JM; d.NJ = l.NJ; d.nblocks = l.nblocks; d.ncc = l.ncc;
  d.n_ob = (int)l.ob_kind.size();
  d.n_ai = (int)l.ai_a.size();
  d.sj_nh = l.sj_nh;
  d.off_fhh = l.off_fhh; d.off_fpp = l.off_fpp; d.off_fph = l.off_fph; d.slab = l.slab;
  d.n_unique = l.n_unique; d.cc_size = l.cc_size; d.wcc_size = l.wcc_size;
  std::vector<int> ncls(l.nblocks * 3);
  for (int q = 0; q < l.nblocks; ++q)
    for (int c = 0; c < 3; ++c) ncls[q * 3 + c] = l.ncls[q][c];
  pk.add(l.jj, &d.jj); pk.add(l.ll, &d.ll); pk.add(l.tz, &d.tz); pk.add(l.con, &d.con); pk.add(l.loc, &d.loc);
  pk.add(l.holes, &d.holes); pk.add(l.parts, &d.parts);
  pk.add(l.same_start, &d.same_start); pk.add(l.same_count, &d.same_count); pk.add(l.same_list, &d.same_list);
  pk.add(l.lamJ, &d.lamJ); pk.add(ncls, &d.ncls); pk.add(l.pair_off, &d.pair_off);
  pk.add(l.pair_a, &d.pair_a); pk.add(l.pair_b, &d.pair_b); pk.add(l.pairpos, &d.pairpos);
  pk.add(l.goff, &d.goff); pk.add(l.gn1, &d.gn1); pk.add(l.gn2, &d.gn2); pk.add(l.uoff, &d.uoff);
  pk.add(l.cc_rlen, &d.cc_rlen); pk.add(l.cc_nph, &d.cc_nph); pk.add(l.cc_J, &d.cc_J);
  pk.add(l.cc_off, &d.cc_off); pk.add(l.wcc_off, &d.wcc_off);
  pk.add(l.cc_row_off, &d.cc_row_off); pk.add(l.cc_col_off, &d.cc_col_off);
  pk.add(l.cc_ra, &d.cc_ra); pk.add(l.cc_rb, &d.cc_rb); pk.add(l.cc_cp, &d.cc_cp); pk.add(l.cc_ch, &d.cc_ch);
  pk.add(l.ccr, &d.ccr);
  // transposed copies (b fastest) for warps whose lanes vary the second orbit
  std::vector<int> ccr_t(l.ccr.size()), ppos_t(l.pairpos.size());
  for (int a = 0; a < l.N; ++a)
    for (int b = 0; b < l.N; ++b)
      for (int h = 0; h < l.NJ; ++h) {
        ccr_t[((size_t)a * l.NJ + h) * l.N + b] = l.ccr[((size_t)a * l.N + b) * l.NJ + h];
        ppos_t[((size_t)a * l.NJ + h) * l.N + b] = l.pairpos[((size_t)a * l.N + b) * l.NJ + h];
      }
  pk.add(ccr_t, &d.ccr_t);
  pk.add(ppos_t, &d.pairpos_t);
  pk.add(l.ob_kind, &d.ob_kind); pk.add(l.ob_p, &d.ob_p); pk.add(l.ob_q, &d.ob_q);
  pk.add(l.ob_pk, &d.ob_pk); pk.add(l.ob_qk, &d.ob_qk);
  pk.add(l.ai_a, &d.ai_a); pk.add(l.ai_i, &d.ai_i);
  pk.add(l.sj_off, &d.sj_off); pk.add(l.sj_j3min, &d.sj_j3min); pk.add(l.sj_j6min, &d.sj_j6min);
  pk.add(l.sj_n6, &d.sj_n6); pk.add(l.sj_val, &d.sj_val);
  std::vector<float> sjf(l.sj_val.begin(), l.sj_val.end());
  pk.add(sjf, &d.sj_valf);
  // GEMM plans
  pphh_probs = build_pphh_problems(l.nblocks, l.ncls, l.goff);
  pphh_tiles = build_tiles(pphh_probs, 64, 64);
  wcc_probs = build_wcc_problems(l.ncc, l.cc_rlen, l.cc_nph, l.cc_off, l.wcc_off);
  wcc_tiles = build_tiles(wcc_probs, 64, 64);
  // 222_pp_hh intermediates: every W1 / W2 problem writes its whole array, so only the arrays
  // no problem writes (channels without pp or without hh pairs), and E0 and the one-body
  // part, are cleared before the products (src/commutators.f90:581-768 leaves them zero)
  for (int w = 0; w < 2; ++w) {
    std::vector<char> covered((size_t)l.nblocks * 6, 0);
    for (const GemmProb& p : pphh_probs)
      if (p.c_id == (w ? kOpW2 : kOpW1))
        for (int k = 0; k < l.nblocks * 6; ++k)
          if (l.goff[k] == p.c_off && p.M == l.gn1[k] && p.N == l.gn2[k] && p.M * (int64_t)p.N > 0) covered[k] = 1;
    std::vector<int64_t>& runs = w ? zero_runs_w2 : zero_runs_w1;
    runs.clear();
    auto add = [&](int64_t a, int64_t n) {
      if (n <= 0) return;
      if (!runs.empty() && runs[runs.size() - 2] + runs.back() == a) runs.back() += n;
      else { runs.push_back(a); runs.push_back(n); }
    };
    add(0, l.goff[0]);
    for (int k = 0; k < l.nblocks * 6; ++k)
      if (!covered[k]) add(l.goff[k], (int64_t)l.gn1[k] * l.gn2[k]);
    // one CTA per run of at most 32768 elements (k_zero_runs)
    std::vector<int64_t> split;
    for (size_t r = 0; r < runs.size(); r += 2)
      for (int64_t o = 0; o < runs[r + 1]; o += 32768) {
        split.push_back(runs[r] + o);
        split.push_back(std::min<int64_t>(32768, runs[r + 1] - o));
      }
    runs.swap(split);
  }
  // Frobenius-norm segments: chunks of at most 64K elements inside one array
  std::vector<int64_t> s_start;
  std::vector<int> s_len;
  std::vector<int8_t> s_w;
  auto add_seg = [&](int64_t off, int64_t n, int w) {
    for (int64_t o = 0; o < n; o += 65536) {
      s_start.push_back(off + o);
      s_len.push_back((int)std::min<int64_t>(65536, n - o));
      s_w.push_back((int8_t)w);
    }
  };
  add_seg(l.off_fhh, (int64_t)l.A * l.A, 1);
  add_seg(l.off_fph, (int64_t)l.P * l.A, 2);
  add_seg(l.off_fpp, (int64_t)l.P * l.P, 1);
  for (int k = 0; k < l.nblocks * 6; ++k) add_seg(l.goff[k], (int64_t)l.gn1[k] * l.gn2[k], kSquare[k % 6] ? 1 : 2);
  nseg = (int)s_start.size();
  // 222_pp_hh accumulation tiles: (array, row0, col0, square); square arrays by tile pairs
  for (int k = 0; k < l.nblocks * 6; ++k) {
    const int n1 = l.gn1[k], n2 = l.gn2[k];
    if ((int64_t)n1 * n2 == 0) continue;
    if (kSquare[k % 6]) {
      for (int i0 = 0; i0 < n1; i0 += 32)
        for (int j0 = i0; j0 < n1; j0 += 32) upd_tiles.push_back(make_int4(k, i0, j0, 1));
    } else {
      for (int j0 = 0; j0 < n2; j0 += 32)
        for (int i0 = 0; i0 < n1; i0 += 32) upd_tiles.push_back(make_int4(k, i0, j0, 0));
    }
  }
  const GemmProb* pp_p = nullptr; const GemmTile* pp_t = nullptr;
  const GemmProb* wc_p = nullptr; const GemmTile* wc_t = nullptr;
  const int64_t* seg_s = nullptr; const int* seg_l = nullptr; const int8_t* seg_w = nullptr;
  pk.add(pphh_probs, &pp_p); pk.add(pphh_tiles, &pp_t); pk.add(wcc_probs, &wc_p); pk.add(wcc_tiles, &wc_t);
  pk.add(s_start, &seg_s); pk.add(s_len, &seg_l); pk.add(s_w, &seg_w);
  const int4* ut = nullptr;
  pk.add(upd_tiles, &ut);
  const int64_t *zr1 = nullptr, *zr2 = nullptr;
  pk.add(zero_runs_w1, &zr1);
  pk.add(zero_runs_w2, &zr2);

  CK(cuda(cudaMalloc(&d_tables, pk.buf.size()), "cudaMalloc(tables)"));
  CK(cuda(cudaMemcpy(d_tables, pk.buf.data(), pk.buf.size(), cudaMemcpyHostToDevice), "cudaMemcpy(tables)"));
  for (auto& f : pk.fix) *f.second = static_cast<const char*>(d_tables) + f.first;
  d_pphh_probs = pp_p; d_pphh_tiles = pp_t; d_wcc_probs = wc_p; d_wcc_tiles = wc_t;
  d_seg_start = seg_s; d_seg_len = seg_l; d_seg_w = seg_w;
  d_upd_tiles = ut;
  d_zero_runs_w1 = zr1;
  d_zero_runs_w2 = zr2;
  partial_capacity = std::max(nseg, l.nblocks) + 64;
  CK(cuda(cudaMalloc(&d_partial, sizeof(double) * partial_capacity), "cudaMalloc(partials)"));
  CK(cuda(cudaMalloc(&d_scalars, sizeof(double) * 64), "cudaMalloc(scalars)"));
  CK(cuda(cudaMallocHost(&h_scalars, sizeof(double) * 64), "cudaMallocHost(scalars)"));
  CK(cuda(cudaMalloc(&d_mono, sizeof(double) * (size_t)l.N * l.N), "cudaMalloc(monopole)"));
  return IMSRG_OK;
}

imsrg_status Ctx::ensure_workspace() {
  if (d_w1) return IMSRG_OK;
  const size_t sb = sizeof(double) * (size_t)L.slab;
  CK(cuda(cudaMalloc(&d_w1, sb), "cudaMalloc(w1)"));
  CK(cuda(cudaMalloc(&d_w2, sb), "cudaMalloc(w2)"));
  CK(cuda(cudaMalloc(&d_lcc, sizeof(double) * std::max<int64_t>(L.cc_size, 1)), "cudaMalloc(LCC)"));
  CK(cuda(cudaMalloc(&d_rcc, sizeof(double) * std::max<int64_t>(L.cc_size, 1)), "cudaMalloc(RCC)"));
  return IMSRG_OK;
}

// FP64 WCC workspace of the plain path (1.46 GiB at eMax=10), allocated on first use
imsrg_status Ctx::ensure_wcc() {
  if (d_wcc) return IMSRG_OK;
  CK(cuda(cudaMalloc(&d_wcc, sizeof(double) * std::max<int64_t>(L.wcc_size, 1)), "cudaMalloc(WCC)"));
  CK(cuda(cudaMemsetAsync(d_wcc, 0, sizeof(double) * std::max<int64_t>(L.wcc_size, 1), stream), "memset(WCC)"));
  return IMSRG_OK;
}

imsrg_status Ctx::ensure_flow_workspace() {
  if (d_int1) return IMSRG_OK;
  const size_t sb = sizeof(double) * (size_t)L.slab;
  CK(cuda(cudaMalloc(&d_int1, sb), "cudaMalloc(INT1)"));
  CK(cuda(cudaMalloc(&d_int2, sb), "cudaMalloc(INT2)"));
  CK(cuda(cudaMalloc(&d_ad, sb), "cudaMalloc(AD)"));
  return IMSRG_OK;
}

Ctx::~Ctx() {
  for (void* p : {(void*)d_tables, (void*)d_partial, (void*)d_scalars, (void*)d_mono, (void*)d_w1, (void*)d_w2,
                  (void*)d_lcc, (void*)d_rcc, (void*)d_wcc, (void*)d_int1, (void*)d_int2, (void*)d_ad, (void*)d_gen})
    if (p) cudaFree(p);
  if (h_scalars) cudaFreeHost(h_scalars);
  quads_release();
  for (auto& m : prof_marks) cudaEventDestroy(m.second);
  for (auto e : prof_pool) cudaEventDestroy(e);
  if (ev_begin) cudaEventDestroy(ev_begin);
  if (ev_end) cudaEventDestroy(ev_end);
  if (ev_ext_in) cudaEventDestroy(ev_ext_in);
  if (ev_ext_out) cudaEventDestroy(ev_ext_out);
  if (stream) cudaStreamSynchronize(stream);
  for (double* p : op_pool) cudaFree(p);
  tc_release();
  graph_release();
  adjoint_release();
  tensor_release();
  hf_release();
  if (stream) cudaStreamDestroy(stream);
}

// ---------------------------------------------------------------- building blocks
imsrg_status Ctx::pandya(const double* op, int herm, double* cc) {
  if (L.cc_size == 0) return IMSRG_OK;
  k_pandya<<<grid_for(L.cc_size), kThreads, 0, stream>>>(D, op, herm, cc);
  return launched("k_pandya");
}

imsrg_status Ctx::e0(const double* Lp, int hL, const double* Rp, int hR, double* RES, double* out) {
  k_e0_partial<<<L.nblocks + 1, 256, 0, stream>>>(D, Lp, hL, Rp, hR, d_partial);
  CK(launched("k_e0_partial"));
  k_e0_final<<<1, 32, 0, stream>>>(D, d_partial, RES, out);
  return launched("k_e0_final");
}

imsrg_status Ctx::c111(const double* Lp, int hL, const double* Rp, int hR, double* RES) {
  const int64_t n = (int64_t)L.A * L.A + (int64_t)L.P * L.A + (int64_t)L.P * L.P;
  k_comm111<<<grid_for(n * 32), kThreads, 0, stream>>>(D, Lp, hL, Rp, hR, RES);
  return launched("k_comm111");
}

imsrg_status Ctx::c121(const double* Lp, int hL, const double* Rp, int hR, double* RES, int hRES) {
  if (D.n_ob == 0) return IMSRG_OK;
  k_comm121<<<(D.n_ob * 32 + kThreads - 1) / kThreads, kThreads, 0, stream>>>(D, Lp, hL, Rp, hR, RES, hRES);
  return launched("k_comm121");
}

imsrg_status Ctx::c122(const double* Lp, int hL, const double* Rp, int hR, double* RES, int hRES) {
  if (L.n_unique == 0) return IMSRG_OK;
  k_comm122<<<grid_for(L.n_unique), kThreads, 0, stream>>>(D, Lp, hL, Rp, hR, RES, hRES);
  return launched("k_comm122");
}

// w1, w2 of 222_pp_hh: the parts no product writes are cleared
imsrg_status Ctx::pphh_clear(double* w1, double* w2) {
  if (!zero_runs_w1.empty()) {
    k_zero_runs<<<(int)zero_runs_w1.size() / 2, 256, 0, stream>>>(w1, d_zero_runs_w1);
    CK(launched("k_zero_runs"));
  }
  if (!zero_runs_w2.empty()) {
    k_zero_runs<<<(int)zero_runs_w2.size() / 2, 256, 0, stream>>>(w2, d_zero_runs_w2);
    CK(launched("k_zero_runs"));
  }
  return IMSRG_OK;
}

imsrg_status Ctx::pphh_clear_f(float* w1, float* w2) {
  if (!zero_runs_w1.empty()) {
    k_zero_runs_f<<<(int)zero_runs_w1.size() / 2, 256, 0, stream>>>(w1, d_zero_runs_w1);
    CK(launched("k_zero_runs_f"));
  }
  if (!zero_runs_w2.empty()) {
    k_zero_runs_f<<<(int)zero_runs_w2.size() / 2, 256, 0, stream>>>(w2, d_zero_runs_w2);
    CK(launched("k_zero_runs_f"));
  }
  return IMSRG_OK;
}

// RES += W1 - W2 - pm (W1 - W2)^T on the square arrays, RES += W1 - W2 on the others
imsrg_status Ctx::pphh_accumulate(int hL, int hR, double* RES, const double* w1, const double* w2) {
  if (!upd_tiles.empty()) {
    k_pphh_update_tiled<<<(int)upd_tiles.size(), 256, 0, stream>>>(D, d_upd_tiles, RES, w1, w2, (double)(hL * hR));
    CK(launched("k_pphh_update_tiled"));
  }
  mark(kPhasePphhUpdate);
  return IMSRG_OK;
}



imsrg_status Ctx::pphh(const double* Lp, int hL, const double* Rp, int hR, double* RES, double* w1, double* w2) {
  CK(pphh_clear(w1, w2));
  if (precision != IMSRG_PREC_FP64) {
    CK(tc_pphh(Lp, hL, Rp, hR, w1, w2));
  } else if (!pphh_tiles.empty()) {
    GemmOperands ops{};
    ops.in[kOpL] = Lp; ops.in[kOpR] = Rp;
    ops.out[kOpW1] = w1; ops.out[kOpW2] = w2;
    ops.hL = hL; ops.hR = hR;
    k_gemm_fp64<<<(int)pphh_tiles.size(), 256, 0, stream>>>(d_pphh_probs, d_pphh_tiles, ops);
    CK(launched("k_gemm_fp64(pphh)"));
  }
  mark(kPhasePphhGemm);
  return pphh_accumulate(hL, hR, RES, w1, w2);
}

imsrg_status Ctx::c221_f(int hL, int hR, double* RES, int hRES, const float* w1, const float* w2) {
  if (D.n_ob == 0) return IMSRG_OK;
  k_comm221f<<<D.n_ob, 256, 0, stream>>>(D, hL * hR, RES, hRES, w1, w2);
  return launched("k_comm221f");
}

imsrg_status Ctx::c221(int hL, int hR, double* RES, int hRES, const double* w1, const double* w2) {
  if (D.n_ob == 0) return IMSRG_OK;
  k_comm221<<<(D.n_ob * 32 + kThreads - 1) / kThreads, kThreads, 0, stream>>>(D, hL * hR, RES, hRES, w1, w2);
  return launched("k_comm221");
}

imsrg_status Ctx::ph(const double* lcc, int hL, const double* rcc, int hR, double* RES, int hRES, double* wcc) {
  // the piecewise entry point keeps the reference's FP64 WCC; the mixed-precision full
  // commutator (tc_commutator) uses the fused split-BF16 path instead
  if (!wcc_tiles.empty()) {
    GemmOperands ops{};
    ops.in[kOpLCC] = lcc; ops.in[kOpRCC] = rcc;
    ops.out[kOpWCC] = wcc;
    ops.hL = hL; ops.hR = hR;
    k_gemm_fp64<<<(int)wcc_tiles.size(), 256, 0, stream>>>(d_wcc_probs, d_wcc_tiles, ops);
    CK(launched("k_gemm_fp64(wcc)"));
  }
  mark(kPhasePhGemm);
  if (L.n_unique == 0) return IMSRG_OK;
  k_comm222ph<<<grid_for(L.n_unique), kThreads, 0, stream>>>(D, wcc, hL, hR, RES, hRES);
  CK(launched("k_comm222ph"));
  mark(kPhaseRecouple);
  return IMSRG_OK;
}

imsrg_status Ctx::commutator(const double* Lp, int hL, const double* Rp, int hR, double* RES, int hRES, bool with_e0) {
  CK(ensure_workspace());
  if (precision != IMSRG_PREC_FP64) return tc_commutator(Lp, hL, Rp, hR, RES, hRES, with_e0);
  mark(kPhaseStart);
  CK(pandya(Rp, hR, d_rcc));
  CK(pandya(Lp, hL, d_lcc));
  mark(kPhasePandya);
  if (with_e0) CK(e0(Lp, hL, Rp, hR, RES, nullptr));
  CK(c111(Lp, hL, Rp, hR, RES));
  CK(c121(Lp, hL, Rp, hR, RES, hRES));
  mark(kPhaseOneBody);
  CK(c122(Lp, hL, Rp, hR, RES, hRES));
  mark(kPhase122);
  CK(pphh(Lp, hL, Rp, hR, RES, d_w1, d_w2));
  CK(c221(hL, hR, RES, hRES, d_w1, d_w2));
  mark(kPhase221);
  CK(ensure_wcc());
  CK(ph(d_lcc, hL, d_rcc, hR, RES, hRES, d_wcc));
  return IMSRG_OK;
}

imsrg_status Ctx::axpby(const double* A, double ax, const double* B, double bx, double* C) {
  k_axpby<<<grid_for(L.slab), kThreads, 0, stream>>>(L.slab, A, ax, B, bx, C);
  return launched("k_axpby");
}

// Y += a X and the Frobenius norm of X times scale into d_scalars[slot], in one pass (E0 of Y
// updated only with with_e0); no synchronization
imsrg_status Ctx::axpy_frob_async(double* Y, double a, const double* X, double scale, int slot, bool with_e0) {
  if (nseg == 0) {
    CK(axpby(Y, 1.0, X, a, Y));
    return frob_async(X, scale, slot);
  }
  k_axpy_frob<<<nseg, 256, 0, stream>>>(Y, a, X, d_seg_start, d_seg_len, d_seg_w, d_partial, with_e0 ? 1 : 0);
  CK(launched("k_axpy_frob"));
  k_sum_sqrt<<<1, 1024, 0, stream>>>(d_partial, nseg, scale, d_scalars + slot);
  return launched("k_sum_sqrt");
}

// Frobenius norm times scale into d_scalars[slot] (device); no synchronization
imsrg_status Ctx::frob_async(const double* op, double scale, int slot) {
  if (nseg == 0) return cuda(cudaMemsetAsync(d_scalars + slot, 0, sizeof(double), stream), "memset(norm)");
  k_frob_partial<<<nseg, 256, 0, stream>>>(op, d_seg_start, d_seg_len, d_seg_w, d_partial);
  CK(launched("k_frob_partial"));
  k_sum_sqrt<<<1, 1024, 0, stream>>>(d_partial, nseg, scale, d_scalars + slot);
  return launched("k_sum_sqrt");
}

imsrg_status Ctx::read_scalars(int n) {
  CK(cuda(cudaMemcpyAsync(h_scalars, d_scalars, sizeof(double) * n, cudaMemcpyDeviceToHost, stream), "D2H scalars"));
  return cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
}

imsrg_status Ctx::white(const double* H, int hH, double* ETA) {
  CK(cuda(cudaMemsetAsync(ETA, 0, sizeof(double) * (size_t)L.slab, stream), "memset(ETA)"));
  k_monopole<<<(L.N * L.N + kThreads - 1) / kThreads, kThreads, 0, stream>>>(D, H, hH, d_mono);
  CK(launched("k_monopole"));
  if (D.n_ai > 0) {
    k_white_1b<<<(D.n_ai + kThreads - 1) / kThreads, kThreads, 0, stream>>>(D, H, hH, ETA);
    CK(launched("k_white_1b"));
  }
  dim3 grid(16, L.nblocks);
  k_white_2b<<<grid, kThreads, 0, stream>>>(D, H, hH, d_mono, ETA);
  return launched("k_white_2b");
}

// build_gs_atan (Hnum == Hden) and build_gs_atanxx (src/generators.f90:163-374)
imsrg_status Ctx::atan_generator(const double* Hden, int hden, const double* Hnum, double* ETA) {
  CK(cuda(cudaMemsetAsync(ETA, 0, sizeof(double) * (size_t)L.slab, stream), "memset(ETA)"));
  k_monopole<<<(L.N * L.N + kThreads - 1) / kThreads, kThreads, 0, stream>>>(D, Hden, hden, d_mono);
  CK(launched("k_monopole"));
  if (D.n_ai > 0) {
    k_atan_1b<<<(D.n_ai + kThreads - 1) / kThreads, kThreads, 0, stream>>>(D, Hden, hden, Hnum, ETA);
    CK(launched("k_atan_1b"));
  }
  dim3 grid(16, L.nblocks);
  k_atan_2b<<<grid, kThreads, 0, stream>>>(D, Hden, hden, Hnum, d_mono, ETA);
  return launched("k_atan_2b");
}

// build_gs_w2 (src/generators.f90:109-160): 1.5 atan(H) + 0.5 atanxx(H, [atan(H), H]), the
// commutator in the context's precision; three slab workspaces kept between calls
imsrg_status Ctx::w2_generator(const double* H, int hH, double* ETA) {
  if (!d_gen) {
    CK(cuda(cudaMalloc(&d_gen, 3 * sizeof(double) * (size_t)L.slab), "cudaMalloc(w2 generator workspace)"));
  }
  double* eta1 = d_gen;
  double* h2 = d_gen + L.slab;
  double* eta2 = d_gen + 2 * L.slab;
  CK(atan_generator(H, hH, H, eta1));
  CK(commutator(eta1, -1, H, hH, h2, hH, true));
  CK(atan_generator(H, hH, h2, eta2));
  return axpby(eta1, 1.5, eta2, 0.5, ETA);
}

// MAGNUS_EXPAND (src/IMSRG_MAGNUS.f90:620-691) with device-resident operators; the
// early-exit tests read two norms back per nested commutator, as the reference decides
// on host scalars.
imsrg_status Ctx::magnus_expand(double* DG, int hDG, const double* G, int hG, int* used) {
  CK(ensure_workspace());
  CK(ensure_flow_workspace());
  const double conv = (double)1e-6f;
  const double* cof = kMagnusCof;
  double advals[8] = {0};
  CK(frob_async(DG, 1.0, 0));
  CK(frob_async(G, 1.0, 1));
  CK(read_scalars(2));
  advals[1] = h_scalars[0];
  const double fullnorm = h_scalars[1];
  *used = 0;
  if (fullnorm < (double)1e-9f) return IMSRG_OK;
  int qq = 1;
  // ad^(i-1) and ad^i alternate between two buffers (the first input is DG itself, read before
  // DG is updated); DG += cof ad^i with the norm of ad^i in the same pass (E0 of DG kept: the
  // nested commutators do not form one)
  for (int i = 2; i <= 7; ++i) {
    const double adnorm = advals[i - qq];
    qq = (std::fabs(cof[i - 1]) > (double)1e-6f) ? 1 : 2;
    if (std::fabs(adnorm / fullnorm) < conv) break;
    const double* ad = (i == 2) ? DG : ((i & 1) ? d_int2 : d_ad);
    double* out = (i & 1) ? d_ad : d_int2;
    CK(commutator(G, hG, ad, hDG, out, hDG, false));
    ++*used;
    CK(axpy_frob_async(DG, cof[i - 1], out, std::fabs(cof[i - 1]), 0, false));
    CK(read_scalars(1));
    advals[i] = h_scalars[0];
  }
  return IMSRG_OK;
}

// BCH_EXPAND (src/IMSRG_MAGNUS.f90:149-234)
imsrg_status Ctx::bch_expand(double* HS, const double* G, int hG, const double* H, int hH, int max_terms,
                             double conv, int* terms, bool cr, bool quads) {
  CK(ensure_workspace());
  CK(ensure_flow_workspace());
  double* int3 = nullptr;  // quads: the correction added to the next nested commutator
  if (quads) {
    CK(quads_prepare());
    int3 = quads_int3();
    CK(cuda(cudaMemsetAsync(int3, 0, sizeof(double) * (size_t)L.slab, stream), "memset(INT3)"));
  }
  const size_t sb = sizeof(double) * (size_t)L.slab;
  CK(cuda(cudaMemcpyAsync(HS, H, sb, cudaMemcpyDeviceToDevice, stream), "copy HS"));
  // ad^(n-1)(H) and ad^n(H) alternate between two buffers; the commutator assigns every
  // element of its output (E0 included), so neither a copy nor a clear is needed
  double coef = 1.0;
  int iw;
  for (iw = 2; iw <= max_terms; ++iw) {
    coef = cr ? coef / iw : coef / (iw - 1.0);  // CR_EXPAND: 1/n! on ad^(n-1)(H)
    const double* ad = (iw == 2) ? H : ((iw & 1) ? d_int2 : d_ad);
    double* out = (iw & 1) ? d_ad : d_int2;
    CK(commutator(G, hG, ad, hH, out, hH, true));
    if (quads) {
      CK(axpby(out, 1.0, int3, 1.0, out));
      CK(restore_quadrupoles(ad, hH, G, hG, int3));
    }
    CK(axpy_frob_async(HS, coef, out, coef, 0, true));
    CK(read_scalars(1));
    if (h_scalars[0] < conv) break;
  }
  *terms = (iw > max_terms) ? max_terms - 1 : iw - 1;
  if (iw > max_terms && !cr) return fail(IMSRG_ERR_NOT_CONVERGED, "BCH series did not converge within max_terms");
  return IMSRG_OK;  // CR_EXPAND ends after max_terms without an error, as the reference does
}

// ====================================================================== C ABI
namespace {

imsrg_status check_op(Ctx* c, const imsrg_op* op, const char* name) {
  if (!op || op->owner != c) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, std::string(name) + ": operator of another context or NULL");
  return IMSRG_OK;
}
imsrg_status check_cc(Ctx* c, const imsrg_cc* cc, int kind, const char* name) {
  if (!cc || cc->owner != c) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, std::string(name) + ": cc matrix of another context or NULL");
  if (cc->kind != kind)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, std::string(name) + (kind ? ": expected a WCC workspace" : ": expected a CCX matrix"));
  return IMSRG_OK;
}

}  // namespace

#define CTX(ptr)                                                                         \
  if (!(ptr)) return IMSRG_ERR_INVALID_ARGUMENT;                                         \
  Ctx* c = reinterpret_cast<Ctx*>(ptr);                                                  \
  if (c->device < 0) return c->fail(IMSRG_ERR_UNSUPPORTED, "host-only context (device < 0)"); \
  {                                                                                      \
    cudaError_t _e = cudaSetDevice(c->device);                                           \
    if (_e != cudaSuccess) return c->cuda(_e, "cudaSetDevice");                          \
  }

extern "C" {

imsrg_status imsrg_ctx_create(const imsrg_basis* b, int32_t device, imsrg_ctx** out) {
  if (!b || !out || !b->nn || !b->ll || !b->jj || !b->itzp || !b->con) return IMSRG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  Ctx* c = new (std::nothrow) Ctx();
  if (!c) return IMSRG_ERR_OUT_OF_MEMORY;
  c->device = device;
  std::string e = build_layout(c->L, b->norbits, b->nn, b->ll, b->jj, b->itzp, b->con, b->eMax, b->hw, b->Aprot,
                               b->Aneut);
  if (!e.empty()) {
    delete c;
    return IMSRG_ERR_INVALID_ARGUMENT;
  }
  if (device < 0) {  // host-only context: layout queries and input preparation
    *out = reinterpret_cast<imsrg_ctx*>(c);
    return IMSRG_OK;
  }
  imsrg_status s = c->cuda(cudaSetDevice(device), "cudaSetDevice");
  if (s == IMSRG_OK) s = c->cuda(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  if (s == IMSRG_OK) s = c->cuda(cudaEventCreateWithFlags(&c->ev_ext_in, cudaEventDisableTiming), "cudaEventCreate");
  if (s == IMSRG_OK) s = c->cuda(cudaEventCreateWithFlags(&c->ev_ext_out, cudaEventDisableTiming), "cudaEventCreate");
  if (s == IMSRG_OK) s = c->upload_tables();
  if (s != IMSRG_OK) {
    delete c;
    return s;
  }
  *out = reinterpret_cast<imsrg_ctx*>(c);
  return IMSRG_OK;
}

imsrg_status imsrg_ctx_destroy(imsrg_ctx* ctx) {
  if (!ctx) return IMSRG_OK;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (c->device >= 0) {
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
  }
  delete c;
  return IMSRG_OK;
}

const char* imsrg_last_error(const imsrg_ctx* ctx) {
  if (!ctx) return "NULL context";
  return reinterpret_cast<const Ctx*>(ctx)->err.c_str();
}

imsrg_status imsrg_ctx_sizes(const imsrg_ctx* ctx, int64_t* slab, int64_t* cc, int64_t* wcc, int32_t* nblocks,
                             int32_t* ncc) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  const Ctx* c = reinterpret_cast<const Ctx*>(ctx);
  if (slab) *slab = c->L.slab;
  if (cc) *cc = c->L.cc_size;
  if (wcc) *wcc = c->L.wcc_size;
  if (nblocks) *nblocks = c->L.nblocks;
  if (ncc) *ncc = c->L.ncc;
  return IMSRG_OK;
}

imsrg_status imsrg_block_info(const imsrg_ctx* ctx, int32_t* lamJ, int32_t* lamP, int32_t* lamT, int32_t* npp,
                              int32_t* nph, int32_t* nhh) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  const Layout& L = reinterpret_cast<const Ctx*>(ctx)->L;
  for (int q = 0; q < L.nblocks; ++q) {
    if (lamJ) lamJ[q] = L.lamJ[q];
    if (lamP) lamP[q] = L.lamP[q];
    if (lamT) lamT[q] = L.lamT[q];
    if (npp) npp[q] = L.ncls[q][0];
    if (nph) nph[q] = L.ncls[q][1];
    if (nhh) nhh[q] = L.ncls[q][2];
  }
  return IMSRG_OK;
}

imsrg_status imsrg_block_pairs(const imsrg_ctx* ctx, int32_t q, int32_t cls, int32_t* out) {
  if (!ctx || !out) return IMSRG_ERR_INVALID_ARGUMENT;
  const Layout& L = reinterpret_cast<const Ctx*>(ctx)->L;
  if (q < 0 || q >= L.nblocks || cls < 0 || cls > 2) return IMSRG_ERR_INVALID_ARGUMENT;
  const int o = L.pair_off[q * 3 + cls], n = L.ncls[q][cls];
  for (int k = 0; k < n; ++k) {
    out[2 * k] = L.pair_a[o + k];
    out[2 * k + 1] = L.pair_b[o + k];
  }
  return IMSRG_OK;
}

imsrg_status imsrg_cc_info(const imsrg_ctx* ctx, int32_t* rlen, int32_t* nph, int32_t* J) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  const Layout& L = reinterpret_cast<const Ctx*>(ctx)->L;
  for (int q = 0; q < L.ncc; ++q) {
    if (rlen) rlen[q] = L.cc_rlen[q];
    if (nph) nph[q] = L.cc_nph[q];
    if (J) J[q] = L.cc_J[q];
  }
  return IMSRG_OK;
}

imsrg_status imsrg_set_precision(imsrg_ctx* ctx, int32_t mode) {
  CTX(ctx);
  if (mode != IMSRG_PREC_FP64 && mode != IMSRG_PREC_BF16X3 && mode != IMSRG_PREC_BF16X6 && mode != IMSRG_PREC_TF32X3)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "unknown precision mode");
  if (mode != IMSRG_PREC_FP64) CK(c->tc_prepare(mode));
  c->precision = mode;
  return IMSRG_OK;
}

imsrg_status imsrg_synchronize(imsrg_ctx* ctx) {
  CTX(ctx);
  CK(c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize"));
  return c->tc_error();
}

imsrg_status imsrg_set_wait_limit(imsrg_ctx* ctx, int64_t nanoseconds) {
  CTX(ctx);
  if (nanoseconds < 0) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_set_wait_limit: negative limit");
  c->tc_wait_ns = nanoseconds ? (unsigned long long)nanoseconds : 2000000000ull;
  return IMSRG_OK;
}

imsrg_status imsrg_test_unarmed_stage(imsrg_ctx* ctx, int32_t enable) {
  CTX(ctx);
  c->tc_unarmed_next = enable ? 1 : 0;
  return IMSRG_OK;
}

imsrg_status imsrg_launch_count(imsrg_ctx* ctx, int64_t* count) {
  if (!ctx || !count) return IMSRG_ERR_INVALID_ARGUMENT;
  *count = reinterpret_cast<Ctx*>(ctx)->launches;
  return IMSRG_OK;
}

imsrg_status imsrg_timer_begin(imsrg_ctx* ctx) {
  CTX(ctx);
  if (!c->ev_begin) CK(c->cuda(cudaEventCreate(&c->ev_begin), "cudaEventCreate"));
  if (!c->ev_end) CK(c->cuda(cudaEventCreate(&c->ev_end), "cudaEventCreate"));
  return c->cuda(cudaEventRecord(c->ev_begin, c->stream), "cudaEventRecord");
}

imsrg_status imsrg_timer_end(imsrg_ctx* ctx, float* ms) {
  CTX(ctx);
  if (!ms || !c->ev_begin) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_timer_begin was not called");
  CK(c->cuda(cudaEventRecord(c->ev_end, c->stream), "cudaEventRecord"));
  CK(c->cuda(cudaEventSynchronize(c->ev_end), "cudaEventSynchronize"));
  return c->cuda(cudaEventElapsedTime(ms, c->ev_begin, c->ev_end), "cudaEventElapsedTime");
}

imsrg_status imsrg_profile_phases(imsrg_ctx* ctx, int32_t enable) {
  CTX(ctx);
  CK(c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize"));
  for (auto& m : c->prof_marks) c->prof_pool.push_back(m.second);
  c->prof_marks.clear();
  c->prof = enable != 0;
  return IMSRG_OK;
}

imsrg_status imsrg_profile_read(imsrg_ctx* ctx, float* ms_per_phase, int32_t* count_per_phase) {
  CTX(ctx);
  if (!ms_per_phase || !count_per_phase) return IMSRG_ERR_INVALID_ARGUMENT;
  CK(c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize"));
  for (int p = 0; p < IMSRG_NUM_PHASES; ++p) {
    ms_per_phase[p] = 0.f;
    count_per_phase[p] = 0;
  }
  for (size_t i = 1; i < c->prof_marks.size(); ++i) {
    const int p = c->prof_marks[i].first;
    if (p == kPhaseStart || p < 0 || p >= IMSRG_NUM_PHASES) continue;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->prof_marks[i - 1].second, c->prof_marks[i].second);
    ms_per_phase[p] += ms;
    count_per_phase[p] += 1;
  }
  return IMSRG_OK;
}

imsrg_status imsrg_op_create(imsrg_ctx* ctx, int32_t herm, imsrg_op** out) {
  CTX(ctx);
  if (!out || (herm != 1 && herm != -1)) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "herm must be +1 or -1");
  *out = nullptr;
  imsrg_op* op = new (std::nothrow) imsrg_op();
  if (!op) return IMSRG_ERR_OUT_OF_MEMORY;
  const size_t sb = sizeof(double) * (size_t)c->L.slab;
  imsrg_status s = IMSRG_OK;
  if (!c->op_pool.empty()) {  // recycled slab: stream order makes the reuse safe
    op->d = c->op_pool.back();
    c->op_pool.pop_back();
  } else {
    s = c->cuda(cudaMalloc(&op->d, sb), "cudaMalloc(operator)");
  }
  if (s == IMSRG_OK) s = c->cuda(cudaMemsetAsync(op->d, 0, sb, c->stream), "memset(operator)");
  if (s != IMSRG_OK) {
    if (op->d) cudaFree(op->d);
    delete op;
    return s;
  }
  op->herm = herm;
  op->owner = c;
  *out = op;
  return IMSRG_OK;
}

imsrg_status imsrg_op_destroy(imsrg_ctx* ctx, imsrg_op* op) {
  CTX(ctx);
  if (!op) return IMSRG_OK;
  CK(check_op(c, op, "imsrg_op_destroy"));
  // keep up to 16 GiB of operator slabs for reuse (work still queued on the context's
  // stream finishes before a later op_create's memset on the same stream touches them)
  const size_t sb = sizeof(double) * (size_t)c->L.slab;
  if ((c->op_pool.size() + 1) * sb <= (size_t(16) << 30)) {
    c->op_pool.push_back(op->d);
  } else {
    cudaStreamSynchronize(c->stream);
    cudaFree(op->d);
  }
  delete op;
  return IMSRG_OK;
}

imsrg_status imsrg_op_set_herm(imsrg_ctx* ctx, imsrg_op* op, int32_t herm) {
  CTX(ctx);
  CK(check_op(c, op, "imsrg_op_set_herm"));
  if (herm != 1 && herm != -1) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "herm must be +1 or -1");
  op->herm = herm;
  return IMSRG_OK;
}

imsrg_status imsrg_op_get_herm(imsrg_ctx* ctx, const imsrg_op* op, int32_t* herm) {
  CTX(ctx);
  CK(check_op(c, op, "imsrg_op_get_herm"));
  if (!herm) return IMSRG_ERR_INVALID_ARGUMENT;
  *herm = op->herm;
  return IMSRG_OK;
}

imsrg_status imsrg_op_upload_slab(imsrg_ctx* ctx, imsrg_op* op, const double* host) {
  CTX(ctx);
  CK(check_op(c, op, "imsrg_op_upload_slab"));
  if (!host) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "NULL host slab");
  return c->cuda(cudaMemcpyAsync(op->d, host, sizeof(double) * (size_t)c->L.slab, cudaMemcpyHostToDevice, c->stream),
                 "H2D slab");
}

imsrg_status imsrg_op_download_slab(imsrg_ctx* ctx, const imsrg_op* op, double* host) {
  CTX(ctx);
  CK(check_op(c, op, "imsrg_op_download_slab"));
  if (!host) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "NULL host slab");
  CK(c->cuda(cudaMemcpyAsync(host, op->d, sizeof(double) * (size_t)c->L.slab, cudaMemcpyDeviceToHost, c->stream),
             "D2H slab"));
  return c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
}

imsrg_status imsrg_op_upload(imsrg_ctx* ctx, imsrg_op* op, const double* const* gam, const double* fhh,
                             const double* fph, const double* fpp, double E0) {
  CTX(ctx);
  CK(check_op(c, op, "imsrg_op_upload"));
  const Layout& L = c->L;
  std::vector<double> h((size_t)L.slab);
  h[0] = E0;
  if ((L.A * L.A && !fhh) || (L.P * L.A && !fph) || (L.P * L.P && !fpp))
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "NULL one-body array");
  if (L.A) std::memcpy(&h[L.off_fhh], fhh, sizeof(double) * L.A * L.A);
  if (L.P) std::memcpy(&h[L.off_fpp], fpp, sizeof(double) * L.P * L.P);
  if (L.P * L.A) std::memcpy(&h[L.off_fph], fph, sizeof(double) * L.P * L.A);
  for (int k = 0; k < L.nblocks * 6; ++k) {
    const int64_t n = (int64_t)L.gn1[k] * L.gn2[k];
    if (!n) continue;
    if (!gam || !gam[k]) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "NULL pointer for a non-empty gam array");
    std::memcpy(&h[L.goff[k]], gam[k], sizeof(double) * n);
  }
  CK(c->cuda(cudaMemcpyAsync(op->d, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, c->stream), "H2D"));
  return c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
}

imsrg_status imsrg_op_download(imsrg_ctx* ctx, const imsrg_op* op, double* const* gam, double* fhh, double* fph,
                               double* fpp, double* E0) {
  CTX(ctx);
  CK(check_op(c, op, "imsrg_op_download"));
  const Layout& L = c->L;
  std::vector<double> h((size_t)L.slab);
  CK(c->cuda(cudaMemcpyAsync(h.data(), op->d, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream), "D2H"));
  CK(c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize"));
  if (E0) *E0 = h[0];
  if (fhh && L.A) std::memcpy(fhh, &h[L.off_fhh], sizeof(double) * L.A * L.A);
  if (fpp && L.P) std::memcpy(fpp, &h[L.off_fpp], sizeof(double) * L.P * L.P);
  if (fph && L.P * L.A) std::memcpy(fph, &h[L.off_fph], sizeof(double) * L.P * L.A);
  if (gam)
    for (int k = 0; k < L.nblocks * 6; ++k) {
      const int64_t n = (int64_t)L.gn1[k] * L.gn2[k];
      if (n && gam[k]) std::memcpy(gam[k], &h[L.goff[k]], sizeof(double) * n);
    }
  return IMSRG_OK;
}

imsrg_status imsrg_op_device_slab(imsrg_ctx* ctx, imsrg_op* op, double** dev) {
  CTX(ctx);
  CK(check_op(c, op, "imsrg_op_device_slab"));
  if (!dev) return IMSRG_ERR_INVALID_ARGUMENT;
  *dev = op->d;
  return IMSRG_OK;
}

imsrg_status imsrg_op_get_e0(imsrg_ctx* ctx, const imsrg_op* op, double* E0) {
  CTX(ctx);
  CK(check_op(c, op, "imsrg_op_get_e0"));
  if (!E0) return IMSRG_ERR_INVALID_ARGUMENT;
  CK(c->cuda(cudaMemcpyAsync(c->h_scalars, op->d, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "D2H E0"));
  CK(c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize"));
  *E0 = c->h_scalars[0];
  return IMSRG_OK;
}

imsrg_status imsrg_pinned_alloc(int64_t bytes, void** host_ptr) {
  if (!host_ptr || bytes <= 0) return IMSRG_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaMallocHost(host_ptr, (size_t)bytes);
  return e == cudaSuccess ? IMSRG_OK : IMSRG_ERR_OUT_OF_MEMORY;
}

imsrg_status imsrg_pinned_free(void* host_ptr) {
  if (host_ptr) cudaFreeHost(host_ptr);
  return IMSRG_OK;
}

imsrg_status imsrg_copy_sq_op(imsrg_ctx* ctx, const imsrg_op* H, imsrg_op* op) {
  CTX(ctx);
  CK(check_op(c, H, "imsrg_copy_sq_op"));
  CK(check_op(c, op, "imsrg_copy_sq_op"));
  op->herm = H->herm;
  return c->cuda(cudaMemcpyAsync(op->d, H->d, sizeof(double) * (size_t)c->L.slab, cudaMemcpyDeviceToDevice, c->stream),
                 "copy_sq_op");
}

imsrg_status imsrg_clear_sq_op(imsrg_ctx* ctx, imsrg_op* C) {
  CTX(ctx);
  CK(check_op(c, C, "imsrg_clear_sq_op"));
  return c->cuda(cudaMemsetAsync(C->d, 0, sizeof(double) * (size_t)c->L.slab, c->stream), "clear_sq_op");
}

imsrg_status imsrg_add_sq_op(imsrg_ctx* ctx, const imsrg_op* A, double ax, const imsrg_op* B, double bx,
                             imsrg_op* C) {
  CTX(ctx);
  CK(check_op(c, A, "imsrg_add_sq_op"));
  CK(check_op(c, B, "imsrg_add_sq_op"));
  CK(check_op(c, C, "imsrg_add_sq_op"));
  return c->axpby(A->d, ax, B->d, bx, C->d);
}

imsrg_status imsrg_scale_sq_op(imsrg_ctx* ctx, imsrg_op* A, double ax) {
  CTX(ctx);
  CK(check_op(c, A, "imsrg_scale_sq_op"));
  return c->axpby(A->d, ax, A->d, 0.0, A->d);
}

imsrg_status imsrg_mat_frob_norm(imsrg_ctx* ctx, const imsrg_op* op, double* out) {
  CTX(ctx);
  CK(check_op(c, op, "imsrg_mat_frob_norm"));
  if (!out) return IMSRG_ERR_INVALID_ARGUMENT;
  CK(c->frob_async(op->d, 1.0, 0));
  CK(c->read_scalars(1));
  *out = c->h_scalars[0];
  return IMSRG_OK;
}

imsrg_status imsrg_check_conversions(imsrg_ctx* ctx, const double* host_x, const float* host_y, int64_t n,
                                     float* out_f32, double* out_f64) {
  CTX(ctx);
  if (n < 0 || (n > 0 && (!host_x || !host_y || !out_f32 || !out_f64))) return IMSRG_ERR_INVALID_ARGUMENT;
  if (n == 0) return IMSRG_OK;
  void* d = nullptr;
  const size_t bx = sizeof(double) * (size_t)n, by = sizeof(float) * (size_t)n;
  CK(c->cuda(cudaMalloc(&d, bx + by + 2 * by + 2 * bx), "cudaMalloc(conversion check)"));
  // [x: n doubles | out_f64: 2n doubles | y: n floats | out_f32: 2n floats]
  double* dx = static_cast<double*>(d);
  double* dd = dx + n;
  float* dy = reinterpret_cast<float*>(dd + 2 * n);
  float* df = dy + n;
  imsrg_status st = c->cuda(cudaMemcpyAsync(dx, host_x, bx, cudaMemcpyHostToDevice, c->stream), "H2D x");
  if (st == IMSRG_OK) st = c->cuda(cudaMemcpyAsync(dy, host_y, by, cudaMemcpyHostToDevice, c->stream), "H2D y");
  if (st == IMSRG_OK) {
    k_convert_check<<<(int)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, c->stream>>>(dx, dy, n, df, dd);
    st = c->launched("k_convert_check");
  }
  if (st == IMSRG_OK) st = c->cuda(cudaMemcpyAsync(out_f32, df, 2 * by, cudaMemcpyDeviceToHost, c->stream), "D2H f32");
  if (st == IMSRG_OK) st = c->cuda(cudaMemcpyAsync(out_f64, dd, 2 * bx, cudaMemcpyDeviceToHost, c->stream), "D2H f64");
  if (st == IMSRG_OK) st = c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  cudaFree(d);
  return st;
}

imsrg_status imsrg_mbpt2(imsrg_ctx* ctx, const imsrg_op* H, double* out) {
  CTX(ctx);
  CK(check_op(c, H, "imsrg_mbpt2"));
  if (!out) return IMSRG_ERR_INVALID_ARGUMENT;
  k_mbpt2_partial<<<c->L.nblocks, 256, 0, c->stream>>>(c->D, H->d, H->herm, c->d_partial);
  CK(c->launched("k_mbpt2_partial"));
  k_sum<<<1, 1024, 0, c->stream>>>(c->d_partial, c->L.nblocks, c->d_scalars);
  CK(c->launched("k_sum"));
  CK(c->read_scalars(1));
  *out = c->h_scalars[0];
  return IMSRG_OK;
}

imsrg_status imsrg_cc_create(imsrg_ctx* ctx, int32_t kind, imsrg_cc** out) {
  CTX(ctx);
  if (!out || (kind != 0 && kind != 1)) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "kind must be 0 (CCX) or 1 (WCC)");
  *out = nullptr;
  imsrg_cc* cc = new (std::nothrow) imsrg_cc();
  if (!cc) return IMSRG_ERR_OUT_OF_MEMORY;
  cc->n = kind ? c->L.wcc_size : c->L.cc_size;
  cc->kind = kind;
  cc->owner = c;
  cc->herm = 1;
  const size_t bytes = sizeof(double) * (size_t)std::max<int64_t>(cc->n, 1);
  imsrg_status s = c->cuda(cudaMalloc(&cc->d, bytes), "cudaMalloc(cc)");
  if (s == IMSRG_OK) s = c->cuda(cudaMemsetAsync(cc->d, 0, bytes, c->stream), "memset(cc)");
  if (s != IMSRG_OK) {
    if (cc->d) cudaFree(cc->d);
    delete cc;
    return s;
  }
  *out = cc;
  return IMSRG_OK;
}

imsrg_status imsrg_cc_destroy(imsrg_ctx* ctx, imsrg_cc* cc) {
  CTX(ctx);
  if (!cc) return IMSRG_OK;
  if (cc->owner != c) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "cc matrix of another context");
  cudaStreamSynchronize(c->stream);
  cudaFree(cc->d);
  delete cc;
  return IMSRG_OK;
}

imsrg_status imsrg_cc_download(imsrg_ctx* ctx, const imsrg_cc* cc, double* host) {
  CTX(ctx);
  if (!cc || cc->owner != c || !host) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_cc_download");
  if (cc->n == 0) return IMSRG_OK;
  CK(c->cuda(cudaMemcpyAsync(host, cc->d, sizeof(double) * cc->n, cudaMemcpyDeviceToHost, c->stream), "D2H cc"));
  return c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
}

imsrg_status imsrg_calculate_cross_coupled(imsrg_ctx* ctx, const imsrg_op* HS, imsrg_cc* CCME) {
  CTX(ctx);
  CK(check_op(c, HS, "imsrg_calculate_cross_coupled"));
  CK(check_cc(c, CCME, 0, "imsrg_calculate_cross_coupled"));
  CCME->herm = HS->herm;
  return c->pandya(HS->d, HS->herm, CCME->d);
}

imsrg_status imsrg_commutator_110(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, double* out) {
  CTX(ctx);
  CK(check_op(c, L, "imsrg_commutator_110"));
  CK(check_op(c, R, "imsrg_commutator_110"));
  if (!out) return IMSRG_ERR_INVALID_ARGUMENT;
  CK(c->e0(L->d, L->herm, R->d, R->herm, nullptr, c->d_scalars));
  CK(c->read_scalars(2));
  *out = c->h_scalars[0];
  return IMSRG_OK;
}

imsrg_status imsrg_commutator_220(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, double* out) {
  CTX(ctx);
  CK(check_op(c, L, "imsrg_commutator_220"));
  CK(check_op(c, R, "imsrg_commutator_220"));
  if (!out) return IMSRG_ERR_INVALID_ARGUMENT;
  CK(c->e0(L->d, L->herm, R->d, R->herm, nullptr, c->d_scalars));
  CK(c->read_scalars(2));
  *out = c->h_scalars[1];
  return IMSRG_OK;
}

#define THREE_OPS(name)                  \
  CTX(ctx);                              \
  CK(check_op(c, L, name));              \
  CK(check_op(c, R, name));              \
  CK(check_op(c, RES, name));

imsrg_status imsrg_commutator_111(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES) {
  THREE_OPS("imsrg_commutator_111");
  return c->c111(L->d, L->herm, R->d, R->herm, RES->d);
}

imsrg_status imsrg_commutator_121(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES) {
  THREE_OPS("imsrg_commutator_121");
  return c->c121(L->d, L->herm, R->d, R->herm, RES->d, RES->herm);
}

imsrg_status imsrg_commutator_122(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES) {
  THREE_OPS("imsrg_commutator_122");
  return c->c122(L->d, L->herm, R->d, R->herm, RES->d, RES->herm);
}

imsrg_status imsrg_commutator_222_pp_hh(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES,
                                        imsrg_op* w1, imsrg_op* w2) {
  THREE_OPS("imsrg_commutator_222_pp_hh");
  CK(check_op(c, w1, "imsrg_commutator_222_pp_hh"));
  CK(check_op(c, w2, "imsrg_commutator_222_pp_hh"));
  return c->pphh(L->d, L->herm, R->d, R->herm, RES->d, w1->d, w2->d);
}

imsrg_status imsrg_commutator_221(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES,
                                  const imsrg_op* w1, const imsrg_op* w2) {
  THREE_OPS("imsrg_commutator_221");
  CK(check_op(c, w1, "imsrg_commutator_221"));
  CK(check_op(c, w2, "imsrg_commutator_221"));
  return c->c221(L->herm, R->herm, RES->d, RES->herm, w1->d, w2->d);
}

imsrg_status imsrg_commutator_222_ph(imsrg_ctx* ctx, const imsrg_cc* LCC, const imsrg_cc* RCC, imsrg_op* RES,
                                     imsrg_cc* WCC) {
  CTX(ctx);
  CK(check_cc(c, LCC, 0, "imsrg_commutator_222_ph"));
  CK(check_cc(c, RCC, 0, "imsrg_commutator_222_ph"));
  CK(check_cc(c, WCC, 1, "imsrg_commutator_222_ph"));
  CK(check_op(c, RES, "imsrg_commutator_222_ph"));
  return c->ph(LCC->d, LCC->herm, RCC->d, RCC->herm, RES->d, RES->herm, WCC->d);
}

imsrg_status imsrg_commutator(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES, int32_t flags) {
  THREE_OPS("imsrg_commutator");
  if (RES == L || RES == R) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "RES must not alias L or R");
  return c->commutator(L->d, L->herm, R->d, R->herm, RES->d, RES->herm, (flags & IMSRG_COMM_E0) != 0);
}

imsrg_status imsrg_build_gs_white(imsrg_ctx* ctx, const imsrg_op* H, imsrg_op* ETA) {
  CTX(ctx);
  CK(check_op(c, H, "imsrg_build_gs_white"));
  CK(check_op(c, ETA, "imsrg_build_gs_white"));
  if (H == ETA) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "ETA must not alias H");
  ETA->herm = -1;
  return c->white(H->d, H->herm, ETA->d);
}

imsrg_status imsrg_build_gs_atan(imsrg_ctx* ctx, const imsrg_op* H, imsrg_op* ETA) {
  CTX(ctx);
  CK(check_op(c, H, "imsrg_build_gs_atan"));
  CK(check_op(c, ETA, "imsrg_build_gs_atan"));
  if (H == ETA) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_build_gs_atan: ETA must differ from H");
  ETA->herm = -1;
  return c->atan_generator(H->d, H->herm, H->d, ETA->d);
}

imsrg_status imsrg_build_gs_atanxx(imsrg_ctx* ctx, const imsrg_op* Hold, const imsrg_op* H, imsrg_op* ETA) {
  CTX(ctx);
  CK(check_op(c, Hold, "imsrg_build_gs_atanxx"));
  CK(check_op(c, H, "imsrg_build_gs_atanxx"));
  CK(check_op(c, ETA, "imsrg_build_gs_atanxx"));
  if (ETA == H || ETA == Hold) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_build_gs_atanxx: ETA must differ");
  ETA->herm = -1;
  return c->atan_generator(Hold->d, Hold->herm, H->d, ETA->d);
}

imsrg_status imsrg_build_gs_w2(imsrg_ctx* ctx, const imsrg_op* H, imsrg_op* ETA) {
  CTX(ctx);
  CK(check_op(c, H, "imsrg_build_gs_w2"));
  CK(check_op(c, ETA, "imsrg_build_gs_w2"));
  if (H == ETA) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_build_gs_w2: ETA must differ from H");
  ETA->herm = -1;
  return c->w2_generator(H->d, H->herm, ETA->d);
}

imsrg_status imsrg_magnus_expand(imsrg_ctx* ctx, imsrg_op* DG, const imsrg_op* G, int32_t* used) {
  CTX(ctx);
  CK(check_op(c, DG, "imsrg_magnus_expand"));
  CK(check_op(c, G, "imsrg_magnus_expand"));
  int u = 0;
  imsrg_status s = c->magnus_expand(DG->d, DG->herm, G->d, G->herm, &u);
  if (used) *used = u;
  return s;
}

imsrg_status imsrg_euler_step(imsrg_ctx* ctx, imsrg_op* G, const imsrg_op* DG, double* s, double stp) {
  CTX(ctx);
  CK(check_op(c, G, "imsrg_euler_step"));
  CK(check_op(c, DG, "imsrg_euler_step"));
  CK(c->axpby(G->d, 1.0, DG->d, stp, G->d));
  if (s) *s += stp;
  return IMSRG_OK;
}

imsrg_status imsrg_bch_expand(imsrg_ctx* ctx, imsrg_op* HS, const imsrg_op* G, const imsrg_op* H, int32_t max_terms,
                              double conv, int32_t* terms_used) {
  CTX(ctx);
  CK(check_op(c, HS, "imsrg_bch_expand"));
  CK(check_op(c, G, "imsrg_bch_expand"));
  CK(check_op(c, H, "imsrg_bch_expand"));
  if (HS == G || HS == H) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "HS must not alias G or H");
  if (max_terms < 2) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "max_terms must be >= 2");
  HS->herm = H->herm;
  int t = 0;
  imsrg_status s = c->bch_expand(HS->d, G->d, G->herm, H->d, H->herm, max_terms, conv, &t);
  if (terms_used) *terms_used = t;
  return s;
}

imsrg_status imsrg_bch_expand_quads(imsrg_ctx* ctx, imsrg_op* HS, const imsrg_op* G, const imsrg_op* H,
                                    int32_t max_terms, double conv, int32_t* terms_used) {
  CTX(ctx);
  CK(check_op(c, HS, "imsrg_bch_expand_quads"));
  CK(check_op(c, G, "imsrg_bch_expand_quads"));
  CK(check_op(c, H, "imsrg_bch_expand_quads"));
  if (HS == G || HS == H) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "HS must not alias G or H");
  if (max_terms < 2) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "max_terms must be >= 2");
  HS->herm = H->herm;
  int t = 0;
  imsrg_status s = c->bch_expand(HS->d, G->d, G->herm, H->d, H->herm, max_terms, conv, &t, false, true);
  if (terms_used) *terms_used = t;
  return s;
}

imsrg_status imsrg_cr_expand(imsrg_ctx* ctx, imsrg_op* HS, const imsrg_op* G, const imsrg_op* H, int32_t max_terms,
                             double conv, int32_t* terms_used) {
  CTX(ctx);
  CK(check_op(c, HS, "imsrg_cr_expand"));
  CK(check_op(c, G, "imsrg_cr_expand"));
  CK(check_op(c, H, "imsrg_cr_expand"));
  if (HS == G || HS == H) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "HS must not alias G or H");
  if (max_terms < 2) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "max_terms must be >= 2");
  HS->herm = H->herm;
  int t = 0;
  imsrg_status s = c->bch_expand(HS->d, G->d, G->herm, H->d, H->herm, max_terms, conv, &t, true);
  if (terms_used) *terms_used = t;
  return s;
}

imsrg_status imsrg_magnus_step(imsrg_ctx* ctx, imsrg_op* HS, imsrg_op* G, imsrg_op* DG, const imsrg_op* H, double ds,
                               int32_t bch_max_terms, double bch_conv, int32_t use_graph, imsrg_step_info* info) {
  CTX(ctx);
  CK(check_op(c, HS, "imsrg_magnus_step"));
  CK(check_op(c, G, "imsrg_magnus_step"));
  CK(check_op(c, DG, "imsrg_magnus_step"));
  CK(check_op(c, H, "imsrg_magnus_step"));
  if (HS == G || HS == H || HS == DG || G == DG || G == H || DG == H)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "HS, G, DG and H must be distinct operators");
  if (bch_max_terms < 2) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "max_terms must be >= 2");
  if (!use_graph && !info) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "the eager step needs info");
  HS->herm = H->herm;
  DG->herm = -1;
  return c->magnus_step(HS->d, G->d, G->herm, DG->d, H->d, H->herm, ds, bch_max_terms, bch_conv, use_graph != 0,
                        info);
}

imsrg_status imsrg_magnus_step_host(imsrg_ctx* ctx, imsrg_op* HS, imsrg_op* G, imsrg_op* DG, imsrg_op* H,
                                    double* hs_host, double* g_host, double* dg_host, const double* h_host, double ds,
                                    int32_t bch_max_terms, double bch_conv, int32_t use_graph, imsrg_step_info* info) {
  CTX(ctx);
  CK(check_op(c, HS, "imsrg_magnus_step_host"));
  CK(check_op(c, G, "imsrg_magnus_step_host"));
  CK(check_op(c, DG, "imsrg_magnus_step_host"));
  CK(check_op(c, H, "imsrg_magnus_step_host"));
  if (HS == G || HS == H || HS == DG || G == DG || G == H || DG == H)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "HS, G, DG and H must be distinct operators");
  if (!hs_host || !g_host || !dg_host || !h_host)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_magnus_step_host: null host buffer");
  if (hs_host == g_host || hs_host == dg_host || g_host == dg_host)
    return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_magnus_step_host: the output buffers must be distinct");
  if (bch_max_terms < 2) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "max_terms must be >= 2");
  if (!info) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "imsrg_magnus_step_host needs info (it waits for the step)");
  HS->herm = H->herm;
  G->herm = -1;
  DG->herm = -1;
  const StepHostIO io{hs_host, g_host, dg_host, h_host};
  return c->magnus_step(HS->d, G->d, G->herm, DG->d, H->d, H->herm, ds, bch_max_terms, bch_conv, use_graph != 0,
                        info, &io);
}

imsrg_status imsrg_magnus_step_counters(imsrg_ctx* ctx, int64_t* commutators, int64_t* kernels, int64_t* steps,
                                        int64_t* unconverged) {
  CTX(ctx);
  if (!commutators || !kernels || !steps || !unconverged) return IMSRG_ERR_INVALID_ARGUMENT;
  return c->step_counters(commutators, kernels, steps, unconverged);
}

}  // extern "C"
