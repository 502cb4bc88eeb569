// Engine state behind the opaque C-ABI handles.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "dev.cuh"
#include "gemm.h"
#include "layout.h"
#include "tc.h"

namespace imsrg {
struct TcState;
}
struct StepGraph;
// The flow state of a step in the caller's pinned host memory (slab format): inputs G (Omega),
// DG (eta) and H, outputs HS, G and DG
struct StepHostIO {
  double* hs;
  double* g;
  double* dg;
  const double* h;
};
struct AdjointState;
struct TensorState;
struct imsrg_eom;
struct QuadState;
struct HFState;

// MAGNUS_EXPAND coefficients as the literals of src/IMSRG_MAGNUS.f90:646
constexpr double kMagnusCof[7] = {1.0, -0.5, .0833333333, 0.0, -0.00138888888, 0.0, 3.306878e-5};

// phases of one commutator for per-phase event timing (imsrg_profile_read)
enum Phase : int {
  kPhaseStart = 0,
  kPhasePandya = 1,
  kPhaseOneBody = 2,
  kPhase122 = 3,
  kPhasePphhSplit = 4,
  kPhasePphhGemm = 5,
  kPhasePphhSmall = 6,
  kPhasePphhUpdate = 7,
  kPhase221 = 8,
  kPhasePhGemm = 9,
  kPhaseRecouple = 10,
  kPhaseMirror = 11,
};

struct Ctx {
  imsrg::Layout L;
  imsrg::DevLayout D{};
  int device = 0;
  int precision = IMSRG_PREC_FP64;
  cudaStream_t stream = nullptr;
  std::string err;

  void* d_tables = nullptr;
  std::vector<imsrg::GemmProb> pphh_probs, wcc_probs;
  std::vector<imsrg::GemmTile> pphh_tiles, wcc_tiles;
  const imsrg::GemmProb* d_pphh_probs = nullptr;
  const imsrg::GemmTile* d_pphh_tiles = nullptr;
  const imsrg::GemmProb* d_wcc_probs = nullptr;
  const imsrg::GemmTile* d_wcc_tiles = nullptr;
  const int64_t* d_seg_start = nullptr;
  const int* d_seg_len = nullptr;
  const int8_t* d_seg_w = nullptr;
  int nseg = 0;
  double* d_partial = nullptr;
  int64_t partial_capacity = 0;  // entries of d_partial
  double* d_scalars = nullptr;
  double* h_scalars = nullptr;
  double* d_mono = nullptr;
  std::vector<int4> upd_tiles;
  const int4* d_upd_tiles = nullptr;
  // (start, length) runs of w1 / w2 that no 222_pp_hh product writes
  std::vector<int64_t> zero_runs_w1, zero_runs_w2;
  const int64_t* d_zero_runs_w1 = nullptr;
  const int64_t* d_zero_runs_w2 = nullptr;
  // commutator workspaces (w1, w2: sq_op shaped; LCC/RCC: CCX; WCC: rlen x rlen blocks)
  double *d_w1 = nullptr, *d_w2 = nullptr, *d_lcc = nullptr, *d_rcc = nullptr, *d_wcc = nullptr;
  // Magnus / BCH intermediates
  double *d_int1 = nullptr, *d_int2 = nullptr, *d_ad = nullptr;
  double* d_gen = nullptr;  // w2 generator workspace (3 slabs)
  imsrg::TcState* tc = nullptr;
  // limit of every bounded device wait of the tensor-core kernels (imsrg_set_wait_limit), and the
  // one-shot test switch that leaves one pipeline stage of the next GEMM launch unarmed
  unsigned long long tc_wait_ns = 2000000000ull;
  int tc_unarmed_next = 0;
  StepGraph* sg = nullptr;  // captured Magnus step (graph.cu)
  AdjointState* adj = nullptr;  // reverse-mode workspaces (adjoint.cu)
  HFState* hf = nullptr;        // Hartree-Fock tables (hf.cu)
  QuadState* qs = nullptr;      // quadrupole restoration of BCH_EXPAND (quads.cu)
  std::vector<double*> op_pool;  // slabs of destroyed operators, reused by imsrg_op_create
  // kernel launches issued (cumulative) and optional per-phase CUDA-event timing
  int64_t launches = 0;
  bool prof = false;
  std::vector<std::pair<int, cudaEvent_t>> prof_marks;
  std::vector<cudaEvent_t> prof_pool;
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
  // order a call on a caller's stream (imsrg_mat_frob_norm_noalloc) after the context's queued
  // work, and the context's later work after it
  cudaEvent_t ev_ext_in = nullptr, ev_ext_out = nullptr;
  void mark(int phase);

  ~Ctx();
  imsrg_status fail(imsrg_status code, const std::string& msg);
  imsrg_status cuda(cudaError_t e, const char* what);
  imsrg_status launched(const char* what);
  imsrg_status upload_tables();
  imsrg_status ensure_workspace();
  imsrg_status ensure_flow_workspace();

  imsrg_status pandya(const double* op, int herm, double* cc);
  imsrg_status e0(const double* L, int hL, const double* R, int hR, double* RES, double* out);
  imsrg_status c111(const double* L, int hL, const double* R, int hR, double* RES);
  imsrg_status c121(const double* L, int hL, const double* R, int hR, double* RES, int hRES);
  imsrg_status c122(const double* L, int hL, const double* R, int hR, double* RES, int hRES);
  imsrg_status pphh(const double* L, int hL, const double* R, int hR, double* RES, double* w1, double* w2);
  imsrg_status pphh_clear(double* w1, double* w2);
  imsrg_status pphh_accumulate(int hL, int hR, double* RES, const double* w1, const double* w2);
  imsrg_status c221(int hL, int hR, double* RES, int hRES, const double* w1, const double* w2);
  // the same on FP32 W1 / W2 (the mixed commutator's own workspaces, same element offsets)
  imsrg_status pphh_clear_f(float* w1, float* w2);
  imsrg_status c221_f(int hL, int hR, double* RES, int hRES, const float* w1, const float* w2);
  imsrg_status ensure_wcc();
  imsrg_status ph(const double* lcc, int hL, const double* rcc, int hR, double* RES, int hRES, double* wcc);
  imsrg_status commutator(const double* L, int hL, const double* R, int hR, double* RES, int hRES, bool with_e0);
  imsrg_status axpby(const double* A, double ax, const double* B, double bx, double* C);
  imsrg_status axpy_frob_async(double* Y, double a, const double* X, double scale, int slot, bool with_e0);
  imsrg_status frob_async(const double* op, double scale, int slot);
  imsrg_status read_scalars(int n);
  imsrg_status white(const double* H, int hH, double* ETA);
  imsrg_status atan_generator(const double* Hden, int hden, const double* Hnum, double* ETA);
  imsrg_status w2_generator(const double* H, int hH, double* ETA);
  imsrg_status magnus_expand(double* DG, int hDG, const double* G, int hG, int* used);
  // cr: CR_EXPAND's coefficients 1/n! (src/IMSRG_MAGNUS.f90:532-617) and no error after max_terms;
  // quads: BCH_EXPAND with quads = 'y' (restore_quadrupoles after every nested commutator)
  imsrg_status bch_expand(double* HS, const double* G, int hG, const double* H, int hH, int max_terms, double conv,
                          int* terms, bool cr = false, bool quads = false);
  imsrg_status quads_prepare();
  void quads_release();
  double* quads_int3();
  imsrg_status restore_quadrupoles(const double* X, int hX, const double* OM, int hOM, double* RES);

  // one Magnus step, eager or replayed from a CUDA graph (graph.cu)
  imsrg_status magnus_step(double* HS, double* G, int hG, double* DG, const double* H, int hH, double ds,
                           int max_terms, double conv, bool use_graph, imsrg_step_info* info,
                           const StepHostIO* hio = nullptr);
  imsrg_status graph_capture(double* HS, double* G, int hG, double* DG, const double* H, int hH, double ds,
                             int max_terms, double conv, const StepHostIO* hio);
  template <class F>
  imsrg_status capture_if(cudaGraphConditionalHandle h, F&& body);
  imsrg_status step_counters(int64_t* commutators, int64_t* kernels, int64_t* steps, int64_t* unconverged);
  imsrg_status graph_release();

  // reverse mode (FP64) of the commutator, the White generator and the slab inner product (adjoint.cu)
  imsrg_status adjoint_prepare();
  void adjoint_release();
  imsrg_status commutator_vjp(const double* L, int hL, const double* R, int hR, int hRES, bool with_e0,
                              const double* Cb, double* Lb, double* Rb);
  imsrg_status white_vjp(const double* H, int hH, const double* ETAb, double* Hb);
  imsrg_status dot(const double* A, const double* B, double* out);

  // rank-lambda tensor operators (tensor.cu)
  imsrg_status tensor_state(int rank, int dpar, TensorState** out);
  imsrg_status tensor_tc_prepare(TensorState& S);
  void tensor_release();
  imsrg_status tensor_commutator(TensorState& S, const double* L, int hL, const double* R, int hR, double* RES,
                                 int pieces);
  imsrg_status tensor_frob(TensorState& S, const double* op, double scale, int slot);
  imsrg_status bch_tensor(TensorState& S, const double* G, int hG, double* HS, int max_terms, double conv, int* terms);
  // perturbative triples after the flow (triples.cu)
  imsrg_status restore_triples(const double* H, const double* OM, double* e3, int64_t* items);
  // EOM-IMSRG ladder operators (eom.cu)
  imsrg_status eom_matvec(imsrg_eom& E, const double* H, const double* d_v, double* d_w);
  imsrg_status eom_matvec_host(imsrg_eom& E, const double* H, const double* v, double* w);
  imsrg_status eom_matvec_graph(imsrg_eom& E, const double* H);
  imsrg_status eom_lanczos(imsrg_eom& E, const double* H, int nev, double tol, int max_restarts, double* energies,
                           double* vectors, int32_t* matvecs, int32_t* restarts);

  // Hartree-Fock and normal ordering (hf.cu)
  imsrg_status hf_prepare();
  void hf_release();
  imsrg_status hf_mean_field(const double* op, int herm, std::vector<double>& M);
  imsrg_status hf_transform_2b(double* op, int herm, const double* coefs);
  imsrg_status hf_run(double* op, int herm, int mode, int max_iter, const double* coefs_in, double* coefs_out,
                      imsrg_hf_info* info);

  // tensor-core (split-BF16, tcgen05) path, gemm_tc.cu
  imsrg_status tc_prepare(int mode);
  imsrg_status tc_pphh(const double* L, int hL, const double* R, int hR, double* w1, double* w2);
  imsrg_status tc_wcc(const double* lcc, const double* rcc, double* wcc);
  imsrg_status tc_gemm(const imsrg::TcProb* probs, const imsrg::TcTile* tiles, int ntiles, imsrg::TcOut out, int hL,
                       int hR, int wmax);
  imsrg_status tc_error();
  imsrg_status tc_commutator(const double* L, int hL, const double* R, int hR, double* RES, int hRES, bool with_e0);
  void tc_release();
  imsrg_status tc_gemm_on(const CUtensorMap& map, int64_t slice_rows, const imsrg::TcProb* probs,
                          const imsrg::TcTile* tiles, int ntiles, imsrg::TcOut out, int hL, int hR, int wmax = 128);
  imsrg_status tc_encode_map(CUtensorMap* map, void* buf, int64_t total_rows);
  imsrg_status tc_split_on(const imsrg::TcSplitOp* ops, const imsrg::SplitChunk* chunks, int nchunks, const double* L,
                           const double* R, void* buf, int64_t slice_elems);
  int tc_slices() const;      // operand slices of the tensor-core path (0 before tc_prepare)
  int tc_tile_k() const;      // K values per 128-byte tile row of the operand slices (64 BF16, 32 TF32)
  int tc_elem_bytes() const;  // bytes per operand value (2 BF16, 4 TF32)
  int tc_kind() const;        // operand type of the slices (0 BF16, 1 TF32)
  imsrg_status tc_g122_partition(int tiny_cap, int small_cap);
  imsrg_status tc_set_tiles(const int* wmax, const bool* narrow, int order);
  imsrg_status tc_autotune(const double* L, int hL, const double* R, int hR, double* RES, imsrg_tune_info* info);
};

#define CK_TC(expr)              \
  do {                           \
    imsrg_status _s = (expr);    \
    if (_s != IMSRG_OK) return _s; \
  } while (0)

struct imsrg_op {
  double* d = nullptr;
  int herm = 1;
  Ctx* owner = nullptr;
};

struct imsrg_cc {
  double* d = nullptr;
  int64_t n = 0;
  int kind = 0;
  int herm = 1;
  Ctx* owner = nullptr;
};
