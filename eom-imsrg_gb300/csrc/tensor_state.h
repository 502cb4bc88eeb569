// Device state of a (rank, dpar) tensor layout and the C-ABI tensor operator handle, shared by
// the tensor commutator (tensor.cu) and the EOM ladder operators (eom.cu).
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include <vector>

#include "engine.h"
#include "gemm.h"
#include "tc.h"
#include "tensor.h"

using imsrg::DevTLayout;
using imsrg::ElemSegs;
using imsrg::ExcBlock;
using imsrg::GemmProb;
using imsrg::GemmTile;
using imsrg::SplitChunk;
using imsrg::TcProb;
using imsrg::TcSplitOp;
using imsrg::TcTile;
using imsrg::TLayout;

// pieces flag of Ctx::tensor_commutator: recouple every nonzero Wx / Wy element of TS_222_ph
// (the EOM product) instead of those above 1e-6 (TS_commutator_222_ph)
constexpr int kTensorExactPh = 512;
// pieces flag: R is an excitation operator (fph and (pp,hh) / (hh,pp) elements only) and only
// the fph and (pp,hh) / (hh,pp) elements of RES are computed (the rest of RES is undefined);
// implies kTensorExactPh; its ladder and particle-hole products run in FP64, or as FP32 SIMT
// GEMMs in the mixed modes
constexpr int kTensorExcitation = 1024;

// output slot of the second product of a tensor ladder problem (TcOut::f64 index)
constexpr int kTensorOpW3 = 7;

// device state of one (rank, dpar) layout
struct TensorState {
  TLayout T;
  DevTLayout DT{};
  void* tables = nullptr;
  const GemmProb* pphh_p = nullptr;
  const GemmTile* pphh_t = nullptr;
  int n_pphh_t = 0;
  // excitation mode: the ladder terms with a (pp,hh) / (hh,pp) R operand and the output arrays
  const GemmProb* exc_p = nullptr;
  const GemmTile* exc_t = nullptr;
  int n_exc_t = 0;
  ElemSegs exc_segs;
  int64_t exc_n2 = 0;
  // excitation-mode particle-hole products: per cross-coupled channel the (particle, hole) and
  // (hole, particle) rows (host offsets, device lists) and per tensor block the packed GEMMs
  std::vector<int> pe_off, hp_off;
  const int* d_pe = nullptr;
  const int* d_hp = nullptr;
  // ... batched over the blocks: ExcBlock table, prefix counts of the Pandya and scatter
  // elements, the grouped GEMM, and the CCR / CCX / Wx / Wy buffers (allocated on first use)
  const ExcBlock* x_blk = nullptr;
  const int64_t* x_pre_p = nullptr;
  const int64_t* x_pre_s = nullptr;
  const GemmProb* x_p = nullptr;
  const GemmTile* x_t = nullptr;
  int x_nblk = 0, x_n_t = 0;
  int64_t x_np = 0, x_ns = 0, x_sizes[4] = {0, 0, 0, 0};
  double* x_buf[4] = {nullptr, nullptr, nullptr, nullptr};
  // per cross-coupled block: GEMM problems (Wx, Wy) and their tile range
  const GemmProb* cb_p = nullptr;
  const GemmTile* cb_t = nullptr;
  std::vector<int> cb_tile_start, cb_tile_n;
  const int64_t* seg_start = nullptr;
  const int* seg_len = nullptr;
  const int8_t* seg_w = nullptr;
  int nseg = 0;
  double *w1 = nullptr, *w2 = nullptr;           // tensor-shaped ladder intermediates
  double *ccx = nullptr, *ccr = nullptr;         // cross-coupled tensor blocks
  double *wx = nullptr, *wy = nullptr;           // recoupling products
  double *bch_a = nullptr, *bch_b = nullptr;     // BCH_TENSOR terms
  // split-BF16 tensor-core form of the ladder's products through pp pairs (mixed modes):
  // one single-term problem per product, the first product of a (block, class pair) into
  // w1, the second into w3; the products through hh pairs (K = nhh) stay FP64 into w2
  int tc_S = 0, tc_kind = 0;  // slices and operand type the tensor-core plan was built for
  void* tc_buf = nullptr;
  int64_t tc_slice_rows = 0, tc_slice_elems = 0;
  CUtensorMap tc_map;
  void* tc_tables = nullptr;
  const TcSplitOp* tc_ops = nullptr;
  const SplitChunk* tc_chunks = nullptr;
  const TcProb* tc_probs = nullptr;
  const TcTile* tc_tiles = nullptr;
  const GemmProb* hh_p = nullptr;
  const GemmTile* hh_t = nullptr;
  int tc_nchunks = 0, tc_ntiles = 0, n_hh_t = 0;
  double* w3 = nullptr;
  // particle-hole products on the same tensor cores: the cross-coupled L of every channel is
  // split once per commutator (LCC rows, K = nph); per cross-coupled tensor block, CCR and CCX
  // are split into shared regions of the buffer and Wx = -LCC(qa) CCR, Wy = CCX LCC(qb)^T run
  // as single-term problems
  int ph_lcc_nchunks = 0;
  std::vector<int> ph_chunk_start, ph_chunk_n, ph_tile_start, ph_tile_n;  // per block
};

struct imsrg_tensor {
  double* d = nullptr;
  int herm = 1;
  TensorState* ts = nullptr;
  Ctx* owner = nullptr;
};
