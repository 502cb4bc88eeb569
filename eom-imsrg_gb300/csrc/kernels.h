// Kernel declarations shared by the engine translation unit.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

#include "dev.cuh"
#include "pair_groups.h"
#include "gemm.h"
#include "tc.h"

namespace imsrg {

__global__ void k_pandya(DevLayout D, const double* op, int herm, double* cc);
__global__ void k_comm122(DevLayout D, const double* L, int hL, const double* R, int hR, double* RES, int hRES);
__global__ void k_pphh_update(DevLayout D, double* RES, const double* w1, const double* w2, double pm);
__global__ void k_comm222ph(DevLayout D, const double* WCC, int hL, int hR, double* RES, int hRES);
__global__ void k_comm111(DevLayout D, const double* L, int hL, const double* R, int hR, double* RES);
__global__ void k_comm121(DevLayout D, const double* L, int hL, const double* R, int hR, double* RES, int hRES);
__global__ void k_comm221(DevLayout D, int pm, double* RES, int hRES, const double* w1, const double* w2);
__global__ void k_e0_partial(DevLayout D, const double* L, int hL, const double* R, int hR, double* partial);
__global__ void k_e0_final(DevLayout D, const double* partial, double* RES, double* out);
__global__ void k_pphh_update_tiled(DevLayout D, const int4* tiles, double* RES, const double* w1, const double* w2,
                                    double pm);
__global__ void k_comm111f(DevLayout D, const double* L, int hL, const double* R, int hR, double* RES);
__global__ void k_comm221f(DevLayout D, int pm, double* RES, int hRES, const float* w1, const float* w2);

__global__ void k_monopole(DevLayout D, const double* H, int hH, double* mono);
__global__ void k_white_1b(DevLayout D, const double* H, int hH, double* ETA);
__global__ void k_white_2b(DevLayout D, const double* H, int hH, const double* mono, double* ETA);
__global__ void k_atan_1b(DevLayout D, const double* Hden, int hden, const double* Hnum, double* ETA);
__global__ void k_atan_2b(DevLayout D, const double* Hden, int hden, const double* Hnum, const double* mono,
                          double* ETA);
__global__ void k_axpby(int64_t n, const double* A, double ax, const double* B, double bx, double* C);
__global__ void k_frob_partial(const double* op, const int64_t* seg_start, const int* seg_len, const int8_t* seg_w,
                               double* partial);
__global__ void k_axpy_frob(double* Y, double a, const double* X, const int64_t* seg_start, const int* seg_len,
                            const int8_t* seg_w, double* partial, int with_e0);
__global__ void k_sum_sqrt(const double* partial, int n, double scale, double* out);
__global__ void k_mbpt2_partial(DevLayout D, const double* H, int hH, double* partial);
__global__ void k_sum(const double* partial, int n, double* out);
__global__ void k_zero_runs(double* x, const int64_t* runs);
__global__ void k_zero_runs_f(float* x, const int64_t* runs);
__global__ void k_convert_check(const double* x, const float* y, int64_t n, float* out_f32, double* out_f64);

__global__ void k_gemm_fp64(const GemmProb* probs, const GemmTile* tiles, GemmOperands ops);

// mixed-precision companions (kernels_mixed.cu)
void launch_pandya_tc(int S, int kind, int nchunks, cudaStream_t stream, const DevLayout& D, const PandyaChunk* chunks,
                      const PandyaOps& ops, void* buf, int64_t slice_elems, const int* swap_row);
__global__ void k_pphh_update_mirror_f(DevLayout D, const int4* tiles, double* RES, const float* w1, const float* w2,
                                       float pm, int herm);

}  // namespace imsrg
