// Particle-hole recoupling of the mixed path (recouple.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "dev.cuh"
#include "layout.h"

namespace imsrg {

// The X column offset of every pair (a, b) at every J' = 2h, [(a * N + b) * NJ + h]
// (-1 where (a, b) is not in the cross-coupled channel of J')
std::vector<int> build_xcol(const Layout& L);

// The X elements the recoupling reads, as store masks for the X product's epilogue: per
// cross-coupled channel q (rlen rows and columns) and 32-row block b, one bit per column,
// word mask_off[q] + b * ceil(rlen / 32) + column / 32 (mask_off[q] = -1 for an empty channel).
std::vector<unsigned> build_x_read_mask(const Layout& L, const std::vector<uint64_t>& quads, std::vector<int>& mask_off);

struct RecoupleTraffic {
  int64_t x_reads, x_distinct, res_elems, aux_bytes;
};
// the X elements the recoupling reads (each once, counted from the quadruple list), the RES
// elements it adds into, and the bytes of its quadruple list and index tables
RecoupleTraffic recouple_traffic(const Layout& L, const std::vector<uint64_t>& quads);

// one thread per quadruple; min_blocks 4, 6 or 8 (launch-bounds variants)
void launch_recouple_q(int min_blocks, int grid, cudaStream_t st, const DevLayout& D, const uint64_t* quads,
                       int64_t nquads, const int* xcol, const float* X, double* RES);

}  // namespace imsrg
