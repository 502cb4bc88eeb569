// Plan of the grouped particle-hole recoupling (recouple.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "dev.cuh"
#include "layout.h"

namespace imsrg {

constexpr int kRcThreads = 256;  // threads per CTA of the recoupling kernel
constexpr int kRcChunk = 16;   // quadruples of a group staged at a time
constexpr int kRcMaxU = 52;    // J' of both terms together (eMax <= 12: 2 x 26)
// shared memory per warp: X columns of the direct and exchange J' (2 x 32 int64), the chunk's
// j list and output prefix (2 x kRcChunk int), its staged (quadruple, J') values
constexpr int kRcWarpSlotBytes = 2 * 32 * 8 + 2 * kRcChunk * 4 + kRcChunk * kRcMaxU * 4;
constexpr int kRcMaxGroup = 0xFFFF;

// one (i, k, l) group: x = i | k << 16, y = l | nq << 16, z = first quadruple
struct __align__(16) RcGroup {
  int x, y, z, w;
};
// a run of groups of one triple (ji, jk, jl)
struct RcTask {
  int g0, ng, triple, pad;
};
// staged 6j blocks of one triple: nfl floats from table + off
struct __align__(16) RcTriple {
  int64_t off;
  int nfl;
  int16_t ji, jk, jl, nud, nue, pad0, pad1, pad2;
};

struct RecouplePlan {
  std::vector<RcGroup> groups;  // in task order
  std::vector<RcTask> tasks;    // one CTA each
  std::vector<RcTriple> triples;
  std::vector<float> table;
  int acc_off = 0;              // floats of shared memory before the per-warp slots
  size_t smem_bytes = 0;
};

std::string build_recouple_plan(const Layout& L, const std::vector<uint64_t>& quads, RecouplePlan& P);

struct RecoupleTraffic {
  int64_t x_reads, x_distinct, res_elems, aux_bytes;
};
RecoupleTraffic recouple_traffic(const Layout& L, const std::vector<uint64_t>& quads, const RecouplePlan& P);
void launch_recouple_g(const RecouplePlan& P, cudaStream_t st, const DevLayout& D, const RcTask* tasks,
                       const RcGroup* groups, const RcTriple* triples, const float* table, const uint64_t* quads,
                       const int* xcol, const float* X, double* RES);
// one thread per quadruple; min_blocks 4, 6 or 8 (launch-bounds variants)
void launch_recouple_q(int min_blocks, int grid, cudaStream_t st, const DevLayout& D, const uint64_t* quads,
                       int64_t nquads, const int* xcol, const float* X, double* RES);
std::vector<int> build_xcol(const Layout& L);
cudaError_t recouple_g_smem_attr(size_t smem);

}  // namespace imsrg
