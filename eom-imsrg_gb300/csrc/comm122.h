// commutator_122 of the mixed path by pair-group sub-blocks (comm122.cu): the host plan and
// its launch.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "dev.cuh"
#include "layout.h"
#include "pair_groups.h"

namespace imsrg {

constexpr int kG122Threads = 256;
constexpr int kG122MaxElems = 4095;  // elements of one sub-block (the 20-bit division below)

// One group-pair sub-block (G1 <= G2) of channel q, everything the kernel needs about it.
struct __align__(16) G122Task {
  int eoff, pad;       // first code word of its elements in the element table
  int q;               // channel
  unsigned nn;         // block sizes n0 | n1 << 8 | n2 << 16 | n3 << 24 (bra: n0 n1, ket: n2 n3)
  int fb[4];           // offsets of the four blocks' f matrices in the (fL, fR) table
  int m0, m2, mb;      // ceil(2^20 / n) for n0, n2 and n0 n1: floor(e / n) = (e m) >> 20
  int flags;           // 1: G1 != G2, 2: both bra blocks equal, 4: both ket blocks equal
};

// A run of tasks for one warp: x = first task, y = count | lanes << 16 (lanes 0: four 8-lane
// groups, task k on group k mod 4; 1: the whole warp, one task after another).
// Code word of one element (x0 + n0 (x1 + n1 (x2 + n2 x3))) of a sub-block: its storage position
// in the upper triangle or rectangular array where the stored operators keep it (bits 0-27),
// swapped (bit 28: the element is herm times the stored one, and for G1 == G2 the element of
// the transposed position stores the result), the sign (bit 29) and size (bits 30-31: 1, sqrt 2,
// 2) of pre, V_A = pre x stored.
constexpr unsigned kG122IdxBits = 28;
struct G122Plan {
  std::vector<unsigned> codes;   // the element table: per task of `all`, its elements' code words
  std::vector<int64_t> elems;    // per task of `all`: elements of its sub-block
  std::vector<G122Task> all;     // every task, channel by channel
  // launch order for the current caps: the big tasks (one CTA each) first, then the warp tasks
  std::vector<G122Task> tasks;
  std::vector<int2> items;
  int nbig = 0;
  int tiny_cap = 64, warp_cap = 256;
  int nmax4 = 1;
  size_t smem_bytes = 0;         // per CTA
};

// the pair table and the task list (once per basis)
std::string build_g122_plan(const Layout& L, const PairGroups& G, G122Plan& P);
// the launch order for caps: tasks of at most tiny_cap elements on 8 lanes, at most warp_cap
// on a warp, larger ones on a CTA
std::string g122_partition(G122Plan& P, int tiny_cap, int warp_cap);
size_t g122_smem_bytes(int tiny_cap, int warp_cap, int nmax4);
cudaError_t g122_smem_attr(size_t smem);
cudaError_t g122_blocks_per_sm(size_t smem, int* n);  // resident CTAs of the 122 kernel per SM

// f(x, y) of L and R on every block, as (fL, fR) pairs; also clears the work counter
__global__ void k_comm122_fb2(DevLayout D, PairGroupsDev G, int nspb, const double* L, int hL, const double* R, int hR,
                              float2* FB, int* counter);
void launch_comm122(int grid, size_t smem, cudaStream_t st, const DevLayout& D, const G122Task* tasks,
                    const int2* items, int nitems, int nbig, int* counter, const unsigned* codes, int slice_f2, int sub_f2,
                    const double* L, int hL, const double* R, int hR, double* RES, int hRES, const float2* FB);

}  // namespace imsrg
