// Plans of the tensor-core (split-BF16 tcgen05) path.
#pragma once
#include <cstdint>

namespace imsrg {

// tile shape of the split operand buffers: 128 rows of 64 K-contiguous bf16 per tile
constexpr int kTcTileRows = 128, kTcTileK = 64;

// term sign: bit 0 times herm(L), bit 1 times herm(R), bit 2 negative
enum TcSign : int { kSignHL = 1, kSignHR = 2, kSignNeg = 4 };

// one FP64 array whose columns become K-major rows of the split operand buffer
struct TcSplitOp {
  int64_t src_off;
  int src;       // 0 = L, 1 = R
  int rows, K;   // rows = columns of the stored array, K = its leading dimension
  int nkb;       // K blocks of 64
  int tile_base;
  int trans;     // 1: rows are the stored array's rows, element (r, k) at src[r + k*ld]
  int ld;        // leading dimension of the stored array when trans
};

struct TcTermDesc {
  int a_tile, b_tile;  // first tile of the A / B operand (row block 0, K block 0)
  int sign;            // TcSign
};

// C = sum over nterm (<= 4) terms of sign * A_t B_t^T, all terms with the same K blocks.
// With kseg > 0 the problem is one term whose K holds four segments of kseg elements (a
// multiple of 16): the products of segment j carry the sign t[j].sign.  xmask > 0 (FP32
// outputs): only the 32-row column segments whose bit is set in TcOut::xmask are stored, the
// bits of row block b (32 rows) at word xmask - 1 + b * ceil(N / 32) + column / 32.
struct TcProb {
  int64_t c_off;
  int M, N, nkb, nterm;
  int out_f32, c_id, ldc, kseg;
  int xmask, pad;
  TcTermDesc t[4];
};

// one output tile: rows m0 .. m0+127, columns n0 .. n0+w-1 of problem prob (n0 a multiple of
// 128, w a multiple of 16, 16 <= w <= the kernel's widest tile)
struct TcTile {
  int prob, m0, n0, w;
};

// width of the tile at column n0 of an N-column problem: the widest tile, or with narrow
// tiles the columns left rounded up to a multiple of 16
inline int tc_tile_width(int N, int n0, int wmax, bool narrow) {
  if (!narrow) return wmax;
  const int left = N - n0;
  return left >= wmax ? wmax : ((left + 15) / 16) * 16;
}

// Pandya chunk: elements [e0, e0 + n) of cross-coupled channel q (row-major, nph columns),
// with mnph = ceil(2^32 / nph) so that row = umulhi(e, mnph) (exact for e * nph < 2^32)
struct PandyaChunk {
  int q, e0, n;
  unsigned mnph;
};
// the two operators of one Pandya launch ([0] R, [1] L); per channel the first tiles of the
// K-concatenated operands A = [phiL | phiR | Ls | Rs] and B = [phiR | phiL | Rs | Ls] of the
// recoupling input, their K blocks and the segment length
struct PandyaOps {
  const double* op[2];
  int herm[2];
  const int* tile_a;
  const int* tile_b;
  const int* nkb;
  const int* seg;
};

// split chunk: a contiguous run of rows of one split operand
struct SplitChunk {
  int op;
  int r0, r1;
};

struct TcOut {
  double* f64[8];
  float* f32;   // out_f32 == 1
  float* f32b;  // out_f32 == 2
  float* w1f;   // when set: the W1 problems (c_id kOpW1) store FP32 here, same element offsets
  const unsigned* xmask;  // store masks of the problems with xmask > 0
};

}  // namespace imsrg
