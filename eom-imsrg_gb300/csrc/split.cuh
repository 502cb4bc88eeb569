// Operand slices of the tensor-core products: an FP32 value split into S terms of the
// operand type, x = h0 + h1 [+ h2], each term the rounding of what the previous ones left.
//   __nv_bfloat16 : round to nearest even (kind::f16 products), 64 values per 128-byte tile row
//   float (TF32)  : cvt.rna.tf32.f32 (10-bit mantissa, low 13 bits zero; kind::tf32 products),
//                   32 values per 128-byte tile row
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace imsrg {

template <typename T>
struct SplitElem;

template <>
struct SplitElem<__nv_bfloat16> {
  static constexpr int kPerRow = 64;
  __device__ static __forceinline__ __nv_bfloat16 take(float& rem) {
    const __nv_bfloat16 h = __float2bfloat16_rn(rem);
    rem -= __bfloat162float(h);
    return h;
  }
  __device__ static __forceinline__ __nv_bfloat16 neg(__nv_bfloat16 h) { return __hneg(h); }
};

template <>
struct SplitElem<float> {
  static constexpr int kPerRow = 32;
  __device__ static __forceinline__ float take(float& rem) {
    uint32_t t;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(rem));
    const float h = __uint_as_float(t);
    rem -= h;
    return h;
  }
  __device__ static __forceinline__ float neg(float h) { return -h; }
};

// element offset of (row r, k) of an operand whose tiles start at tile_base, nkb K blocks per
// row block, in the 128-row tiles of one slice
template <typename T>
__device__ __forceinline__ int64_t split_offset(int tile_base, int nkb, int r, int k) {
  constexpr int BKe = SplitElem<T>::kPerRow;
  return ((int64_t)(tile_base + (r >> 7) * nkb + k / BKe) * 128 + (r & 127)) * BKe + (k % BKe);
}

}  // namespace imsrg
