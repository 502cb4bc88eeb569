// White generator, operator algebra (axpy, Frobenius norm, MBPT2) -- FP64.
#include "dev.cuh"
#include "kernels.h"

namespace imsrg {

// twobody_monopole for all orbit pairs (src/basic_IMSRG.f90:2075-2090): mono[a*N+b]
__global__ void k_monopole(DevLayout D, const double* __restrict__ H, int hH, double* __restrict__ mono) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= D.N * D.N) return;
  const int a = t / D.N, b = t % D.N;
  const int ja = D.jj[a], jb = D.jj[b];
  double sm = 0.0;
  for (int JT = abs(ja - jb); JT <= ja + jb; JT += 2) sm += (JT + 1) * d_v_elem(D, H, hH, a, b, a, b, JT);
  mono[t] = sm / (ja + 1.0) / (jb + 1.0);
}

// build_gs_white one-body part (src/generators.f90:22-52); ETA is zeroed by the caller
__global__ void k_white_1b(DevLayout D, const double* __restrict__ H, int hH, double* __restrict__ ETA) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= D.n_ai) return;
  const int a = D.ai_a[w], i = D.ai_i[w];
  const int ak = D.parts[a], ik = D.holes[i];
  const int ji = D.jj[ik];
  double Eden = 0.0;
  for (int JT = 0; JT <= 2 * ji; JT += 2) Eden = Eden - (JT + 1) * d_v_elem(D, H, hH, ak, ik, ak, ik, JT);
  Eden = Eden / (ji + 1.0) / (ji + 1.0);
  Eden = Eden + H[D.off_fpp + a + (int64_t)a * D.P] - H[D.off_fhh + i + (int64_t)i * D.A];
  ETA[D.off_fph + a + (int64_t)i * D.P] = H[D.off_fph + a + (int64_t)i * D.P] / Eden;
}

// build_gs_white two-body part (src/generators.f90:56-104): blockIdx.y = channel
__global__ void k_white_2b(DevLayout D, const double* __restrict__ H, int hH, const double* __restrict__ mono,
                           double* __restrict__ ETA) {
  const int q = blockIdx.y;
  const int np = D.ncls[q * 3], nh = D.ncls[q * 3 + 2];
  const int64_t n = (int64_t)np * nh;
  const int64_t off = D.goff[q * 6 + 2];
  const int N = D.N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int JX = (int)(t / np), IX = (int)(t - (int64_t)JX * np);
    const int o1 = D.pair_off[q * 3] + IX, o2 = D.pair_off[q * 3 + 2] + JX;
    const int a = D.pair_a[o1], b = D.pair_b[o1], i = D.pair_a[o2], j = D.pair_b[o2];
    double Eden = 0.0;
    Eden = Eden + mono[a * N + b];
    Eden = Eden + mono[i * N + j];
    Eden = Eden - mono[a * N + i];
    Eden = Eden - mono[a * N + j];
    Eden = Eden - mono[i * N + b];
    Eden = Eden - mono[j * N + b];
    Eden = Eden + d_f_elem(D, H, hH, a, a) + d_f_elem(D, H, hH, b, b) - d_f_elem(D, H, hH, i, i) -
           d_f_elem(D, H, hH, j, j);
    ETA[off + t] = H[off + t] / Eden;
  }
}

// build_gs_atan / build_gs_atanxx one-body part (src/generators.f90:163-215, 271-323):
// eta = atan(2 N / Eden) * 0.5, numerators from Hnum, White denominators from Hden
__global__ void k_atan_1b(DevLayout D, const double* __restrict__ Hden, int hden, const double* __restrict__ Hnum,
                          double* __restrict__ ETA) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= D.n_ai) return;
  const int a = D.ai_a[w], i = D.ai_i[w];
  const int ak = D.parts[a], ik = D.holes[i];
  const int ji = D.jj[ik];
  double Eden = 0.0;
  for (int JT = 0; JT <= 2 * ji; JT += 2) Eden = Eden - (JT + 1) * d_v_elem(D, Hden, hden, ak, ik, ak, ik, JT);
  Eden = Eden / (ji + 1.0) / (ji + 1.0);
  Eden = Eden + Hden[D.off_fpp + a + (int64_t)a * D.P] - Hden[D.off_fhh + i + (int64_t)i * D.A];
  ETA[D.off_fph + a + (int64_t)i * D.P] = atan(2 * Hnum[D.off_fph + a + (int64_t)i * D.P] / Eden) * 0.5;
}

// two-body part (src/generators.f90:216-265, 324-373): blockIdx.y = channel
__global__ void k_atan_2b(DevLayout D, const double* __restrict__ Hden, int hden, const double* __restrict__ Hnum,
                          const double* __restrict__ mono, double* __restrict__ ETA) {
  const int q = blockIdx.y;
  const int np = D.ncls[q * 3], nh = D.ncls[q * 3 + 2];
  const int64_t n = (int64_t)np * nh;
  const int64_t off = D.goff[q * 6 + 2];
  const int N = D.N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int JX = (int)(t / np), IX = (int)(t - (int64_t)JX * np);
    const int o1 = D.pair_off[q * 3] + IX, o2 = D.pair_off[q * 3 + 2] + JX;
    const int a = D.pair_a[o1], b = D.pair_b[o1], i = D.pair_a[o2], j = D.pair_b[o2];
    double Eden = 0.0;
    Eden = Eden + mono[a * N + b];
    Eden = Eden + mono[i * N + j];
    Eden = Eden - mono[a * N + i];
    Eden = Eden - mono[a * N + j];
    Eden = Eden - mono[i * N + b];
    Eden = Eden - mono[j * N + b];
    Eden = Eden + d_f_elem(D, Hden, hden, a, a) + d_f_elem(D, Hden, hden, b, b) - d_f_elem(D, Hden, hden, i, i) -
           d_f_elem(D, Hden, hden, j, j);
    ETA[off + t] = 0.5 * atan(2 * Hnum[off + t] / Eden);
  }
}

// add_sq_op (src/basic_IMSRG.f90:3551-3579): C = ax*A + bx*B over the whole slab
__global__ void k_axpby(int64_t n, const double* __restrict__ A, double ax, const double* __restrict__ B, double bx,
                        double* __restrict__ C) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    C[e] = A[e] * ax + B[e] * bx;
}

// mat_frob_norm (src/basic_IMSRG.f90:4056-4087), stage 1: one partial per segment.
// Segments are host-made chunks of one array each, with weight 1 (square) or 2.
__global__ void k_frob_partial(const double* __restrict__ op, const int64_t* __restrict__ seg_start,
                               const int* __restrict__ seg_len, const int8_t* __restrict__ seg_w,
                               double* __restrict__ partial) {
  __shared__ double red[256];
  const int s = blockIdx.x;
  const double* x = op + seg_start[s];
  const int n = seg_len[s];
  double acc = 0.0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) acc += x[t] * x[t];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int k = blockDim.x >> 1; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[s] = red[0] * seg_w[s];
}

// stage 2: out = sqrt(sum of partials) (fixed order); optional scale (|cof| or coef)
// Y += a X over the norm segments (every element but E0; E0 too when with_e0) and the
// segments' weighted sums of X^2 (as k_frob_partial on X): one pass instead of two
__global__ void k_axpy_frob(double* __restrict__ Y, double a, const double* __restrict__ X,
                            const int64_t* __restrict__ seg_start, const int* __restrict__ seg_len,
                            const int8_t* __restrict__ seg_w, double* __restrict__ partial, int with_e0) {
  __shared__ double red[256];
  const int s = blockIdx.x;
  const int64_t o = seg_start[s];
  const int n = seg_len[s];
  if (s == 0 && threadIdx.x == 0 && with_e0) Y[0] += a * X[0];
  double acc = 0.0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const double x = X[o + t];
    Y[o + t] += a * x;
    acc += x * x;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int k = blockDim.x >> 1; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[s] = red[0] * seg_w[s];
}
__global__ void k_sum_sqrt(const double* __restrict__ partial, int n, double scale, double* __restrict__ out) {
  __shared__ double red[1024];
  double acc = 0.0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) acc += partial[t];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int k = blockDim.x >> 1; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sqrt(red[0]) * scale;
}

// mbpt2 (src/basic_IMSRG.f90:4165-4199): one block per channel, then a fixed-order sum
__global__ void k_mbpt2_partial(DevLayout D, const double* __restrict__ H, int hH, double* __restrict__ partial) {
  __shared__ double red[256];
  const int q = blockIdx.x;
  const int np = D.ncls[q * 3], nh = D.ncls[q * 3 + 2];
  const int64_t n = (int64_t)np * nh;
  const double* X = H + D.goff[q * 6 + 2];
  double acc = 0.0;
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) {
    const int JJ = (int)(t / np), II = (int)(t - (int64_t)JJ * np);
    const int o1 = D.pair_off[q * 3] + II, o2 = D.pair_off[q * 3 + 2] + JJ;
    const int i = D.pair_a[o1], j = D.pair_b[o1], k = D.pair_a[o2], l = D.pair_b[o2];
    const double eden = d_f_elem(D, H, hH, k, k) + d_f_elem(D, H, hH, l, l) - d_f_elem(D, H, hH, i, i) -
                        d_f_elem(D, H, hH, j, j);
    acc += X[t] * X[t] / eden;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int k = blockDim.x >> 1; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[q] = (D.lamJ[q] + 1.0) * red[0];
}

__global__ void k_sum(const double* __restrict__ partial, int n, double* __restrict__ out) {
  __shared__ double red[1024];
  double acc = 0.0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) acc += partial[t];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int k = blockDim.x >> 1; k > 0; k >>= 1) {
    if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// Self-check of the integer conversions of dev.cuh against the GPU's conversion
// instructions: out_f32 = [f64_to_f32(x) | __double2float_rn(x)], out_f64 = [f32_to_f64(y) |
// (double)y], n entries each.
__global__ void k_convert_check(const double* __restrict__ x, const float* __restrict__ y, int64_t n,
                                float* __restrict__ out_f32, double* __restrict__ out_f64) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    out_f32[t] = f64_to_f32(x[t]);
    out_f32[n + t] = __double2float_rn(x[t]);
    out_f64[t] = f32_to_f64(y[t]);
    out_f64[n + t] = (double)y[t];
  }
}

// zero the (start, length) run blockIdx.x of a slab
__global__ void k_zero_runs(double* __restrict__ x, const int64_t* __restrict__ runs) {
  const int64_t a = runs[2 * blockIdx.x], n = runs[2 * blockIdx.x + 1];
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) x[a + e] = 0.0;
}
__global__ void k_zero_runs_f(float* __restrict__ x, const int64_t* __restrict__ runs) {
  const int64_t a = runs[2 * blockIdx.x], n = runs[2 * blockIdx.x + 1];
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) x[a + e] = 0.0f;
}

}  // namespace imsrg
