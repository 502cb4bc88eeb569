// Frobenius norm of a device operator for callers that cannot allocate GPU memory.
//
// Some callers may not call cudaMalloc at the point where they need this value: code
// running inside a host callback or a memory pool that forbids new allocations, a host
// program whose allocator owns all device memory, or a Fortran driver that hands the
// library only buffers it allocated itself.  This entry point uses no allocation of its
// own: its only scratch (one partial sum per operator segment) lives in the fixed
// device array below, which exists on every GPU that loads the library until the
// process exits.
#include <cuda_runtime.h>

#include "engine.h"
#include "kernels.h"

namespace {

constexpr int kNoAllocMaxSegments = IMSRG_NOALLOC_MAX_SEGMENTS;

// Scratch of imsrg_mat_frob_norm_noalloc: shared by every call on this device.
static __device__ __align__(256) double g_noalloc_partials[kNoAllocMaxSegments];

// Device address of the scratch array on the current device (the host-side symbol is only
// a stand-in).  Looked up on every call: the lookup is cheap, and an address cached across
// calls would go stale if the program reset the device (cudaDeviceReset) in between.
imsrg_status scratch_address(Ctx* c, double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
  if (e != cudaSuccess) return c->cuda(e, "cudaGetSymbolAddress(g_noalloc_partials)");
  *out = static_cast<double*>(p);
  return IMSRG_OK;
}

}  // namespace

extern "C" imsrg_status imsrg_mat_frob_norm_noalloc(imsrg_ctx* ctx, const double* dev_slab, double* dev_out,
                                                    void* stream) {
  if (!ctx) return IMSRG_ERR_INVALID_ARGUMENT;
  Ctx* c = reinterpret_cast<Ctx*>(ctx);
  if (c->device < 0) return c->fail(IMSRG_ERR_UNSUPPORTED, "host-only context (device < 0)");
  if (!dev_slab || !dev_out) return c->fail(IMSRG_ERR_INVALID_ARGUMENT, "NULL operator or output pointer");
  if (c->nseg > kNoAllocMaxSegments)
    return c->fail(IMSRG_ERR_UNSUPPORTED,
                   "operator has " + std::to_string(c->nseg) + " norm segments; imsrg_mat_frob_norm_noalloc supports at most " +
                       std::to_string(kNoAllocMaxSegments));
  const cudaError_t se = cudaSetDevice(c->device);
  if (se != cudaSuccess) return c->cuda(se, "cudaSetDevice");
  double* partials = nullptr;
  const imsrg_status st = scratch_address(c, &partials);
  if (st != IMSRG_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The context queues its work on its own non-blocking stream, which does not order itself
  // against the caller's stream: wait for what is queued there (it may still be writing the
  // operator), and make the context's later work wait for this call (it may overwrite the
  // operator while the norm still reads it).
  const bool other = (s != c->stream);
  if (other) {
    imsrg_status r = c->cuda(cudaEventRecord(c->ev_ext_in, c->stream), "cudaEventRecord");
    if (r == IMSRG_OK) r = c->cuda(cudaStreamWaitEvent(s, c->ev_ext_in, 0), "cudaStreamWaitEvent");
    if (r != IMSRG_OK) return r;
  }
  imsrg_status r;
  if (c->nseg == 0) {
    r = c->cuda(cudaMemsetAsync(dev_out, 0, sizeof(double), s), "memset(norm)");
  } else {
    // every partial the second stage reads is written by the first: nothing to clear
    imsrg::k_frob_partial<<<c->nseg, 256, 0, s>>>(dev_slab, c->d_seg_start, c->d_seg_len, c->d_seg_w, partials);
    r = c->launched("k_frob_partial");
    if (r == IMSRG_OK) {
      imsrg::k_sum_sqrt<<<1, 1024, 0, s>>>(partials, c->nseg, 1.0, dev_out);
      r = c->launched("k_sum_sqrt");
    }
  }
  if (r != IMSRG_OK || !other) return r;
  r = c->cuda(cudaEventRecord(c->ev_ext_out, s), "cudaEventRecord");
  if (r == IMSRG_OK) r = c->cuda(cudaStreamWaitEvent(c->stream, c->ev_ext_out, 0), "cudaStreamWaitEvent");
  return r;
}
