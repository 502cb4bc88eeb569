// Tensor-core (tcgen05) split-BF16 path: placeholder until the kernels land.
#include "engine.h"

imsrg_status Ctx::tc_prepare(int) { return fail(IMSRG_ERR_UNSUPPORTED, "tensor-core path not built yet"); }
imsrg_status Ctx::tc_pphh(const double*, int, const double*, int, double*, double*) {
  return fail(IMSRG_ERR_UNSUPPORTED, "tensor-core path not built yet");
}
imsrg_status Ctx::tc_wcc(const double*, const double*, double*) {
  return fail(IMSRG_ERR_UNSUPPORTED, "tensor-core path not built yet");
}
void Ctx::tc_release() {}
