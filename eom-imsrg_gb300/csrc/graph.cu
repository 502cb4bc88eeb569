// One step of the Magnus flow captured as a CUDA graph.
//
// The step is the loop body of magnus_decouple (src/IMSRG_MAGNUS.f90:47-110):
//   MAGNUS_EXPAND(DG, G)        dOmega = sum_i cof_i ad_Omega^(i-1)(eta)      (:620-691)
//   euler_step(G, DG)           Omega += ds * dOmega                          (:754-764)
//   BCH_EXPAND(HS, G, H)        H(s) = sum_n ad_Omega^n(H) / n!               (:149-234)
//   build_gs_white(HS, DG)      eta(s)                                        (src/generators.f90:4-106)
//   mbpt2(HS)                   convergence measure                           (src/basic_IMSRG.f90:4165-4199)
// The reference leaves both series early on host-side norm tests.  Here every nested
// commutator of a series is the body of a conditional IF node; a one-thread kernel at the
// end of each body applies the same test to the norm on the device and sets the condition
// of the next body, so a whole step replays with one graph launch and no host round trip.
// The kernels, their order and their arguments are those of the eager drivers in
// engine.cu, so graph and eager steps give bit-identical operators.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "../../include/imsrg_gb300.h"
#include "engine.h"
#include "kernels.h"

using namespace imsrg;

// device-side state of the current step plus counters accumulated over all steps
struct StepState {
  double advals[8];
  double fullnorm;
  double mbpt2;
  double e0;
  int qq;
  int magnus_used;
  int bch_terms;
  int bch_converged;
  long long tot_commutators;
  long long tot_kernels;
  long long tot_unconverged;
  long long tot_steps;
};

struct StepGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t side = nullptr;
  // copy branches of a step with host I/O (captured into the graph) and their fork / join events
  cudaStream_t cp[3] = {nullptr, nullptr, nullptr};
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  StepHostIO hio{};
  StepState* d_state = nullptr;
  StepState* h_state = nullptr;
  // key of the captured step
  double* HS = nullptr;
  double* G = nullptr;
  double* DG = nullptr;
  const double* H = nullptr;
  int hH = 0, hG = 0, precision = -1, max_terms = 0;
  double ds = 0, conv = 0;
};

namespace {

__device__ __forceinline__ int magnus_qq(double cof) { return (fabs(cof) > (double)1e-6f) ? 1 : 2; }

// Opens the Magnus series (the tests before the loop of MAGNUS_EXPAND) and decides the
// first nested commutator.  scal[0] = ||DG||, scal[1] = ||G||.
__global__ void k_magnus_begin(const double* scal, StepState* st, cudaGraphConditionalHandle first, double conv,
                               double cof1) {
  st->magnus_used = 0;
  st->bch_terms = 0;
  st->bch_converged = 0;
  for (int i = 0; i < 8; ++i) st->advals[i] = 0.0;
  st->advals[1] = scal[0];
  st->fullnorm = scal[1];
  st->qq = 1;
  if (st->fullnorm < (double)1e-9f) {
    cudaGraphSetConditional(first, 0);
    return;
  }
  const double adnorm = st->advals[2 - st->qq];
  st->qq = magnus_qq(cof1);
  cudaGraphSetConditional(first, fabs(adnorm / st->fullnorm) < conv ? 0u : 1u);
}

// End of Magnus term i: records ||term|| (scal[0], already times |cof_i|) and decides term i+1.
__global__ void k_magnus_next(int i, const double* scal, StepState* st, cudaGraphConditionalHandle next, int has_next,
                              double conv, double cof_next, int body_kernels) {
  st->advals[i] = scal[0];
  st->magnus_used += 1;
  st->tot_commutators += 1;
  st->tot_kernels += body_kernels;
  if (!has_next) return;
  const double adnorm = st->advals[i + 1 - st->qq];
  st->qq = magnus_qq(cof_next);
  cudaGraphSetConditional(next, fabs(adnorm / st->fullnorm) < conv ? 0u : 1u);
}

// End of BCH term iw: scal[0] = coef * ||ad^(iw-1)||; the series stops below conv.
__global__ void k_bch_next(int iw, const double* scal, StepState* st, cudaGraphConditionalHandle next, int has_next,
                           double conv, int body_kernels) {
  st->bch_terms = iw - 1;
  st->tot_commutators += 1;
  st->tot_kernels += body_kernels;
  if (scal[0] < conv) {
    st->bch_converged = 1;
    if (has_next) cudaGraphSetConditional(next, 0);
    return;
  }
  if (has_next) cudaGraphSetConditional(next, 1);
}

__global__ void k_step_end(const double* HS, StepState* st, int fixed_kernels) {
  st->e0 = HS[0];
  st->tot_kernels += fixed_kernels;
  st->tot_steps += 1;
  if (!st->bch_converged) st->tot_unconverged += 1;
}

}  // namespace

imsrg_status Ctx::graph_release() {
  if (!sg) return IMSRG_OK;
  if (sg->exec) cudaGraphExecDestroy(sg->exec);
  if (sg->graph) cudaGraphDestroy(sg->graph);
  if (sg->side) cudaStreamDestroy(sg->side);
  for (cudaStream_t c : sg->cp)
    if (c) cudaStreamDestroy(c);
  for (cudaEvent_t e : sg->ev)
    if (e) cudaEventDestroy(e);
  if (sg->d_state) cudaFree(sg->d_state);
  if (sg->h_state) cudaFreeHost(sg->h_state);
  delete sg;
  sg = nullptr;
  return IMSRG_OK;
}

// Appends an IF node with condition `h` to the graph captured on `stream` and captures
// body() into it on the side stream.
template <class F>
imsrg_status Ctx::capture_if(cudaGraphConditionalHandle h, F&& body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  CK_TC(cuda(cudaStreamGetCaptureInfo(stream, &cs, nullptr, &g, &deps, nullptr, &nd), "cudaStreamGetCaptureInfo"));
  if (cs != cudaStreamCaptureStatusActive) return fail(IMSRG_ERR_CUDA, "graph capture is not active");
  cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeIf;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  CK_TC(cuda(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p), "cudaGraphAddNode(conditional)"));
  CK_TC(cuda(cudaStreamUpdateCaptureDependencies(stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies),
             "cudaStreamUpdateCaptureDependencies"));
  cudaGraph_t bodyg = p.conditional.phGraph_out[0];
  CK_TC(cuda(cudaStreamBeginCaptureToGraph(sg->side, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
             "cudaStreamBeginCaptureToGraph"));
  cudaStream_t main = stream;
  stream = sg->side;
  imsrg_status s = body();
  stream = main;
  cudaGraph_t out = nullptr;
  imsrg_status e = cuda(cudaStreamEndCapture(sg->side, &out), "cudaStreamEndCapture(body)");
  return s != IMSRG_OK ? s : e;
}

// Captures the whole step (see the file comment); the eager drivers are
// Ctx::magnus_expand, Ctx::axpby (euler_step), Ctx::bch_expand, Ctx::white and imsrg_mbpt2.
imsrg_status Ctx::graph_capture(double* HS, double* G, int hG, double* DG, const double* H, int hH, double ds,
                                int max_terms, double conv, const StepHostIO* hio) {
  const size_t sb = sizeof(double) * (size_t)L.slab;
  const double mconv = (double)1e-6f;
  const int hDG = -1;
  const int nmag = 6;                   // nested commutators i = 2..7 of MAGNUS_EXPAND
  const int nbch = max_terms - 1;       // iw = 2..max_terms of BCH_EXPAND
  std::vector<cudaGraphConditionalHandle> hm(nmag), hb(nbch);
  cudaGraph_t g = nullptr;
  CK_TC(cuda(cudaGraphCreate(&g, 0), "cudaGraphCreate"));
  for (int i = 0; i < nmag; ++i)
    CK_TC(cuda(cudaGraphConditionalHandleCreate(&hm[i], g, 0, cudaGraphCondAssignDefault), "conditional handle"));
  for (int i = 0; i < nbch; ++i)
    CK_TC(cuda(cudaGraphConditionalHandleCreate(&hb[i], g, i == 0 ? 1u : 0u, cudaGraphCondAssignDefault),
               "conditional handle"));
  const bool prof_was = prof;
  prof = false;
  const int64_t l_start = launches;
  imsrg_status s = cuda(cudaStreamBeginCaptureToGraph(stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
                        "cudaStreamBeginCaptureToGraph");
  int64_t fixed = 0;
  // with host I/O the copies are nodes of the graph: Omega and eta up first; H0 up on a side
  // branch joined before BCH_EXPAND (it overlaps MAGNUS_EXPAND); Omega down on a side branch
  // once euler_step has finished it (it overlaps BCH_EXPAND); H(s) down beside the generator
  // and MBPT(2); eta down last
  cudaStream_t* cp = sg->cp;
  cudaEvent_t* ev = sg->ev;
  auto fork = [&](cudaEvent_t e, cudaStream_t to) -> imsrg_status {
    CK_TC(cuda(cudaEventRecord(e, stream), "cudaEventRecord(fork)"));
    return cuda(cudaStreamWaitEvent(to, e, 0), "cudaStreamWaitEvent(fork)");
  };
  auto run = [&]() -> imsrg_status {
    if (hio) {
      CK_TC(cuda(cudaMemcpyAsync(G, hio->g, sb, cudaMemcpyHostToDevice, stream), "H2D Omega"));
      CK_TC(cuda(cudaMemcpyAsync(DG, hio->dg, sb, cudaMemcpyHostToDevice, stream), "H2D eta"));
      CK_TC(fork(ev[0], cp[0]));
      CK_TC(cuda(cudaMemcpyAsync(const_cast<double*>(H), hio->h, sb, cudaMemcpyHostToDevice, cp[0]), "H2D H"));
      CK_TC(cuda(cudaEventRecord(ev[1], cp[0]), "cudaEventRecord(H up)"));
    }
    // ---- MAGNUS_EXPAND
    int64_t l0 = launches;
    CK_TC(frob_async(DG, 1.0, 0));
    CK_TC(frob_async(G, 1.0, 1));
    k_magnus_begin<<<1, 1, 0, stream>>>(d_scalars, sg->d_state, hm[0], mconv, kMagnusCof[1]);
    CK_TC(launched("k_magnus_begin"));
    fixed += launches - l0;
    for (int i = 2; i <= 7; ++i) {
      const double cof = kMagnusCof[i - 1];
      // the same alternating buffers as Ctx::magnus_expand
      const double* ad = (i == 2) ? DG : ((i & 1) ? d_int2 : d_ad);
      double* out = (i & 1) ? d_ad : d_int2;
      CK_TC(capture_if(hm[i - 2], [&]() -> imsrg_status {
        const int64_t b0 = launches;
        CK_TC(commutator(G, hG, ad, hDG, out, hDG, false));
        CK_TC(axpy_frob_async(DG, cof, out, std::fabs(cof), 0, false));
        const int body = (int)(launches - b0) + 1;
        const bool has_next = i < 7;
        k_magnus_next<<<1, 1, 0, stream>>>(i, d_scalars, sg->d_state, has_next ? hm[i - 1] : hm[0], has_next ? 1 : 0,
                                           mconv, has_next ? kMagnusCof[i] : 0.0, body);
        return launched("k_magnus_next");
      }));
    }
    // ---- euler_step
    l0 = launches;
    CK_TC(axpby(G, 1.0, DG, ds, G));
    if (hio) {
      CK_TC(fork(ev[2], cp[1]));
      CK_TC(cuda(cudaMemcpyAsync(hio->g, G, sb, cudaMemcpyDeviceToHost, cp[1]), "D2H Omega"));
      CK_TC(cuda(cudaEventRecord(ev[3], cp[1]), "cudaEventRecord(Omega down)"));
      CK_TC(cuda(cudaStreamWaitEvent(stream, ev[1], 0), "cudaStreamWaitEvent(H up)"));
    }
    // ---- BCH_EXPAND
    CK_TC(cuda(cudaMemcpyAsync(HS, H, sb, cudaMemcpyDeviceToDevice, stream), "copy HS"));
    fixed += launches - l0;
    double coef = 1.0;
    for (int iw = 2; iw <= max_terms; ++iw) {
      coef = coef / (iw - 1.0);
      const double c = coef;
      // the same alternating buffers as Ctx::bch_expand
      const double* ad = (iw == 2) ? H : ((iw & 1) ? d_int2 : d_ad);
      double* out = (iw & 1) ? d_ad : d_int2;
      CK_TC(capture_if(hb[iw - 2], [&]() -> imsrg_status {
        const int64_t b0 = launches;
        CK_TC(commutator(G, hG, ad, hH, out, hH, true));
        CK_TC(axpy_frob_async(HS, c, out, c, 0, true));
        const int body = (int)(launches - b0) + 1;
        const bool has_next = iw < max_terms;
        k_bch_next<<<1, 1, 0, stream>>>(iw, d_scalars, sg->d_state, has_next ? hb[iw - 1] : hb[0], has_next ? 1 : 0,
                                        conv, body);
        return launched("k_bch_next");
      }));
    }
    if (hio) {
      CK_TC(fork(ev[4], cp[2]));
      CK_TC(cuda(cudaMemcpyAsync(hio->hs, HS, sb, cudaMemcpyDeviceToHost, cp[2]), "D2H H(s)"));
      CK_TC(cuda(cudaEventRecord(ev[5], cp[2]), "cudaEventRecord(H(s) down)"));
    }
    // ---- generator and MBPT(2) of the new H(s)
    l0 = launches;
    CK_TC(white(HS, hH, DG));
    k_mbpt2_partial<<<L.nblocks, 256, 0, stream>>>(D, HS, hH, d_partial);
    CK_TC(launched("k_mbpt2_partial"));
    k_sum<<<1, 1024, 0, stream>>>(d_partial, L.nblocks, &sg->d_state->mbpt2);
    CK_TC(launched("k_sum"));
    fixed += launches - l0 + 1;
    k_step_end<<<1, 1, 0, stream>>>(HS, sg->d_state, (int)fixed);
    CK_TC(launched("k_step_end"));
    if (hio) {
      CK_TC(cuda(cudaMemcpyAsync(hio->dg, DG, sb, cudaMemcpyDeviceToHost, stream), "D2H eta"));
      CK_TC(cuda(cudaStreamWaitEvent(stream, ev[3], 0), "cudaStreamWaitEvent(Omega down)"));
      CK_TC(cuda(cudaStreamWaitEvent(stream, ev[5], 0), "cudaStreamWaitEvent(H(s) down)"));
    }
    return IMSRG_OK;
  };
  if (s == IMSRG_OK) s = run();
  cudaGraph_t out = nullptr;
  imsrg_status e = cuda(cudaStreamEndCapture(stream, &out), "cudaStreamEndCapture");
  prof = prof_was;
  launches = l_start;  // capture issues no work; replays are counted from the device counters
  if (s == IMSRG_OK) s = e;
  if (s == IMSRG_OK) s = cuda(cudaGraphInstantiate(&sg->exec, g, 0), "cudaGraphInstantiate");
  if (s != IMSRG_OK) {
    cudaGetLastError();
    cudaGraphDestroy(g);
    sg->exec = nullptr;
    return s;
  }
  sg->graph = g;
  return IMSRG_OK;
}

imsrg_status Ctx::magnus_step(double* HS, double* G, int hG, double* DG, const double* H, int hH, double ds,
                              int max_terms, double conv, bool use_graph, imsrg_step_info* info,
                              const StepHostIO* hio) {
  CK_TC(ensure_workspace());
  CK_TC(ensure_flow_workspace());
  if (precision == IMSRG_PREC_FP64 && L.cc_size) CK_TC(ensure_wcc());
  if (!sg) {
    sg = new StepGraph();
    CK_TC(cuda(cudaMalloc(&sg->d_state, sizeof(StepState)), "cudaMalloc(step state)"));
    CK_TC(cuda(cudaMemsetAsync(sg->d_state, 0, sizeof(StepState), stream), "memset(step state)"));
    CK_TC(cuda(cudaMallocHost(&sg->h_state, sizeof(StepState)), "cudaMallocHost(step state)"));
    CK_TC(cuda(cudaStreamCreateWithFlags(&sg->side, cudaStreamNonBlocking), "cudaStreamCreate(side)"));
    for (cudaStream_t& c : sg->cp) CK_TC(cuda(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking), "cudaStreamCreate(copy)"));
    for (cudaEvent_t& e : sg->ev) CK_TC(cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate"));
  }
  const size_t sbytes = sizeof(double) * (size_t)L.slab;
  int rebuilt = 0;
  if (!use_graph) {
    // the eager drivers, with the reference's host-side tests (host I/O as plain copies)
    if (hio) {
      CK_TC(cuda(cudaMemcpyAsync(G, hio->g, sbytes, cudaMemcpyHostToDevice, stream), "H2D Omega"));
      CK_TC(cuda(cudaMemcpyAsync(DG, hio->dg, sbytes, cudaMemcpyHostToDevice, stream), "H2D eta"));
      CK_TC(cuda(cudaMemcpyAsync(const_cast<double*>(H), hio->h, sbytes, cudaMemcpyHostToDevice, stream), "H2D H"));
    }
    int used = 0, terms = 0;
    CK_TC(magnus_expand(DG, -1, G, hG, &used));
    CK_TC(axpby(G, 1.0, DG, ds, G));
    imsrg_status sb = bch_expand(HS, G, hG, H, hH, max_terms, conv, &terms);
    if (sb != IMSRG_OK && sb != IMSRG_ERR_NOT_CONVERGED) return sb;
    CK_TC(white(HS, hH, DG));
    k_mbpt2_partial<<<L.nblocks, 256, 0, stream>>>(D, HS, hH, d_partial);
    CK_TC(launched("k_mbpt2_partial"));
    k_sum<<<1, 1024, 0, stream>>>(d_partial, L.nblocks, d_scalars);
    CK_TC(launched("k_sum"));
    CK_TC(read_scalars(1));
    const double e2 = h_scalars[0];
    if (hio) {
      CK_TC(cuda(cudaMemcpyAsync(hio->hs, HS, sbytes, cudaMemcpyDeviceToHost, stream), "D2H H(s)"));
      CK_TC(cuda(cudaMemcpyAsync(hio->g, G, sbytes, cudaMemcpyDeviceToHost, stream), "D2H Omega"));
      CK_TC(cuda(cudaMemcpyAsync(hio->dg, DG, sbytes, cudaMemcpyDeviceToHost, stream), "D2H eta"));
    }
    double e0 = 0;
    CK_TC(cuda(cudaMemcpyAsync(h_scalars, HS, sizeof(double), cudaMemcpyDeviceToHost, stream), "D2H E0"));
    CK_TC(cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize"));
    e0 = h_scalars[0];
    if (info) {
      info->E0 = e0;
      info->mbpt2 = e2;
      info->magnus_terms = used;
      info->bch_terms = terms;
      info->bch_converged = sb == IMSRG_OK ? 1 : 0;
      info->graph_rebuilt = 0;
    }
    CK_TC(tc_error());
    if (sb != IMSRG_OK) return fail(IMSRG_ERR_NOT_CONVERGED, "BCH series did not converge within max_terms");
    return IMSRG_OK;
  }
  const StepHostIO none{};
  const StepHostIO& io = hio ? *hio : none;
  const bool same = sg->exec && sg->HS == HS && sg->G == G && sg->DG == DG && sg->H == H && sg->hH == hH &&
                    sg->hG == hG && sg->ds == ds && sg->max_terms == max_terms && sg->conv == conv &&
                    sg->precision == precision && sg->hio.hs == io.hs && sg->hio.g == io.g && sg->hio.dg == io.dg &&
                    sg->hio.h == io.h;
  if (!same) {
    if (sg->exec) cudaGraphExecDestroy(sg->exec);
    if (sg->graph) cudaGraphDestroy(sg->graph);
    sg->exec = nullptr;
    sg->graph = nullptr;
    CK_TC(cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize"));
    CK_TC(graph_capture(HS, G, hG, DG, H, hH, ds, max_terms, conv, hio));
    sg->HS = HS; sg->G = G; sg->DG = DG; sg->H = H; sg->hH = hH; sg->hG = hG; sg->hio = io;
    sg->ds = ds; sg->max_terms = max_terms; sg->conv = conv; sg->precision = precision;
    rebuilt = 1;
  }
  CK_TC(cuda(cudaGraphLaunch(sg->exec, stream), "cudaGraphLaunch"));
  if (!info) return IMSRG_OK;
  CK_TC(cuda(cudaMemcpyAsync(sg->h_state, sg->d_state, sizeof(StepState), cudaMemcpyDeviceToHost, stream),
          "D2H step state"));
  CK_TC(cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize"));
  CK_TC(tc_error());
  const StepState& st = *sg->h_state;
  info->E0 = st.e0;
  info->mbpt2 = st.mbpt2;
  info->magnus_terms = st.magnus_used;
  info->bch_terms = st.bch_terms;
  info->bch_converged = st.bch_converged;
  info->graph_rebuilt = rebuilt;
  if (!st.bch_converged) return fail(IMSRG_ERR_NOT_CONVERGED, "BCH series did not converge within max_terms");
  return IMSRG_OK;
}

imsrg_status Ctx::step_counters(int64_t* commutators, int64_t* kernels, int64_t* steps, int64_t* unconverged) {
  if (!sg) {
    *commutators = *kernels = *steps = *unconverged = 0;
    return IMSRG_OK;
  }
  CK_TC(cuda(cudaMemcpyAsync(sg->h_state, sg->d_state, sizeof(StepState), cudaMemcpyDeviceToHost, stream),
          "D2H step state"));
  CK_TC(cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize"));
  *commutators = sg->h_state->tot_commutators;
  *kernels = sg->h_state->tot_kernels;
  *steps = sg->h_state->tot_steps;
  *unconverged = sg->h_state->tot_unconverged;
  return tc_error();
}
