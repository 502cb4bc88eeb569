/*
 * imsrg_gb300.h -- C ABI of the GB300 IMSRG(2) commutator engine.
 *
 * Drop-in for the hot path of EOM-IMSRG: the two-body-truncated commutator
 * (src/commutators.f90, src/cross_coupled.f90), the White generator
 * (src/generators.f90) and the Magnus / BCH loop (src/IMSRG_MAGNUS.f90).
 * Each entry point below names the Fortran routine it replaces.
 *
 * Conventions
 *  - Every function returns an imsrg_status (0 = IMSRG_OK); none aborts the process.
 *    imsrg_last_error() describes the last failure on a context.
 *  - Operators live in device memory, owned by the library.  Their content is the
 *    reference's type(sq_op) flattened as the "sq_op slab" (FP64, column-major,
 *    full square storage):
 *        [E0][fhh A*A][fpp P*P][fph P*A][for q=1..nblocks, g=1..6: gam(g) of block q]
 *    with gam(1..6) = pppp, ppph, pphh, phph, hhhh, phhh.  Block q, its pair lists
 *    and the pair order are those of allocate_blocks (src/basic_IMSRG.f90:521-685).
 *  - Orbit indices in this header are 0-based (Fortran index - 1).
 *  - All work on one context is ordered on that context's CUDA stream; calls that
 *    return host values synchronize it.  A context is thread-compatible, not
 *    thread-safe: serialize calls on one context.
 */
#ifndef IMSRG_GB300_H
#define IMSRG_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t imsrg_status;
#define IMSRG_OK 0
#define IMSRG_ERR_INVALID_ARGUMENT 1
#define IMSRG_ERR_CUDA 2
#define IMSRG_ERR_OUT_OF_MEMORY 3
#define IMSRG_ERR_NOT_CONVERGED 4
#define IMSRG_ERR_MISMATCH 5
#define IMSRG_ERR_UNSUPPORTED 6
#define IMSRG_ERR_TIMEOUT 7 /* a bounded device wait ran out (the kernel stopped, the context stays usable) */

/* arithmetic of the channel contractions (pp/hh ladders and cross-coupled GEMM) */
#define IMSRG_PREC_FP64 0    /* plain FP64 (DFMA) */
#define IMSRG_PREC_BF16X3 1  /* 2-slice split-BF16 operands, 3 products, FP32 accumulate (tcgen05) */
#define IMSRG_PREC_BF16X6 2  /* 3-slice split-BF16 operands, 6 products, FP32 accumulate (tcgen05) */
#define IMSRG_PREC_TF32X3 3  /* TF32-compensated: each FP32 operand = TF32 hi + TF32 lo, 3 products
                                (hi.hi, hi.lo, lo.hi), FP32 accumulate (tcgen05 kind::tf32) */

/* flags of imsrg_commutator */
#define IMSRG_COMM_E0 1      /* also assign RES%E0 = commutator_110 + commutator_220 */

typedef struct imsrg_ctx imsrg_ctx;
typedef struct imsrg_op imsrg_op;
typedef struct imsrg_cc imsrg_cc;

/* The fields of type(spd) the engine needs (src/basic_IMSRG.f90:25-37). */
typedef struct imsrg_basis {
  int32_t norbits;
  const int32_t* nn;
  const int32_t* ll;
  const int32_t* jj;   /* 2j */
  const int32_t* itzp; /* 2tz */
  const int32_t* con;  /* 1 hole, 0 particle */
  int32_t eMax, lMax;
  double hw;
  int32_t Aprot, Aneut;
} imsrg_basis;

/* ---- context: basis, channel layout, index maps, 6j table (read_sp_basis + store_6j +
 *      allocate_blocks + allocate_CCMAT, src/basic_IMSRG.f90:192-382, 521-685, 2227-2332;
 *      src/cross_coupled.f90:61-177).  device < 0 makes a host-only context that answers
 *      the layout queries and imsrg_synthetic_hamiltonian without touching a GPU; every
 *      other call on it returns IMSRG_ERR_UNSUPPORTED. */
imsrg_status imsrg_ctx_create(const imsrg_basis* basis, int32_t device, imsrg_ctx** out);
imsrg_status imsrg_ctx_destroy(imsrg_ctx* ctx);
const char* imsrg_last_error(const imsrg_ctx* ctx);
imsrg_status imsrg_ctx_sizes(const imsrg_ctx* ctx, int64_t* slab, int64_t* cc, int64_t* wcc, int32_t* nblocks,
                             int32_t* ncc);
/* per block: 2J, parity, Tz, npp, nph, nhh (sq_block%lam, %npp, %nph, %nhh) */
imsrg_status imsrg_block_info(const imsrg_ctx* ctx, int32_t* lamJ, int32_t* lamP, int32_t* lamT, int32_t* npp,
                              int32_t* nph, int32_t* nhh);
/* pair list qn(cls+1)%Y of block q as 0-based orbit pairs out[2k], out[2k+1] */
imsrg_status imsrg_block_pairs(const imsrg_ctx* ctx, int32_t q, int32_t cls, int32_t* out);
/* per cross-coupled block: rlen, nph, 2J (cc_mat%rlen, %nph, %Jval) */
imsrg_status imsrg_cc_info(const imsrg_ctx* ctx, int32_t* rlen, int32_t* nph, int32_t* J);
imsrg_status imsrg_set_precision(imsrg_ctx* ctx, int32_t mode);
/* Waits for the context's queued work.  Returns IMSRG_ERR_TIMEOUT when a bounded device wait
 * of a tensor-core kernel ran out since the last call (the reference STOPs where a loop cannot
 * finish, src/IMSRG_MAGNUS.f90:232; here the kernel records a code, stops its other roles,
 * waits for its own copies in flight, frees its tensor memory and returns). */
imsrg_status imsrg_synchronize(imsrg_ctx* ctx);
/* Limit of every bounded device wait of the tensor-core kernels, in nanoseconds (default
 * 2 s; 0 restores the default).  No counterpart in the reference. */
imsrg_status imsrg_set_wait_limit(imsrg_ctx* ctx, int64_t nanoseconds);
/* Test switch, off by default (no counterpart in the reference): with enable != 0 the next
 * tensor-core GEMM launch of this context leaves its first pipeline stage unarmed -- no copy
 * is issued for it and nothing arrives on its barrier -- so the MMA warp's wait on it runs out
 * after the wait limit and imsrg_synchronize reports IMSRG_ERR_TIMEOUT.  The switch resets
 * after that one launch.  For testing the failure path only. */
imsrg_status imsrg_test_unarmed_stage(imsrg_ctx* ctx, int32_t enable);
/* The traffic of the mixed particle-hole recoupling kernel on this basis, counted exactly
 * from its orbit quadruples (no counterpart in the reference): X elements read and how many of
 * them are distinct (FP32), RES elements read-modified-written (FP64), and the bytes of its own
 * index data and 6j blocks.  For roofline figures.  IMSRG_ERR_UNSUPPORTED in FP64 mode. */
imsrg_status imsrg_recouple_traffic(imsrg_ctx* ctx, int64_t* x_reads, int64_t* x_distinct, int64_t* res_elems,
                                    int64_t* aux_bytes);
/* The library's launch-configuration autotuner (no counterpart in the reference, which has
 * no GPU path).  In a mixed mode it times one commutator [L, R] into RES per candidate on
 * this basis and keeps the fastest: the size caps that send the commutator_122 sub-blocks to
 * 8-lane groups, warps or CTAs; the particle-hole recoupling kernel (by orbit groups, or one
 * thread per orbit quadruple with its occupancy variant and CTA count); then, jointly, the tile
 * shape of the persistent tcgen05 GEMM
 * (widest output tile 128 or 256 columns, and whether the last column tile of a problem is only
 * as wide as its columns need, in steps of 16), its tile order, and whether the ladder and the
 * particle-hole products share one launch.  The result of a commutator
 * does not depend on these choices.  A captured Magnus-step graph is dropped and re-captured
 * by the next step.  IMSRG_ERR_UNSUPPORTED in FP64 mode. */
typedef struct {
  int32_t tiny_cap, small_cap; /* sub-blocks up to tiny_cap elements: 8 lanes; up to small_cap: a warp */
  int32_t recouple_ctas;       /* CTAs of the recoupling kernel */
  int32_t gemm_order;          /* 0: tiles with the longest K first, 1: problem order */
  int32_t gemm_wmax;           /* widest output tile of the ladder launch (of the merged launch): 128 or 256 */
  int32_t gemm_narrow;         /* 1: narrow last column tiles (multiples of 16 columns) in that launch */
  double ms_before, ms_after;  /* one commutator before and after tuning */
  int32_t recouple_kind;       /* 1: one thread per orbit quadruple (the only recoupling kernel; other values are rejected) */
  int32_t recouple_min_blocks; /* launch-bounds variant of the recoupling kernel (4, 6 or 8 CTAs per SM) */
  int32_t gemm_merged;         /* 1: ladder and particle-hole products in one launch, 0: two launches */
  int32_t gemm_wmax_x;         /* two launches: widest tile of the particle-hole (X) launch (0: as gemm_wmax) */
  int32_t gemm_narrow_x;       /* two launches: narrow last tiles in the X launch */
} imsrg_tune_info;
imsrg_status imsrg_autotune(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES,
                            imsrg_tune_info* info);
/* Applies a configuration (for instance one that imsrg_autotune reported on an earlier run of
 * this basis) without timing anything; ms_before / ms_after are ignored.  Mixed modes only. */
imsrg_status imsrg_set_tuning(imsrg_ctx* ctx, const imsrg_tune_info* cfg);

/* ---- instrumentation (no reference counterpart: the reference only prints wall time,
 *      print_time, src/basic_IMSRG.f90:152-169) */
/* kernel launches issued on this context so far */
imsrg_status imsrg_launch_count(imsrg_ctx* ctx, int64_t* count);
/* CUDA-event timer on the context's stream: begin, then end returns elapsed ms */
imsrg_status imsrg_timer_begin(imsrg_ctx* ctx);
imsrg_status imsrg_timer_end(imsrg_ctx* ctx, float* ms);
/* per-phase event timing of imsrg_commutator; phases: 1 Pandya, 2 one-body (110/220,
 * 111, 121), 3 122, 4 ladder operand split, 5 ladder GEMM, 6 small-K ladder GEMM,
 * 7 ladder accumulation (in a mixed mode it runs last and also writes the square arrays'
 * lower triangles), 8 221, 9 cross-coupled GEMM, 10 6j recoupling, 11 mirror of the square
 * arrays' lower triangles (no longer a separate pass; kept for the index layout) */
#define IMSRG_NUM_PHASES 12
imsrg_status imsrg_profile_phases(imsrg_ctx* ctx, int32_t enable);
imsrg_status imsrg_profile_read(imsrg_ctx* ctx, float* ms_per_phase, int32_t* count_per_phase);

/* ---- operators: allocate_blocks / duplicate_sq_op (src/basic_IMSRG.f90:521, 2797) */
imsrg_status imsrg_op_create(imsrg_ctx* ctx, int32_t herm, imsrg_op** out);
imsrg_status imsrg_op_destroy(imsrg_ctx* ctx, imsrg_op* op);
imsrg_status imsrg_op_set_herm(imsrg_ctx* ctx, imsrg_op* op, int32_t herm);
imsrg_status imsrg_op_get_herm(imsrg_ctx* ctx, const imsrg_op* op, int32_t* herm);
/* Per-array transfer: gam[q*6+g] points at the contiguous column-major array
 * op%mat(q+1)%gam(g+1)%X (c_loc in Fortran); NULL is allowed for empty arrays. */
imsrg_status imsrg_op_upload(imsrg_ctx* ctx, imsrg_op* op, const double* const* gam, const double* fhh,
                             const double* fph, const double* fpp, double E0);
imsrg_status imsrg_op_download(imsrg_ctx* ctx, const imsrg_op* op, double* const* gam, double* fhh, double* fph,
                               double* fpp, double* E0);
/* whole-slab transfer from / to host memory (pinned memory gives full bandwidth) */
imsrg_status imsrg_op_upload_slab(imsrg_ctx* ctx, imsrg_op* op, const double* host_slab);
imsrg_status imsrg_op_download_slab(imsrg_ctx* ctx, const imsrg_op* op, double* host_slab);
/* device-resident slab (for device-to-device interop, e.g. torch tensors) */
imsrg_status imsrg_op_device_slab(imsrg_ctx* ctx, imsrg_op* op, double** dev_slab);
imsrg_status imsrg_op_get_e0(imsrg_ctx* ctx, const imsrg_op* op, double* E0);
imsrg_status imsrg_pinned_alloc(int64_t bytes, void** host_ptr);
imsrg_status imsrg_pinned_free(void* host_ptr);

/* ---- operator algebra (src/basic_IMSRG.f90) */
imsrg_status imsrg_copy_sq_op(imsrg_ctx* ctx, const imsrg_op* H, imsrg_op* op);                       /* :3005 */
imsrg_status imsrg_clear_sq_op(imsrg_ctx* ctx, imsrg_op* C);                                          /* :3638 */
imsrg_status imsrg_add_sq_op(imsrg_ctx* ctx, const imsrg_op* A, double ax, const imsrg_op* B, double bx,
                             imsrg_op* C);                                                            /* :3551 */
imsrg_status imsrg_scale_sq_op(imsrg_ctx* ctx, imsrg_op* A, double ax);                               /* :3610 */
imsrg_status imsrg_mat_frob_norm(imsrg_ctx* ctx, const imsrg_op* op, double* out);                    /* :4056 */
imsrg_status imsrg_mbpt2(imsrg_ctx* ctx, const imsrg_op* H, double* out);                             /* :4165 */
/* Self-check of the integer FP64 <-> FP32 conversions that the mixed-precision kernels use
 * (round to nearest even; NaN, Inf, overflow and FP32 subnormals as IEEE 754 defines them),
 * against the GPU's own conversion instructions.  No counterpart in the reference (its
 * path is FP64 throughout).  For n inputs: out_f32 = [integer(host_x) | hardware(host_x)]
 * (2n floats), out_f64 = [integer(host_y) | hardware(host_y)] (2n doubles).  Synchronous;
 * allocates device scratch for the call. */
imsrg_status imsrg_check_conversions(imsrg_ctx* ctx, const double* host_x, const float* host_y, int64_t n,
                                     float* out_f32, double* out_f64);

/* Frobenius norm for callers that cannot allocate GPU memory.  No counterpart in the
 * reference.  Same value as imsrg_mat_frob_norm, but for code that must not call
 * cudaMalloc when it needs the norm (an allocator that owns all device memory, a
 * callback or pool that forbids new allocations, a host driver that only passes its own
 * buffers): the call allocates nothing and frees nothing.  dev_slab is any device sq_op
 * slab of this context's layout, dev_out one device double, stream a cudaStream_t
 * (NULL = legacy default stream); the call is asynchronous on that stream.  It is ordered
 * after every call already queued on the context (which may still be writing dev_slab),
 * and the context's later calls wait for it.
 * Scratch is one static device array of IMSRG_NOALLOC_MAX_SEGMENTS doubles (64 KiB) that
 * every GPU loading the library keeps until exit; operators with more norm segments
 * (one per 65536 elements of each array) get IMSRG_ERR_UNSUPPORTED.  Each call looks up
 * the array's device address (cudaGetSymbolAddress); the first call on a device also loads
 * the library's device code there and should come before any stream capture.  All calls
 * share the array: calls that overlap on the GPU (on streams with no ordering between
 * them, from several contexts or threads) race on it. */
#define IMSRG_NOALLOC_MAX_SEGMENTS 8192
imsrg_status imsrg_mat_frob_norm_noalloc(imsrg_ctx* ctx, const double* dev_slab, double* dev_out, void* stream);

/* ---- cross-coupled matrices: type(cc_mat) (src/cross_coupled.f90:11-15)
 * kind 0 = CCX storage (rlen x nph per block, init_ph_mat), kind 1 = WCC workspace
 * (rlen x rlen per block, init_ph_wkspc / allocate_CC_wkspc :1075-1096) */
imsrg_status imsrg_cc_create(imsrg_ctx* ctx, int32_t kind, imsrg_cc** out);
imsrg_status imsrg_cc_destroy(imsrg_ctx* ctx, imsrg_cc* cc);
imsrg_status imsrg_cc_download(imsrg_ctx* ctx, const imsrg_cc* cc, double* host);
/* calculate_cross_coupled(HS, CCME, jbas)  src/cross_coupled.f90:1190 */
imsrg_status imsrg_calculate_cross_coupled(imsrg_ctx* ctx, const imsrg_op* HS, imsrg_cc* CCME);

/* ---- commutator pieces, src/commutators.f90 (same argument meaning and
 *      assign / accumulate semantics as the Fortran) */
imsrg_status imsrg_commutator_110(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, double* out);  /* :10  */
imsrg_status imsrg_commutator_111(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES); /* :36 */
imsrg_status imsrg_commutator_121(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES); /* :83 */
imsrg_status imsrg_commutator_122(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES); /* :283 */
imsrg_status imsrg_commutator_220(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, double* out);  /* :399 */
imsrg_status imsrg_commutator_221(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES,
                                  const imsrg_op* w1, const imsrg_op* w2);                            /* :435 */
imsrg_status imsrg_commutator_222_pp_hh(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES,
                                        imsrg_op* w1, imsrg_op* w2);                                  /* :581 */
imsrg_status imsrg_commutator_222_ph(imsrg_ctx* ctx, const imsrg_cc* LCC, const imsrg_cc* RCC, imsrg_op* RES,
                                     imsrg_cc* WCC);                                                  /* :771 */
/* The whole two-body-truncated [L,R] in the order of src/IMSRG_MAGNUS.f90:207-219:
 * both Pandya transforms, (110+220 when IMSRG_COMM_E0), 111, 121, 122, 222_pp_hh,
 * 221, 222_ph.  Uses the context's workspaces and its precision mode. */
imsrg_status imsrg_commutator(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, imsrg_op* RES, int32_t flags);

/* ---- generator and flow (src/generators.f90, src/IMSRG_MAGNUS.f90) */
imsrg_status imsrg_build_gs_white(imsrg_ctx* ctx, const imsrg_op* H, imsrg_op* ETA);   /* generators.f90:4 */
/* build_gs_atan (src/generators.f90:163-266): eta = atan(2 N / Eden) / 2 with White's numerators
 * and denominators */
imsrg_status imsrg_build_gs_atan(imsrg_ctx* ctx, const imsrg_op* H, imsrg_op* ETA);
/* build_gs_atanxx (src/generators.f90:271-374): numerators from H, denominators from Hold */
imsrg_status imsrg_build_gs_atanxx(imsrg_ctx* ctx, const imsrg_op* Hold, const imsrg_op* H, imsrg_op* ETA);
/* build_gs_w2 (src/generators.f90:109-160), the reference driver's default generator:
 * 1.5 atan(H) + 0.5 atanxx(H, [atan(H), H]), the commutator in the context's precision */
imsrg_status imsrg_build_gs_w2(imsrg_ctx* ctx, const imsrg_op* H, imsrg_op* ETA);
/* MAGNUS_EXPAND(DG, G, AD, jbas) :620 -- DG holds eta on entry and dOmega on exit */
imsrg_status imsrg_magnus_expand(imsrg_ctx* ctx, imsrg_op* DG, const imsrg_op* G, int32_t* commutators_used);
/* euler_step(G, DG, s, stp) :754 -- G += stp*DG; *s += stp */
imsrg_status imsrg_euler_step(imsrg_ctx* ctx, imsrg_op* G, const imsrg_op* DG, double* s, double stp);
/* BCH_EXPAND(HS, G, H, jbas, quads) :149 -- HS = e^G H e^-G; stops when a term's norm
 * times its coefficient drops below conv, or returns IMSRG_ERR_NOT_CONVERGED after
 * max_terms (the reference STOPs after 40). */
imsrg_status imsrg_bch_expand(imsrg_ctx* ctx, imsrg_op* HS, const imsrg_op* G, const imsrg_op* H, int32_t max_terms,
                              double conv, int32_t* terms_used);
/* BCH_EXPAND with quads = 'y': after every nested commutator the correction of
 * restore_quadrupoles (:908-1132) from the previous term is added, then rebuilt from the operator
 * just commuted (FP64 intermediates and insertions; the commutators in the context's precision). */
imsrg_status imsrg_bch_expand_quads(imsrg_ctx* ctx, imsrg_op* HS, const imsrg_op* G, const imsrg_op* H,
                                    int32_t max_terms, double conv, int32_t* terms_used);
/* restore_quadrupoles(X, OM, w1, w2, RES) :908 -- RES = 0 except its pp-hh arrays, which it assigns;
 * RES->herm = 1 */
imsrg_status imsrg_restore_quadrupoles(imsrg_ctx* ctx, const imsrg_op* X, const imsrg_op* OM, imsrg_op* RES);
/* CR_EXPAND(HS, G, H, jbas, quads) :532 -- HS = H + [G,H]/2! + [G,[G,H]]/3! + ..., the operator of
 * the completely renormalised triples (src/main_IMSRG.f90:310); stops when a term's norm times its
 * coefficient drops below conv or after max_terms (the reference: 14, 1e-6), without an error. */
imsrg_status imsrg_cr_expand(imsrg_ctx* ctx, imsrg_op* HS, const imsrg_op* G, const imsrg_op* H, int32_t max_terms,
                             double conv, int32_t* terms_used);

/* One step of magnus_decouple (src/IMSRG_MAGNUS.f90:47-110): MAGNUS_EXPAND(DG, G),
 * euler_step(G, DG, ds), BCH_EXPAND(HS, G, H, max_terms, conv), build_gs_white(HS, DG) and
 * mbpt2(HS).  DG holds eta on entry and the new eta on exit.  With use_graph != 0 the step
 * is captured once as a CUDA graph (both series' early exits are conditional graph nodes
 * decided on the device) and replayed with one launch while the operators and parameters
 * stay the same; the operators are bit-identical to the eager step (use_graph = 0).
 * info != NULL: waits for the step and fills info; returns IMSRG_ERR_NOT_CONVERGED when
 * BCH_EXPAND used all max_terms.  info == NULL (graph only): enqueues the step and returns. */
typedef struct imsrg_step_info {
  double E0;              /* E0 of HS after the step */
  double mbpt2;           /* MBPT(2) energy of HS after the step */
  int32_t magnus_terms;   /* nested commutators in MAGNUS_EXPAND */
  int32_t bch_terms;      /* nested commutators in BCH_EXPAND */
  int32_t bch_converged;  /* 1 when a BCH term fell below conv */
  int32_t graph_rebuilt;  /* 1 when this call captured and instantiated the graph */
} imsrg_step_info;
imsrg_status imsrg_magnus_step(imsrg_ctx* ctx, imsrg_op* HS, imsrg_op* G, imsrg_op* DG, const imsrg_op* H, double ds,
                               int32_t bch_max_terms, double bch_conv, int32_t use_graph, imsrg_step_info* info);
/* The same step with the flow state in the caller's host memory, for a caller that keeps it there
 * between steps (a Fortran driver): uploads Omega (g_host), eta (dg_host) and H (h_host), runs the
 * step and downloads H(s) (hs_host), Omega and eta.  Equal bit for bit to imsrg_op_upload_slab of
 * the three inputs, imsrg_magnus_step and imsrg_op_download_slab of the three outputs, but in the
 * captured step H's upload overlaps MAGNUS_EXPAND, Omega's download BCH_EXPAND and H(s)'s download
 * the generator.  The host buffers are slabs (imsrg_op_upload_slab's format) in pinned memory
 * (imsrg_pinned_alloc); HS, G, DG and H are device workspaces of the context.  Waits for the step.
 * No counterpart in the reference. */
imsrg_status imsrg_magnus_step_host(imsrg_ctx* ctx, imsrg_op* HS, imsrg_op* G, imsrg_op* DG, imsrg_op* H,
                                    double* hs_host, double* g_host, double* dg_host, const double* h_host, double ds,
                                    int32_t bch_max_terms, double bch_conv, int32_t use_graph, imsrg_step_info* info);
/* Totals over all graph-replayed steps of this context (no counterpart in the reference):
 * nested commutators, kernels launched, steps, steps whose BCH series did not converge. */
imsrg_status imsrg_magnus_step_counters(imsrg_ctx* ctx, int64_t* commutators, int64_t* kernels, int64_t* steps,
                                        int64_t* unconverged);

/* ---- rank-lambda tensor operators (BCH_TENSOR, src/IMSRG_MAGNUS.f90:389-464; allocate_tensor,
 * src/basic_IMSRG.f90:688-951).  rank2 and dpar2 are doubled (rank 2 -> 4, even parity -> 0).
 * Slab: [E0][fhh A*A][fpp P*P][fph P*A][block q = (J1 <= J2, Tz, bra parity): tgam(1..9)],
 * tgam = (pp,pp) (pp,ph) (pp,hh) (ph,ph) (hh,hh) (ph,hh) (hh,pp) (ph,pp) (hh,ph), column-major. */
typedef struct imsrg_tensor imsrg_tensor;
imsrg_status imsrg_tensor_sizes(imsrg_ctx* ctx, int32_t rank2, int32_t dpar2, int64_t* slab, int32_t* nblocks);
imsrg_status imsrg_tensor_block_info(imsrg_ctx* ctx, int32_t rank2, int32_t dpar2, int32_t* J1, int32_t* J2,
                                     int32_t* Tz, int32_t* P1);
imsrg_status imsrg_tensor_create(imsrg_ctx* ctx, int32_t rank2, int32_t dpar2, int32_t herm, imsrg_tensor** out);
imsrg_status imsrg_tensor_destroy(imsrg_ctx* ctx, imsrg_tensor* t);
imsrg_status imsrg_tensor_upload_slab(imsrg_ctx* ctx, imsrg_tensor* t, const double* host);
imsrg_status imsrg_tensor_download_slab(imsrg_ctx* ctx, const imsrg_tensor* t, double* host);
/* [L (scalar), R (tensor)] -> RES (RES->herm = -L->herm * R->herm), FP64.  pieces: 1 TS_111,
 * 2 TS_121, 4 TS_211, 8 TS_122, 16 TS_212, 32 TS_222_pp_hh + TS_221, 64 TS_222_ph
 * (src/TS_commutators.f90); 127 = the full commutator.  111 and 122 assign, the rest accumulate.
 * + 512: TS_222_ph recouples every nonzero product element instead of those above 1e-6 in size
 * (src/TS_commutators.f90:1562, 1714), as the EOM product does. */
imsrg_status imsrg_tensor_commutator(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_tensor* R, imsrg_tensor* RES,
                                     int32_t pieces);
/* BCH_TENSOR: HS <- e^G HS e^-G for a hermitian tensor HS and an anti-hermitian scalar G; stops when
 * a term's norm times its coefficient falls below conv (the reference: 1e-6, 30 terms). */
imsrg_status imsrg_bch_tensor(imsrg_ctx* ctx, const imsrg_op* G, imsrg_tensor* HS, int32_t max_terms, double conv,
                              int32_t* terms_used);
/* mat_frob_norm of a tensor operator (src/basic_IMSRG.f90:4056-4087) */
imsrg_status imsrg_tensor_frob_norm(imsrg_ctx* ctx, const imsrg_tensor* t, double* out);

/* ---- perturbative triples (restore_triples, src/IMSRG_MAGNUS.f90:767-902; the main program's
 * 'trips' option, src/main_IMSRG.f90:296-315): the correction summed over the three-body basis
 * of enumerate_three_body (src/basic_IMSRG.f90:4215-4420) of W^2/D (Jtot+1), W the three-body
 * element of [OM, H] (commutator_223_single, src/commutators.f90:928-1325) and D the
 * Epstein-Nesbet denominator with two-body monopoles.  H hermitian (the flowed or the CR_EXPAND
 * Hamiltonian), OM anti-hermitian (Omega).  items (may be NULL): (ppp, hhh) pairs summed. FP64. */
imsrg_status imsrg_restore_triples(imsrg_ctx* ctx, const imsrg_op* H, const imsrg_op* OM, double* e3, int64_t* items);

/* ---- EOM-IMSRG excitation ("ladder") operators (calculate_excited_states,
 * src/EOM_IMSRG.f90:13-98).  A ladder operator of rank rank2/2 and parity change dpar2 (0 or 2)
 * is a tensor whose only amplitudes are fph and the pp-hh arrays tgam(3) / tgam(7), stored with
 * lam(1) = 1 (an amplitude <pp J1|X|hh J2> with J1 > J2 sits in tgam(7) of block (J2, J1),
 * phase 1).  Amplitude vectors are ordered as unwrap_tensor / rewrap_tensor order them
 * (src/EOM_IMSRG.f90:1039-1340): fph of allowed (particle, hole) pairs, particles outer; then
 * per block the tgam(3) elements row by row and, for J1 < J2, the tgam(7) elements row by row,
 * pairs of identical orbits skipped at odd J. */
typedef struct imsrg_eom imsrg_eom;
/* on a host-only context (device < 0) only imsrg_eom_dim and imsrg_eom_amplitude_map work */
imsrg_status imsrg_eom_create(imsrg_ctx* ctx, int32_t rank2, int32_t dpar2, imsrg_eom** out);
imsrg_status imsrg_eom_destroy(imsrg_ctx* ctx, imsrg_eom* eom);
/* the amplitude count N (sps + tps of LANCZOS_DIAGONALIZE, src/EOM_IMSRG.f90:199-262) and the
 * number of one-body (1p1h) amplitudes, which come first */
imsrg_status imsrg_eom_dim(imsrg_ctx* ctx, const imsrg_eom* eom, int64_t* n, int64_t* n1b);
/* per amplitude: slab position, kind (0 fph, 1 tgam(3), 2 tgam(7)), (-1)^((J1-J2)/2) of its block
 * for kind 2, and the slab position of the transposed copy unwrap_tensor writes for J1 == J2
 * blocks (-1 otherwise); any pointer may be NULL */
imsrg_status imsrg_eom_amplitude_map(imsrg_ctx* ctx, const imsrg_eom* eom, int64_t* pos, int8_t* kind, int8_t* phase,
                                     int64_t* mirror);
/* matvec_nonzeroX_prod (src/EOM_IMSRG.f90:518-556): w = rewrap([H, unwrap(v)]) for a hermitian
 * scalar H, the product of the EOM_TS_commutator_* routines (src/EOM_TS_commutators.f90), in
 * the context's precision.  v, w: N host doubles (the _device form: N device doubles). */
imsrg_status imsrg_eom_matvec(imsrg_ctx* ctx, imsrg_eom* eom, const imsrg_op* H, const double* v, double* w);
imsrg_status imsrg_eom_matvec_device(imsrg_ctx* ctx, imsrg_eom* eom, const imsrg_op* H, const double* d_v, double* d_w);
/* unwrap_tensor of host amplitudes into a tensor of the same rank / parity (herm set to 1), and
 * rewrap_tensor back to host amplitudes */
imsrg_status imsrg_eom_unwrap(imsrg_ctx* ctx, imsrg_eom* eom, const double* v, imsrg_tensor* X);
imsrg_status imsrg_eom_rewrap(imsrg_ctx* ctx, imsrg_eom* eom, const imsrg_tensor* X, double* v);
/* LANCZOS_DIAGONALIZE (src/EOM_IMSRG.f90:164-334): the nev eigenvalues of smallest magnitude of
 * the EOM matrix (the excitation energies, ladder_ops(i)%E0), ascending; vectors (N x nev,
 * column-major, may be NULL) receives the normalised amplitude vectors.  Thick-restart Lanczos
 * with 5 nev basis vectors; converged when |beta s| <= tol |theta| for every wanted pair (the
 * reference: dsaupd, which = 'SM', tol 1e-10, 500 iterations).  IMSRG_ERR_NOT_CONVERGED after
 * max_restarts restarts (the results of the last one are still written). */
imsrg_status imsrg_eom_lanczos(imsrg_ctx* ctx, imsrg_eom* eom, const imsrg_op* H, int32_t nev, double tol,
                               int32_t max_restarts, double* energies, double* vectors, int32_t* matvecs,
                               int32_t* restarts);

/* ---- reverse mode (FP64) for adjoint derivatives of a flow (no counterpart in the
 * reference, which has no derivative code).  Each call ACCUMULATES into its outputs:
 * Lb += d<RESb, [L,R]>/dL and Rb += d<RESb, [L,R]>/dR for the FP64 commutator of
 * imsrg_commutator (flags as there, RESb->herm = the herm of RES), the exact transpose of
 * that routine in the plain slab inner product <A,B> = sum_k A[k] B[k]. */
imsrg_status imsrg_commutator_vjp(imsrg_ctx* ctx, const imsrg_op* L, const imsrg_op* R, const imsrg_op* RESb,
                                  imsrg_op* Lb, imsrg_op* Rb, int32_t flags);
/* Hb += d<ETAb, eta(H)>/dH for eta = build_gs_white(H) (numerators and denominators) */
imsrg_status imsrg_white_vjp(imsrg_ctx* ctx, const imsrg_op* H, const imsrg_op* ETAb, imsrg_op* Hb);
/* *out = sum_k A[k] B[k] over the slab (FP64) */
imsrg_status imsrg_dot_sq_op(imsrg_ctx* ctx, const imsrg_op* A, const imsrg_op* B, double* out);

/* ---- flat operator vectors and Omega checkpoints.  vectorize / repackage
 * (src/basic_IMSRG.f90:3929-4053): E0, fhh, fpp, fph in full, then per block and array the
 * on-and-below-diagonal rows of each column of the square arrays and every row of the others;
 * repackage fills the upper triangles with herm x the lower.  The *_slab forms work on host
 * slabs and need no GPU (host-only contexts too).  write/read_omega_checkpoint
 * (src/basic_IMSRG.f90:3215-3407) store the vector of a device operator as a raw stream of
 * neq native-endian FP64 values, the reference's access='stream' file; the caller names the
 * file.  Reading a file whose size is not neq values returns IMSRG_ERR_MISMATCH. */
imsrg_status imsrg_neq(const imsrg_ctx* ctx, int64_t* neq);
imsrg_status imsrg_vectorize_slab(const imsrg_ctx* ctx, const double* host_slab, double* host_vec);
imsrg_status imsrg_repackage_slab(const imsrg_ctx* ctx, const double* host_vec, int32_t herm, double* host_slab);
imsrg_status imsrg_write_omega_checkpoint(imsrg_ctx* ctx, const imsrg_op* G, const char* path);
imsrg_status imsrg_read_omega_checkpoint(imsrg_ctx* ctx, imsrg_op* G, const char* path);

/* ---- input preparation (host, FP64): seeded synthetic Hamiltonian in the reference's
 * me2j -> pn J-scheme layout (read_me2j_interaction, src/interaction_IO.f90:282-557) plus the
 * harmonic-oscillator kinetic energy (calculate_h0_harm_osc, src/basic_IMSRG.f90:2093-2191),
 * with the two-body centre-of-mass term of Htype 1 (-p1.p2 hw/A), normal ordered w.r.t. the
 * reference state (normal_order, src/basic_IMSRG.f90:2419-2550).  Writes one host slab (herm = +1). */
imsrg_status imsrg_synthetic_hamiltonian(imsrg_ctx* ctx, uint64_t seed, double v_scale, double* host_slab);
/* The same Hamiltonian before normal ordering, as calc_HF receives it after read_me2j_interaction
 * and calculate_h0_harm_osc (src/main_IMSRG.f90:125-157): the kinetic energy in fhh/fpp/fph, V in
 * the two-body arrays, E0 = 0. */
imsrg_status imsrg_synthetic_bare_hamiltonian(imsrg_ctx* ctx, uint64_t seed, double v_scale, double* host_slab);
/* The interaction of the synthetic Hamiltonian as me2j record values: four per record (T=0, then
 * T=1 with Mt = -1, 0, +1) in the loop order of read_me2j_interaction (src/interaction_IO.f90:
 * 320-352) over this basis's isospin orbits.  values NULL: *n receives the count. */
imsrg_status imsrg_synthetic_me2j_values(imsrg_ctx* ctx, uint64_t seed, double v_scale, double* values, int64_t* n);
/* read_me2j_interaction (src/interaction_IO.f90:282-557) from the record values of an me2j file
 * for eMax_file (the caller decompresses and parses the text): the proton-neutron J-scheme
 * two-body arrays of host_slab, for the records whose orbits are all in this basis; the rest of
 * the slab is untouched.  htype 1 (the intrinsic Hamiltonian, Lawson beta 0) adds the two-body
 * centre-of-mass term -p1.p2 hw/A (p1_p2, src/basic_IMSRG.f90:4445-4504), htype 0 does not.
 * The synthetic Hamiltonian uses htype 1.  IMSRG_ERR_MISMATCH when n is not the record count
 * of eMax_file. */
imsrg_status imsrg_me2j_to_slab(imsrg_ctx* ctx, const double* values, int64_t n, int32_t emax_file, int32_t htype,
                                double* host_slab);

/* ---- Hartree-Fock and normal ordering (FP64).  The self-consistency loop runs on the host
 * (blocks of orbits sharing (l, j, tz), at most eMax/2+1 orbits each, cyclic Jacobi in place of
 * LAPACK dsyev); the mean-field contraction of V and the two-body basis change run on the device.
 * coefs is the reference's full_sp_block_mat D as one host N x N column-major matrix
 * D(HO orbit, HF orbit); entries between different (l, j, tz) blocks are zero (and ignored). */
typedef struct {
  double e_hf;        /* E0 of the result (e_HF, src/HF_mod.f90:449-478) */
  double crit;        /* last convergence measure: sum over blocks of |eps_new - eps_old|_2 */
  int32_t iterations; /* self-consistency iterations (0 for calc_HO) */
} imsrg_hf_info;
/* calc_HF (src/HF_mod.f90:14-105), without a three-body force: H (herm +1) holds the bare
 * Hamiltonian and is replaced by the normal-ordered Hamiltonian in the HF basis; coefs and info
 * may be NULL.  Iterates while crit > 1e-6 (the reference's literal); IMSRG_ERR_NOT_CONVERGED
 * after max_iter iterations, H unchanged. */
imsrg_status imsrg_calc_hf(imsrg_ctx* ctx, imsrg_op* H, int32_t max_iter, double* coefs, imsrg_hf_info* info);
/* calc_HO (src/HF_mod.f90:107-179): normal ordering w.r.t. the HO reference, coefs = 1 */
imsrg_status imsrg_calc_ho(imsrg_ctx* ctx, imsrg_op* H, double* coefs, imsrg_hf_info* info);
/* sqop_to_HF (src/HF_mod.f90:181-209) of a bare scalar operator: f and V to the basis of coefs,
 * then normal ordering */
imsrg_status imsrg_sqop_to_hf(imsrg_ctx* ctx, imsrg_op* op, const double* coefs);
/* transform_2b_to_HF (src/HF_mod.f90:567-692): the two-body part alone, in place */
imsrg_status imsrg_transform_2b_to_hf(imsrg_ctx* ctx, imsrg_op* op, const double* coefs);
/* normal_order (src/basic_IMSRG.f90:2419-2550): E0 and the one-body elements between orbits
 * sharing (l, j, tz) from the operator's f and V w.r.t. the reference state; V unchanged */
imsrg_status imsrg_normal_order(imsrg_ctx* ctx, imsrg_op* op);

#ifdef __cplusplus
}
#endif
#endif /* IMSRG_GB300_H */
