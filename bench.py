#!/usr/bin/env python
"""Benchmark of the GB300 IMSRG(2) commutator engine.

Workload: the Magnus flow of a seeded synthetic Hamiltonian at eMax=10 (132 j-orbits,
16O-like reference, 132 (J,parity,Tz) channels, 88 cross-coupled channels) with the White
generator.  One "step" is one Magnus step of magnus_decouple (src/IMSRG_MAGNUS.f90:47-110):
MAGNUS_EXPAND, euler_step, BCH_EXPAND truncated at 10 nested commutators or a term norm
below 1e-8, the generator and MBPT(2) -- replayed from one CUDA graph.  The metric counts
the full two-body-truncated commutators [X, Y] those steps execute (counted on the device).

Prints one JSON line.  `value`: mixed-precision (split-BF16 tcgen05) commutators/s with
the operators resident in HBM.  `e2e`: the same metric with the flow's operators kept in
pinned host memory and copied in and out around every imsrg_magnus_step call.  The plain
FP64 GPU path runs the same steps for the speed-up and the |dE0| / ||dH(s)|| comparison.
With --impl reference the CPU restatement of the reference algorithm (FP64, OpenMP on all
host cores, BLAS dgemm) is timed on the same commutators instead.
"""
from __future__ import annotations

import argparse
import ctypes as C
import glob
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "eom-imsrg_gb300"))
sys.path.insert(0, ROOT)

METRIC = "IMSRG(2) commutators/s at eMax=10: mixed vs FP64 GPU at |ΔE0|<1 keV"
UNIT = "commutators/s"


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allreduce_max(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(pg, x: float) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampled every 100 ms in the background; stop() keeps the samples inside [t0, t1]."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = f"/tmp/imsrg_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def wait_running(self, timeout: float = 15.0):
        """Block until nvidia-smi has written two samples (it is past its start-up)."""
        t = time.time()
        while self.proc is not None and time.time() - t < timeout:
            try:
                with open(self.path) as f:
                    if sum(1 for _ in f) >= 2:
                        return
            except OSError:
                pass
            time.sleep(0.1)

    @staticmethod
    def _stamp(s: str) -> float:
        import datetime
        for fmt in ("%Y/%m/%d %H:%M:%S.%f", "%Y/%m/%d %H:%M:%S"):
            try:
                return datetime.datetime.strptime(s, fmt).timestamp()
            except ValueError:
                pass
        return float("nan")

    def stop(self, t0: float, t1: float) -> dict:
        """Summary of the samples taken between wall-clock times t0 and t1 (time.time())."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 10:
                continue
            try:
                rows.append((self._stamp(p[0]), float(p[2]), float(p[3]), p[6:10]))
            except ValueError:
                continue
        os.unlink(self.path)
        inside = [r for r in rows if t0 - 0.05 <= r[0] <= t1 + 0.05]
        sm = [r[1] for r in inside]
        reasons = sorted({k for r in inside for k, v in zip(self.NAMES, r[3]) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(r[2] for r in rows) if rows else None,
                "reasons": reasons, "samples": len(sm), "window_s": round(t1 - t0, 3)}


# ---------------------------------------------------------------- CPU side
def find_blas_dgemm():
    """Address of an exported Fortran-ABI dgemm in a BLAS bundled with numpy/scipy."""
    dirs = []
    for mod in ("numpy", "scipy"):
        try:
            m = __import__(mod)
            base = os.path.dirname(m.__file__)
            dirs += [os.path.join(base, "..", f"{mod}.libs"), os.path.join(base, ".libs")]
        except Exception:
            pass
    for d in dirs:
        for path in sorted(glob.glob(os.path.join(d, "*openblas*.so*"))):
            try:
                lib = C.CDLL(path)
            except OSError:
                continue
            for name, ilp64 in (("scipy_dgemm_64_", True), ("dgemm_64_", True), ("scipy_dgemm_", False),
                                ("dgemm_", False)):
                try:
                    f = getattr(lib, name)
                except AttributeError:
                    continue
                return C.cast(f, C.c_void_p).value, ilp64, f"{os.path.basename(path)}:{name}", lib
    return None, False, "built-in blocked dgemm", None


def cpu_commutators(emax: int, n_warm: int, n_steps: int, seed: int = 1, reference: str = "hf"):
    """Time the CPU restatement of the reference (the oracle) on one [eta, H] commutator per
    step.  Only the oracle runs here: it builds the same seeded bare Hamiltonian as the
    library, brings it to the same reference state (calc_HF, or calc_HO) and its White
    generator, untimed; the timed region is the commutators alone."""
    from oracle import oracle as orc
    from imsrg_gb300.basis import make_basis
    b = make_basis(emax)
    o = orc.Oracle(b)
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    addr, ilp64, blas_name, keep = find_blas_dgemm()
    if addr:
        orc.use_blas_dgemm(addr, ilp64)
    t = time.perf_counter()
    bare = o.synthetic_bare_hamiltonian(seed=seed)
    H = (o.calc_hf(bare) if reference == "hf" else o.calc_ho(bare))[0]
    eta = o.white(H, 1)
    prep_s = time.perf_counter() - t
    for _ in range(n_warm):
        o.commutator(eta, -1, H, 1, 1)
    t = time.perf_counter()
    for _ in range(n_steps):
        o.commutator(eta, -1, H, 1, 1)
    dt = time.perf_counter() - t
    return dt, cores, blas_name, keep, {"reference": reference, "E0": float(H[0]), "prepare_s": prep_s}


def prepared_hamiltonian(eng, reference: str, seed: int = 1, time_transform: bool = False):
    """The flow's starting Hamiltonian: the bare synthetic Hamiltonian (kinetic energy + V)
    after calc_HF on the device (mean-field tensor and two-body basis change on the GPU, the
    small self-consistency loop on the host) or after calc_HO (HO reference).  Returns the
    host slab, D(HO orbit, HF orbit) and a record of the step."""
    bare = eng.synthetic_bare_hamiltonian(seed=seed)
    op = eng.new_op(1, bare)
    eng.synchronize()
    t = time.perf_counter()
    D, info = eng.calc_hf(op) if reference == "hf" else eng.calc_ho(op)
    eng.synchronize()
    rec = {"reference": reference, "E0": info["e_hf"], "iterations": info["iterations"],
           "wall_ms": 1e3 * (time.perf_counter() - t)}
    H = op.download()
    if time_transform and reference == "hf":
        # the two-body basis change alone, CUDA events on the engine's stream (bare V, slab in place)
        A = eng.basis.nholes
        P = eng.basis.norbits - A
        n2b = eng.slab - (1 + A * A + P * P + P * A)
        op.upload(bare)
        eng.transform_2b_to_hf(op, D)  # warm-up (tables, allocation)
        reps = []
        for _ in range(3):
            op.upload(bare)
            eng.synchronize()
            eng.timer_begin()
            eng.transform_2b_to_hf(op, D)
            reps.append(eng.timer_end())
        ms = min(reps)
        rec.update({"transform_2b_ms": ms, "transform_2b_gbs": 2 * 8 * n2b / (ms * 1e-3) / 1e9,
                    "transform_2b_bytes": 2 * 8 * n2b})
    op.close()
    return H, D, rec


# ---------------------------------------------------------------- roofline bookkeeping
def algorithmic_work(eng, mode: str, phase: str, merged: bool = False):
    """Algorithmic bytes (or FLOPs) of one launch of a phase at this basis.

    Bytes count each array the phase must touch once: FP64 operators (8 B), the FP32
    recoupling input X (4 B, wcc_size elements; for the recoupling itself the distinct
    elements it reads, counted by the library), the split operand slices (2 B BF16, 4 B TF32
    per slice).  FLOPs are 2 M N K of the products times the number of slice products.
    merged: the ladder and X products run as one launch (phase pphh_gemm) or two (pphh_gemm,
    ph_gemm)."""
    import numpy as np
    S = {"bf16x3": 3, "bf16x6": 6, "tf32x3": 3, "fp64": 1}[mode]  # slice products per GEMM
    slices = {"bf16x3": 2, "bf16x6": 3, "tf32x3": 2, "fp64": 1}[mode]
    esize = 4 if mode == "tf32x3" else 2                           # bytes per operand value
    info = eng.block_info()
    cc = eng.cc_info()
    if phase == "recouple":   # counted exactly from the quadruples: distinct X reads (FP32), the
        #                        RES elements read and written (FP64), the kernel's index data
        v = [C.c_int64() for _ in range(4)]
        eng._ck(eng.L.imsrg_recouple_traffic(eng.h, *[C.byref(x) for x in v]))
        x_reads, x_distinct, res_elems, aux = (x.value for x in v)
        return "hbm", 4 * x_distinct + 16 * res_elems + aux
    if phase == "pphh_update":  # W1 and W2 (FP32) read where RES is updated, RES's upper triangles and
        #                         rectangular arrays read and written, the lower triangles written
        npp, nph_, nhh = (info[k].astype(np.int64) for k in ("npp", "nph", "nhh"))
        sq_up = int((npp * (npp + 1) // 2 + nph_ * (nph_ + 1) // 2 + nhh * (nhh + 1) // 2).sum())
        rect = int((npp * nph_ + npp * nhh + nph_ * nhh).sum())
        sq_low = int((npp * (npp - 1) // 2 + nph_ * (nph_ - 1) // 2 + nhh * (nhh - 1) // 2).sum())
        return "hbm", (2 * 4 + 16) * (sq_up + rect) + 2 * 4 * sq_low + 8 * sq_low
    if phase == "c122":       # read L and R once, write every unique 2b element of RES once (the
        #                       lower triangles of the square arrays come from the mirror pass)
        npp, nph_, nhh = (info[k].astype(np.int64) for k in ("npp", "nph", "nhh"))
        n_unique = int((npp * (npp + 1) // 2 + nph_ * (nph_ + 1) // 2 + nhh * (nhh + 1) // 2
                        + npp * nph_ + npp * nhh + nph_ * nhh).sum())
        return "hbm", 2 * 8 * eng.slab + 8 * n_unique
    x_flops = 4 * 2 * int((cc["rlen"].astype(np.int64) ** 2 * cc["nph"]).sum()) if mode != "fp64" else 0
    if phase == "ph_gemm":    # X: per cross-coupled channel one product over a K of four nph segments
        return "tensor", x_flops * S
    if phase == "pphh_gemm":  # sum 2 M N K over the K = npp ladder products (and X's when merged),
        #                       times the slice products
        f = x_flops if merged else 0
        for q in range(eng.nblocks):
            np_, nb, nh = int(info["npp"][q]), int(info["nph"][q]), int(info["nhh"][q])
            if np_ == 0:
                continue
            f += 2 * np_ * np_ * np_ + 2 * nh * nh * np_ + 2 * 2 * np_ * nh * np_
            f += 2 * nb * nb * np_ + 2 * 2 * np_ * nb * np_ + 2 * 2 * nb * nh * np_
        return "tensor", f * S
    if phase == "pandya":     # two operators read, each value written to four K segments of the X operands
        return "hbm", 2 * 8 * eng.slab + 2 * 4 * esize * slices * int((cc["rlen"] * cc["nph"]).sum())
    return None, None


def flow_state(eng, H):
    """(HS, G, DG, H) on the device at s = 0: HS = H, Omega = 0, DG = eta(H)."""
    dH = eng.new_op(1, H)
    HS = eng.new_op(1, H)
    G = eng.new_op(-1)
    DG = eng.new_op(-1)
    eng.build_gs_white(HS, DG)
    return HS, G, DG, dH


def flow_workload_name(args, norbits: int) -> str:
    """The benchmark workload, named the same way by both arms."""
    return (f"Magnus flow at eMax={args.emax} ({norbits} orbits, 16O-like), seeded synthetic Hamiltonian after "
            f"calc_{args.reference.upper()}, White generator, ds={args.ds}; a Magnus step = MAGNUS_EXPAND + "
            f"euler_step + BCH_EXPAND (<= {args.bch_max_terms - 1} nested commutators or term norm < "
            f"{args.bch_conv:g}) + generator + MBPT2; unit: one full IMSRG(2) commutator")


def reference_arm(args):
    """The CPU restatement of the reference (FP64, OpenMP on all host cores, BLAS dgemm).

    A step is one full commutator [eta, H] on the flow's starting state, the unit of the
    metric: the commutator's cost does not depend on its operands' values, so the K
    commutators are a bounded sample of the flow's commutators.  Only the oracle is loaded."""
    from imsrg_gb300.basis import make_basis
    dt, cores, blas, _, state = cpu_commutators(args.emax, args.warmup, args.steps, reference=args.reference)
    v = args.steps / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": flow_workload_name(args, make_basis(args.emax).norbits), "emax": args.emax,
                   "ds": args.ds, "step": "one full commutator [eta, H] of the flow (a bounded sample)",
                   "path": "CPU restatement of the reference (FP64, OpenMP)", "blas": blas,
                   "reference_state": state,
                   "inputs": "the oracle's own seeded synthetic Hamiltonian and calc_HF (no product library loaded)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full commutators [eta, H] at eMax={args.emax} on the "
                                   f"{args.reference.upper()} state"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def commutator_workload(args, local: int):
    """K eager [eta, H] commutators at eMax (default 10) on the HF state, after W warm-up ones, in the
    mixed mode with a given launch configuration (--tuning) or the autotuner's: the unit of the
    metric on its own, for profiling (an ncu launch list then holds one commutator's kernels per
    K)."""
    from imsrg_gb300 import Engine, make_basis
    emax = args.emax if args.emax is not None else 10
    b = make_basis(emax)
    eng = Engine(b, device=local, precision=args.mode)
    H, _, hf_rec = prepared_hamiltonian(eng, args.reference, seed=1)
    dH, dE, dR = eng.new_op(1, H), eng.new_op(-1), eng.new_op(1)
    eng.build_gs_white(dH, dE)
    if args.tuning:
        tune = json.loads(args.tuning)
        eng.set_tuning(tune)
    else:
        tune = eng.autotune(dE, dH, dR)
    for _ in range(max(args.warmup, 1)):
        eng.commutator(dE, dH, dR)
    eng.synchronize()
    l0 = eng.launch_count()
    eng.timer_begin()
    for _ in range(args.steps):
        eng.commutator(dE, dH, dR)
    ms = eng.timer_end()
    l1 = eng.launch_count()
    eng.profile_phases(True)  # per-phase event times of further commutators (after the timed ones)
    for _ in range(3):
        eng.commutator(dE, dH, dR)
    phases = eng.profile_read()
    eng.profile_phases(False)
    print(json.dumps({
        "metric": f"IMSRG(2) commutators/s at eMax={emax}, eager [eta,H]", "value": args.steps / (ms * 1e-3),
        "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "tf32" if args.mode == "tf32x3" else "bf16", "data": "synthetic",
        "config": {"workload": f"eager [eta,H] commutators at eMax={emax} ({b.norbits} orbits) on the "
                               f"{args.reference.upper()} state, {args.mode}", "reference_state": hf_rec,
                   "autotune": tune,
                   "phases_ms": {k: round(v[0] / max(v[1], 1), 4) for k, v in phases.items() if v[1]}},
        "gpu_launches": l1 - l0,
    }), flush=True)


def adjoint_workload(args, local: int):
    """dE0/dtheta through a FP64 Magnus flow by the device adjoint, checked against central
    finite differences of the same flow: H(theta) = H0 + sum_k theta_k V_k with K seeded
    channel-structured V_k ~ N(0, 0.1 MeV), theta = 0, eMax=6, ds=0.5 to s=30."""
    import numpy as np
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300.adjoint import EngineBackend, MagnusFlowAdjoint, channel_perturbations
    emax = args.emax if args.emax is not None else 6
    K, h = args.adjoint_k, 1e-4
    steps = int(round(args.s_end / args.ds))
    b = make_basis(emax)
    eng = Engine(b, device=local, precision="fp64")
    # HF frozen: H0 in the HF basis, each V_k moved to the same basis and normal ordered
    H0, Dhf, hf_rec = prepared_hamiltonian(eng, args.reference, seed=1)
    V = channel_perturbations(eng, K, sigma=0.1, seed=2)
    for k, v in enumerate(V):
        op = eng.new_op(1, v)
        eng.sqop_to_hf(op, Dhf)
        V[k] = op.download()
        op.close()
    fl = MagnusFlowAdjoint(EngineBackend(eng), H0, V, ds=args.ds, steps=steps)
    theta = np.zeros(K)
    t = time.perf_counter()
    plan = fl.plan(theta)
    eng.synchronize()
    t_plan = time.perf_counter() - t
    t = time.perf_counter()
    e0 = fl.forward(theta, plan)
    eng.synchronize()
    t_fwd = time.perf_counter() - t
    l0 = eng.launch_count()
    t = time.perf_counter()
    grad = fl.gradient()
    eng.synchronize()
    t_adj = time.perf_counter() - t
    launches = eng.launch_count() - l0
    nfd = K if args.fd_components is None else min(K, args.fd_components)
    fd = np.zeros(nfd)
    t = time.perf_counter()
    for k in range(nfd):
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd[k] = (fl.forward(tp, plan) - fl.forward(tm, plan)) / (2 * h)
    t_fd = time.perf_counter() - t
    err = float(np.max(np.abs(grad[:nfd] - fd)) / np.max(np.abs(fd)))
    print(json.dumps({
        "metric": f"adjoint dE0/dtheta wall time, K={K}, eMax={emax} Magnus flow to s={args.s_end:g}",
        "value": t_adj, "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": 1e3 * t_adj,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"differentiable Magnus flow, eMax={emax} ({b.norbits} orbits), K={K} channel "
                               f"perturbations N(0,0.1 MeV), theta=0, ds={args.ds}, {steps} steps, White generator",
                   "reference_state": hf_rec,
                   "plan_commutators": plan.commutators, "magnus_terms": plan.magnus, "bch_terms": plan.bch,
                   "E0": e0, "forward_s": t_fwd, "plan_s": t_plan, "adjoint_s": t_adj,
                   "adjoint_over_forward": t_adj / t_fwd, "fd_s": t_fd, "fd_h": h, "fd_components": nfd,
                   "grad": grad.tolist(), "fd": fd.tolist(), "max_rel_err_vs_fd": err,
                   "l2": "operators fit in L2 at this size (6.5 MiB per slab)"},
        "gpu_launches": launches,
    }), flush=True)


def precision_workload(args, local: int):
    """eMax=8: one [eta,H] commutator and a 20-step Magnus flow in plain FP64 and in the split-BF16
    modes (6 and 3 slice products, FP32 accumulation); |dE0| and ||dH_2b||_F against FP64."""
    import numpy as np
    from imsrg_gb300 import CONV, Engine, make_basis
    emax = args.emax if args.emax is not None else 8
    b = make_basis(emax)
    A_ = b.nholes
    P_ = b.norbits - A_
    n1 = 1 + A_ * A_ + P_ * P_ + P_ * A_
    H = None
    out = {}
    ref = {}
    for mode in ("fp64", "bf16x6", "bf16x3", "tf32x3"):
        eng = Engine(b, device=local, precision=mode)
        if H is None:
            H, _, hf_rec = prepared_hamiltonian(eng, args.reference, seed=1)
        dH, dE, dR = eng.new_op(1, H), eng.new_op(-1), eng.new_op(1)
        eng.build_gs_white(dH, dE)
        eng.commutator(dE, dH, dR)
        eng.timer_begin()
        for _ in range(5):
            eng.commutator(dE, dH, dR)
        ms = eng.timer_end() / 5
        comm = dR.download()
        st = flow_state(eng, H)
        t = time.perf_counter()
        e0 = [eng.magnus_step(*st, args.ds, 40, CONV, graph=True, allow_unconverged=True)["E0"]
              for _ in range(args.precision_flow_steps)]
        eng.synchronize()
        t_flow = time.perf_counter() - t
        hs = st[0].download()
        if mode == "fp64":
            ref = {"comm": comm, "hs": hs}
        entry = {"commutator_ms": ms, "flow_s": t_flow, "E0_flow": e0[-1]}
        if mode != "fp64":
            entry.update({
                "commutator_dE0_keV": abs(float(comm[0] - ref["comm"][0])) * 1e3,
                "commutator_dH2b_frob_rel": float(np.linalg.norm(comm[n1:] - ref["comm"][n1:]) /
                                                  np.linalg.norm(ref["comm"][n1:])),
                "flow_dE0_keV": abs(float(hs[0] - ref["hs"][0])) * 1e3,
                "flow_dH2b_frob_rel": float(np.linalg.norm(hs[n1:] - ref["hs"][n1:]) / np.linalg.norm(ref["hs"][n1:])),
                "speedup_commutator": out["fp64"]["commutator_ms"] / ms})
        out[mode] = entry
        del st, dH, dE, dR, eng
    print(json.dumps({
        "metric": f"split-BF16 vs FP64 at eMax={emax}: commutator and {args.precision_flow_steps}-step flow",
        "value": out["bf16x6"]["flow_dE0_keV"], "unit": "keV |dE0| (bf16x6 flow)", "n_gpus": 1,
        "steps": args.precision_flow_steps, "warmup": 1, "ms_per_step": 1e3 * out["bf16x6"]["flow_s"] /
        args.precision_flow_steps, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16", "data": "synthetic",
        "config": {"workload": f"[eta,H] and a Magnus flow (ds={args.ds}) at eMax={emax} ({b.norbits} orbits)",
                   "reference_state": hf_rec, "modes": out,
                   "not_built": "FP8 products"},
    }), flush=True)


def hf_flow_workload(args, local: int):
    """The small end-to-end case: calc_HF, then the FP64 Magnus flow (White generator, ds=0.5,
    BCH to 40 terms or term norm < 1e-6) to s=50 at eMax=4, once on the GPU (one CUDA-graph
    replay per step) and once on the CPU restatement of the reference's algorithm (the oracle,
    all host cores): wall time of each and the agreement of E0 and H(s)."""
    import numpy as np
    from imsrg_gb300 import CONV, Engine, make_basis
    from oracle import oracle as orc
    emax = args.emax if args.emax is not None else 4
    steps = int(round(args.s_end / args.ds))
    b = make_basis(emax)
    eng = Engine(b, device=local, precision="fp64")
    H, _, hf_rec = prepared_hamiltonian(eng, args.reference, seed=1)
    st = flow_state(eng, H)
    kw = dict(max_terms=40, conv=CONV, graph=True)
    eng.synchronize()
    c0 = eng.magnus_step_counters()
    t = time.perf_counter()
    for _ in range(steps):
        eng.magnus_step(*st, args.ds, wait=False, **kw)
    eng.synchronize()
    t_gpu = time.perf_counter() - t
    c1 = eng.magnus_step_counters()
    HS_gpu = st[0].download()
    o = orc.Oracle(b)
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    t = time.perf_counter()
    G = o.new()
    DG = o.white(H, 1)
    n_cpu = 0
    for _ in range(steps):
        used = o.magnus_expand(DG, G)
        G += args.ds * DG
        HS, n = o.bch_expand(G, H, 40, orc.BCH_CONV)
        DG = o.white(HS, 1)
        n_cpu += used + n
    t_cpu = time.perf_counter() - t
    n_gpu = c1["commutators"] - c0["commutators"]
    print(json.dumps({
        "metric": f"HF + FP64 Magnus flow to s={args.ds * steps:g} at eMax={emax}, wall time",
        "value": t_gpu, "unit": "s", "n_gpus": 1, "steps": steps, "warmup": 0, "ms_per_step": 1e3 * t_gpu / steps,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"calc_HF, then {steps} Magnus steps (ds={args.ds}) at eMax={emax} ({b.norbits} orbits), "
                               "White generator, BCH <= 40 terms / 1e-6; GPU graph steps vs the CPU restatement",
                   "reference_state": hf_rec, "gpu_s": t_gpu, "cpu_s": t_cpu, "cpu_cores": cores,
                   "cpu_over_gpu": t_cpu / t_gpu, "commutators_gpu": n_gpu, "commutators_cpu": n_cpu,
                   "unconverged_bch_steps_gpu": c1["unconverged"] - c0["unconverged"],
                   "E0_gpu": float(HS_gpu[0]), "E0_cpu": float(HS[0]), "dE0_keV": 1e3 * abs(HS_gpu[0] - HS[0]),
                   "H_max_rel_err": float(np.max(np.abs(HS_gpu - HS)) / np.max(np.abs(HS))),
                   "mbpt2_final": o.mbpt2(HS, 1)},
        "cpu_baseline": {"value": t_cpu, "unit": "s", "cores": cores, "kind": "port",
                         "sample": f"the same {steps}-step flow with the oracle (FP64, OpenMP x{cores})"},
        "gpu_launches": c1["kernels"] - c0["kernels"],
    }), flush=True)


def observables_workload(args, local: int):
    """Mixed-precision Magnus flow at eMax=12 to s=50, then BCH transformations of a scalar r^2
    one-body operator and of a rank-2 one-body tensor (synthetic HO radial matrix elements)
    through the scalar and the tensor commutators; peak HBM, |dE0| and d<r^2> against FP64."""
    import numpy as np
    import torch
    from imsrg_gb300 import CONV, Engine, make_basis
    from imsrg_gb300.operators import q2_operator, r2_operator

    def used_gib():
        free, total = torch.cuda.mem_get_info(local)
        return (total - free) / 2**30

    emax = args.emax if args.emax is not None else 12
    steps = int(round(args.s_end / args.ds))
    b = make_basis(emax)
    A = b.Aprot + b.Aneut
    base = used_gib()
    peak = 0.0
    eng = Engine(b, device=local, precision=args.mode)
    H, Dhf, hf_rec = prepared_hamiltonian(eng, args.reference, seed=1)
    st = flow_state(eng, H)
    kw = dict(max_terms=args.obs_bch_max_terms, conv=CONV, graph=True, allow_unconverged=True)
    e0s, crit = [], []
    t = time.perf_counter()
    for k in range(steps):
        info = eng.magnus_step(*st, args.ds, **kw)
        e0s.append(info["E0"])
        crit.append(abs(info["mbpt2"]))
        peak = max(peak, used_gib())
    eng.synchronize()
    t_flow = time.perf_counter() - t
    counters = eng.magnus_step_counters()
    HS, G = st[0], st[1]
    G_host = G.download()
    # r^2 through BCH_EXPAND with the final Omega, mixed and FP64
    R2 = r2_operator(eng, coefs=Dhf)
    dR2, dR2s = eng.new_op(1, R2), eng.new_op(1)
    t = time.perf_counter()
    n_r2 = eng.bch_expand(dR2s, G, dR2, 40, CONV)
    eng.synchronize()
    t_r2 = time.perf_counter() - t
    r2_mixed = dR2s.E0 / A
    peak = max(peak, used_gib())
    # FP64: the first F steps of the same flow (|dE0|, ||dH||) and the r^2 transformation
    cmp = {}
    eng64 = Engine(b, device=local, precision="fp64")
    st64 = flow_state(eng64, H)
    F = min(args.fp64_steps, steps)
    for _ in range(F):
        eng64.magnus_step(*st64, args.ds, **kw)
    peak = max(peak, used_gib())
    if F:
        stm = flow_state(eng, H)
        for _ in range(F):
            eng.magnus_step(*stm, args.ds, **kw)
        hm, h64 = stm[0].download(), st64[0].download()
        cmp = {"fp64_steps": F, "dE0_keV": abs(float(hm[0] - h64[0])) * 1e3,
               "dH_frob_rel": float(np.linalg.norm(hm - h64) / np.linalg.norm(h64))}
        del stm
    del st64
    G64, R64, R64s = eng64.new_op(-1, G_host), eng64.new_op(1, R2), eng64.new_op(1)
    eng64.bch_expand(R64s, G64, R64, 40, CONV)
    r2_fp64 = R64s.E0 / A
    peak = max(peak, used_gib())
    del G64, R64, R64s, eng64
    # rank-2 tensor through BCH_TENSOR with the final Omega: in the flow's mixed mode (ladder and
    # cross-coupled products on the tensor cores, the other pieces in FP32), then in FP64
    Q = q2_operator(eng, 4, coefs=Dhf)
    dQ = eng.new_tensor(4, 0, 1, Q)
    q0 = dQ.frob()
    t = time.perf_counter()
    n_q = eng.bch_tensor(G, dQ, 30, CONV)
    eng.synchronize()
    t_q = time.perf_counter() - t
    q1 = dQ.frob()
    q_mixed = dQ.download()
    tslab = dQ.slab
    peak = max(peak, used_gib())
    del dQ
    e64q = Engine(b, device=local, precision="fp64")
    G64q, dQ64 = e64q.new_op(-1, G_host), e64q.new_tensor(4, 0, 1, Q)
    t = time.perf_counter()
    n_q64 = e64q.bch_tensor(G64q, dQ64, 30, CONV)
    e64q.synchronize()
    t_q64 = time.perf_counter() - t
    q_fp64 = dQ64.download()
    peak = max(peak, used_gib())
    del G64q, dQ64, e64q
    dq_rel = float(np.linalg.norm(q_mixed - q_fp64) / np.linalg.norm(q_fp64))
    print(json.dumps({
        "metric": f"observables after a mixed-precision Magnus flow, eMax={emax}", "value": r2_mixed,
        "unit": "fm^2 (<r^2> per nucleon)", "n_gpus": 1, "steps": steps, "warmup": 0,
        "ms_per_step": 1e3 * t_flow / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16", "data": "synthetic",
        "config": {"workload": f"Magnus flow at eMax={emax} ({b.norbits} orbits) to s={args.ds * steps:g} with "
                               f"{args.mode} commutators (graph steps, BCH up to {args.obs_bch_max_terms - 1} terms), "
                               "then BCH of r^2 (scalar) and r^2 Y2 (rank 2, tensor commutators in the same mode and in FP64)",
                   "reference_state": hf_rec,
                   "E0_final": e0s[-1], "E0_first_steps": e0s[:5], "mbpt2_final": crit[-1],
                   "flow_s": t_flow, "flow_commutators": counters["commutators"],
                   "r2_mixed_fm2": r2_mixed, "r2_fp64_fm2": r2_fp64, "d_r2_fm2": abs(r2_mixed - r2_fp64),
                   "r2_bare_fm2": R2[0] / A, "r2_bch_terms": n_r2, "r2_bch_s": t_r2,
                   "q2_norm_bare": q0, "q2_norm_evolved": q1, "q2_bch_terms": n_q, "q2_bch_s": t_q,
                   "q2_bch_terms_fp64": n_q64, "q2_bch_s_fp64": t_q64, "q2_mixed_vs_fp64_frob_rel": dq_rel,
                   "tensor_slab_doubles": tslab, "peak_hbm_gib": round(peak - base, 2), **cmp},
    }), flush=True)


def eom_workload(args, local: int):
    """EOM-IMSRG excited states (calculate_excited_states) after a mixed-precision Magnus flow:
    calc_HF, graph steps to s=50, then the Lanczos for J^pi = 0+, 2+ and 3- (nev states each)
    with the EOM product in FP64 and in the flow's mixed mode; wall time of each, the
    energies' agreement, and the EOM product rate against the oracle's on the host cores."""
    import numpy as np
    from imsrg_gb300 import CONV, Engine, make_basis
    from imsrg_gb300.eom import EOM_TOL, LadderSpace
    from oracle import oracle as orc
    emax = args.emax if args.emax is not None else 8
    steps = int(round(args.s_end / args.ds))
    b = make_basis(emax)
    eng = Engine(b, device=local, precision=args.mode)
    H, _, hf_rec = prepared_hamiltonian(eng, args.reference, seed=1)
    st = flow_state(eng, H)
    kw = dict(max_terms=args.obs_bch_max_terms, conv=CONV, graph=True, allow_unconverged=True)
    t = time.perf_counter()
    for _ in range(steps):
        info = eng.magnus_step(*st, args.ds, **kw)
    eng.synchronize()
    t_flow = time.perf_counter() - t
    HS_host = st[0].download()
    del st
    states = [(0, 0), (2, 0), (3, 1)]
    nev = args.eom_states
    res = {}
    total = {}
    for mode in ("fp64", args.mode):
        e = Engine(b, device=local, precision=mode)
        HS = e.new_op(1, HS_host)
        for J, P in states:
            sp = LadderSpace(e, 2 * J, 2 * P)
            v = np.random.default_rng(0).standard_normal(sp.n)
            sp.matvec(HS, v)  # warm-up (tables, workspaces)
            t = time.perf_counter()
            reps = 3
            for _ in range(reps):
                sp.matvec(HS, v)
            t_mv = (time.perf_counter() - t) / reps
            t = time.perf_counter()
            E, V, inf = sp.lanczos(HS, nev, EOM_TOL)
            t_lz = time.perf_counter() - t
            key = f"{J}{'+-'[P]}"
            res.setdefault(key, {"amplitudes": sp.n})[mode] = {
                "energies_MeV": [float(x) for x in E], "n1p1h": [float(np.sum(V[:sp.n1b, i] ** 2)) for i in range(nev)],
                "lanczos_s": t_lz, "matvecs": inf["matvecs"], "restarts": inf["restarts"], "matvec_ms": 1e3 * t_mv}
            total[mode] = total.get(mode, 0.0) + t_lz
            del sp
        del HS, e
    for key, r in res.items():
        r["max_dE_keV"] = 1e3 * float(np.max(np.abs(np.array(r["fp64"]["energies_MeV"]) -
                                                     np.array(r[args.mode]["energies_MeV"]))))
    # the oracle's EOM product (two FP64 scalar-tensor commutators on all host cores), J=0+
    o = orc.Oracle(b)
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    eo = orc.EomOracle(o, 0, 0)
    v = np.random.default_rng(0).standard_normal(eo.n)
    t = time.perf_counter()
    eo.matvec(HS_host, v)
    t_cpu = time.perf_counter() - t
    gpu_mv = res["0+"][args.mode]["matvec_ms"] * 1e-3
    print(json.dumps({
        "metric": f"EOM-IMSRG excited states at eMax={emax}: Lanczos wall time, J^pi 0+ 2+ 3-, {nev} states each",
        "value": total[args.mode], "unit": "s", "n_gpus": 1, "steps": len(states), "warmup": 1,
        "ms_per_step": 1e3 * total[args.mode] / len(states), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
        "config": {"workload": f"calc_HF, {steps} {args.mode} Magnus graph steps (ds={args.ds}) at eMax={emax} "
                               f"({b.norbits} orbits), then calculate_excited_states for 0+, 2+, 3- (nev={nev}, "
                               f"tol={EOM_TOL:.3g}, 5 nev Lanczos vectors) with the EOM product in FP64 and {args.mode}",
                   "reference_state": hf_rec, "flow_s": t_flow, "E0": float(HS_host[0]),
                   "mbpt2_final": info["mbpt2"], "lanczos_s_fp64": total["fp64"], "states": res,
                   "eom_matvecs_per_s_gpu_0+": 1.0 / gpu_mv, "eom_matvecs_per_s_cpu_0+": 1.0 / t_cpu},
        "cpu_baseline": {"value": 1.0 / t_cpu, "unit": "EOM products/s (J=0+)", "cores": cores, "kind": "port",
                         "sample": f"one EOM product for 0+ at eMax={emax} with the oracle (two FP64 scalar-tensor "
                                   f"commutators, OpenMP x{cores})"},
    }), flush=True)


def triples_workload(args, local: int):
    """The driver's triples step (src/main_IMSRG.f90:294-318) after a mixed-precision Magnus flow:
    calc_HF, bf16x6 graph steps to s=50, then restore_triples of (H0, Omega) and of
    (CR_EXPAND(Omega, H0), Omega) on the GPU in FP64, and the first by the oracle on all host
    cores (the CPU baseline)."""
    from imsrg_gb300 import CONV, Engine, make_basis
    from oracle import oracle as orc
    emax = args.emax if args.emax is not None else 8
    steps = int(round(args.s_end / args.ds))
    b = make_basis(emax)
    eng = Engine(b, device=local, precision=args.mode)
    H, _, hf_rec = prepared_hamiltonian(eng, args.reference, seed=1)
    st = flow_state(eng, H)
    kw = dict(max_terms=args.obs_bch_max_terms, conv=CONV, graph=True, allow_unconverged=True)
    t = time.perf_counter()
    for _ in range(steps):
        eng.magnus_step(*st, args.ds, **kw)
    eng.synchronize()
    t_flow = time.perf_counter() - t
    E0 = st[0].E0
    OM = st[1].download()
    del st
    e64 = Engine(b, device=local, precision="fp64")
    dH, dG = e64.new_op(1, H), e64.new_op(-1, OM)
    e64.restore_triples(dH, dG)  # warm-up
    t = time.perf_counter()
    corr, items = e64.restore_triples(dH, dG)
    t_gpu = time.perf_counter() - t
    CR = e64.new_op(1)
    t = time.perf_counter()
    n_cr = e64.cr_expand(CR, dG, dH, 14, CONV)
    corr_cr, _ = e64.restore_triples(CR, dG)
    e64.synchronize()
    t_cr = time.perf_counter() - t
    o = orc.Oracle(b)
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    t = time.perf_counter()
    corr_cpu = o.restore_triples(H, OM)
    t_cpu = time.perf_counter() - t
    print(json.dumps({
        "metric": f"Magnus triples correction at eMax={emax}, wall time", "value": t_gpu, "unit": "s",
        "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": 1e3 * t_gpu, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"calc_HF, {steps} {args.mode} Magnus graph steps (ds={args.ds}) at eMax={emax} "
                               f"({b.norbits} orbits), then restore_triples(H0, Omega) (FP64, {items} ppp-hhh pairs) "
                               "and the completely renormalised form with CR_EXPAND",
                   "reference_state": hf_rec, "flow_s": t_flow, "E0": E0, "triples_MeV": corr,
                   "E0_plus_triples": E0 + corr, "cr_triples_MeV": corr_cr, "cr_expand_terms": n_cr,
                   "cr_triples_s": t_cr, "triples_cpu_MeV": corr_cpu,
                   "rel_diff_gpu_cpu": abs(corr - corr_cpu) / max(abs(corr_cpu), 1e-300),
                   "cpu_s": t_cpu, "cpu_over_gpu": t_cpu / t_gpu},
        "cpu_baseline": {"value": t_cpu, "unit": "s", "cores": cores, "kind": "port",
                         "sample": f"the same restore_triples at eMax={emax} with the oracle (FP64, OpenMP x{cores})"},
    }), flush=True)


def ode_workload(args, local: int):
    """The traditional flow (decouple_hamiltonian, src/IMSRG_ODE.f90:9-178): calc_HF, then the
    Adams integration of dH/ds = [eta, H] over intervals of 0.1 until |MBPT2| < 1e-6 (or s=s_end),
    once with the device derivative and once with the oracle's (all host cores), same integrator."""
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300.ode import decouple_hamiltonian
    from oracle import oracle as orc
    emax = args.emax if args.emax is not None else 4
    b = make_basis(emax)
    eng = Engine(b, device=local, precision="fp64")
    H, _, hf_rec = prepared_hamiltonian(eng, args.reference, seed=1)
    s_max = args.s_end
    t = time.perf_counter()
    res = decouple_hamiltonian(eng, H, s_max=s_max)
    t_gpu = time.perf_counter() - t
    o = orc.Oracle(b)
    cores = os.cpu_count() or 1
    orc.set_threads(cores)

    def oracle_derivative(s, y):
        Hs = eng.repackage(y, 1)
        return eng.vectorize(o.commutator(o.white(Hs, 1), -1, Hs, 1))

    t = time.perf_counter()
    ref = decouple_hamiltonian(eng, H, s_max=s_max, derivative=oracle_derivative)
    t_cpu = time.perf_counter() - t
    print(json.dumps({
        "metric": f"traditional ODE flow at eMax={emax}, wall time", "value": t_gpu, "unit": "s", "n_gpus": 1,
        "steps": len(res.steps) - 1, "warmup": 0, "ms_per_step": 1e3 * t_gpu / max(len(res.steps) - 1, 1),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"calc_HF, then decouple_hamiltonian at eMax={emax} ({b.norbits} orbits): Adams "
                               f"(Shampine-Gordon) integration, relerr = abserr = 1e-6, intervals of 0.1 up to "
                               f"s={s_max:g} or |MBPT2| < 1e-6; device derivative vs the oracle's, same integrator",
                   "reference_state": hf_rec, "s_end": res.steps[-1][1], "E0": res.E0, "E0_cpu": ref.E0,
                   "dE0_keV": 1e3 * abs(res.E0 - ref.E0), "derivatives": res.evaluations,
                   "derivatives_cpu": ref.evaluations, "gpu_s": t_gpu, "cpu_s": t_cpu, "cpu_over_gpu": t_cpu / t_gpu},
        "cpu_baseline": {"value": t_cpu, "unit": "s", "cores": cores, "kind": "port",
                         "sample": f"the same flow with the oracle's derivative (FP64, OpenMP x{cores})"},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20, help="timed Magnus steps")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--emax", type=int, default=None, help="default 10 (flow), 6 (adjoint)")
    ap.add_argument("--workload", default="flow", choices=["flow", "commutator", "adjoint", "observables", "precision",
                                                         "hf-flow", "eom", "triples", "ode"])
    ap.add_argument("--precision-flow-steps", type=int, default=20)
    ap.add_argument("--obs-bch-max-terms", type=int, default=40)
    ap.add_argument("--adjoint-k", type=int, default=16)
    ap.add_argument("--eom-states", type=int, default=4, help="eom workload: states per J^pi")
    ap.add_argument("--s-end", type=float, default=30.0, help="adjoint workload: flow length")
    ap.add_argument("--fd-components", type=int, default=None)
    ap.add_argument("--mode", default=None, choices=["bf16x3", "bf16x6", "tf32x3"],
                    help="mixed mode: default bf16x3 for the flow (the headline), bf16x6 for the other workloads")
    ap.add_argument("--ds", type=float, default=0.5)
    ap.add_argument("--bch-max-terms", type=int, default=11, help="BCH_EXPAND max_terms (10 nested commutators)")
    ap.add_argument("--bch-conv", type=float, default=1e-8)
    ap.add_argument("--fp64-steps", type=int, default=-1,
                    help="FP64 graph steps (rate and |dE0|); -1: the W + K steps of the timed flow; 0 skips")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch configuration")
    ap.add_argument("--tuning", default=None,
                    help="apply this launch configuration (JSON, as config.autotune reports it) instead of tuning")
    ap.add_argument("--reference", default="hf", choices=["hf", "ho"],
                    help="reference state of the flow: calc_HF (default) or calc_HO")
    args = ap.parse_args()
    args.e2e_steps = max(1, args.e2e_steps)
    if args.mode is None:
        args.mode = "bf16x3" if args.workload in ("flow", "commutator") else "bf16x6"
    world, rank, local, pg = dist_setup()

    if args.emax is None and args.workload == "flow":
        args.emax = 10
    if args.impl == "reference":
        if rank == 0:
            if args.emax is None:
                args.emax = 6
            reference_arm(args)
        return
    if args.workload == "adjoint":
        if rank == 0:
            adjoint_workload(args, local)
        return
    if args.workload == "commutator":
        if rank == 0:
            commutator_workload(args, local)
        return
    if args.workload == "hf-flow":
        if rank == 0:
            if args.s_end == 30.0:
                args.s_end = 50.0
            hf_flow_workload(args, local)
        return
    if args.workload == "precision":
        if rank == 0:
            precision_workload(args, local)
        return
    if args.workload == "ode":
        if rank == 0:
            if args.s_end == 30.0:
                args.s_end = 20.0
            ode_workload(args, local)
        return
    if args.workload == "triples":
        if rank == 0:
            if args.s_end == 30.0:
                args.s_end = 50.0
            triples_workload(args, local)
        return
    if args.workload == "eom":
        if rank == 0:
            if args.s_end == 30.0:
                args.s_end = 50.0
            eom_workload(args, local)
        return
    if args.workload == "observables":
        if rank == 0:
            if args.s_end == 30.0:
                args.s_end = 50.0
            observables_workload(args, local)
        return

    from imsrg_gb300 import Engine, make_basis
    import numpy as np

    W = max(args.warmup, 3)
    K = args.steps
    step_kw = dict(max_terms=args.bch_max_terms, conv=args.bch_conv, graph=True)
    b = make_basis(args.emax)
    eng = Engine(b, device=local, precision=args.mode)
    H, _, hf_rec = prepared_hamiltonian(eng, args.reference, seed=1, time_transform=True)
    # the library's autotuner picks the launch configuration on [eta, H] of this basis
    tune = None
    if args.tuning:
        tune = json.loads(args.tuning)
        eng.set_tuning(tune)
    elif not args.no_autotune:
        tH, tE, tR = eng.new_op(1, H), eng.new_op(-1), eng.new_op(1)
        eng.build_gs_white(tH, tE)
        tune = eng.autotune(tE, tH, tR)
        del tH, tE, tR

    # ---- timed: K Magnus steps of the flow, each one CUDA-graph replay (after W warm-up steps)
    # the clock sampler starts before the warm-up: nvidia-smi's own start-up can stall the
    # device for seconds, which must not fall into the timed region
    clocks = ClockSampler(local)
    clocks.start()
    st = flow_state(eng, H)
    e0_steps = []
    for _ in range(W):
        e0_steps.append(eng.magnus_step(*st, args.ds, allow_unconverged=True, **step_kw)["E0"])
    eng.synchronize()
    clocks.wait_running()
    barrier(pg)
    eng.synchronize()
    c0 = eng.magnus_step_counters()
    t_wall0 = time.time()
    eng.timer_begin()
    for _ in range(K):
        eng.magnus_step(*st, args.ds, wait=False, **step_kw)
    ms = eng.timer_end()
    t_wall1 = time.time()
    eng.synchronize()
    c1 = eng.magnus_step_counters()
    barrier(pg)
    clk = clocks.stop(t_wall0, t_wall1)
    ms_max = allreduce_max(pg, ms)
    n_comm = c1["commutators"] - c0["commutators"]
    comm_all = allreduce_sum(pg, n_comm)
    launches_all = int(allreduce_sum(pg, c1["kernels"] - c0["kernels"]))
    value = comm_all / (ms_max * 1e-3)
    timed = {"steps": K, "commutators": n_comm, "unconverged_bch_steps": c1["unconverged"] - c0["unconverged"],
             "s_end": args.ds * (W + K)}
    # the mixed flow's state at the end of the timed region (s = ds * (W + K))
    hs_end, eta_end = st[0].download(), st[2].download()
    del st
    # ---- plain FP64 GPU path: the same flow, same graph step; its rate, and |dE0|, ||dH(s)||
    #      against the mixed flow at the end of the timed region (the default runs the FP64 flow
    #      for the same W + K steps) or after --fp64-steps steps
    cmp = {}
    fp64_rate = None
    F = (W + K) if args.fp64_steps < 0 else args.fp64_steps
    if F > 0:
        eng64 = Engine(b, device=local, precision="fp64")
        st64 = flow_state(eng64, H)
        eng64.magnus_step(*st64, args.ds, allow_unconverged=True, **step_kw)
        if F > 1:
            k0 = eng64.magnus_step_counters()
            eng64.timer_begin()
            for _ in range(F - 1):
                eng64.magnus_step(*st64, args.ds, wait=False, **step_kw)
            ms64 = eng64.timer_end()
            k1 = eng64.magnus_step_counters()
            fp64_rate = (k1["commutators"] - k0["commutators"]) / (ms64 * 1e-3)
        if F == W + K:
            hs_m, eta_m = hs_end, eta_end
        else:
            stm = flow_state(eng, H)
            for _ in range(F):
                eng.magnus_step(*stm, args.ds, allow_unconverged=True, **step_kw)
            hs_m, eta_m = stm[0].download(), stm[2].download()
            del stm
        hs_64 = st64[0].download()
        cmp = {"flow_steps": F, "s_compared": args.ds * F, "E0_mixed": float(hs_m[0]), "E0_fp64": float(hs_64[0]),
               "dE0_keV": abs(float(hs_m[0] - hs_64[0])) * 1e3,
               "dH_frob_rel": float(np.linalg.norm(hs_m - hs_64) / np.linalg.norm(hs_64))}
        # one commutator [eta, H(s)] in both precisions on identical inputs
        dR, dEm, dHm = eng.new_op(1), eng.new_op(-1, eta_m), eng.new_op(1, hs_m)
        dR64 = eng64.new_op(1)
        eng.commutator(dEm, dHm, dR)
        dE64, dHs64 = eng64.new_op(-1, eta_m), eng64.new_op(1, hs_m)
        eng64.commutator(dE64, dHs64, dR64)
        r_m, r_64 = dR.download(), dR64.download()
        cmp.update({"commutator_dE0_keV": abs(float(r_m[0] - r_64[0])) * 1e3,
                    "commutator_max_rel_err": float(np.max(np.abs(r_m - r_64)) / np.max(np.abs(r_64)))})
        del st64, dR64, dE64, dHs64, eng64, dR, dEm, dHm

    # ---- end to end through the C ABI: the flow kept in pinned host memory; every step
    # uploads H, Omega, eta and downloads H(s), Omega, eta (imsrg_magnus_step_host)
    nbytes = 8 * eng.slab
    st = flow_state(eng, H)
    hb = []
    for _ in range(4):
        p = C.c_void_p()
        eng._ck(eng.L.imsrg_pinned_alloc(nbytes, C.byref(p)))
        hb.append(p)
    for op, p in zip(st, hb):
        eng._ck(eng.L.imsrg_op_download_slab(eng.h, op.h, p))
    HS_, G_, DG_, H_ = st
    e2e_comm = 0
    for it in range(args.e2e_steps + 1):
        if it == 1:
            barrier(pg)
            t0 = time.perf_counter()
        # imsrg_magnus_step_host: uploads H, Omega and eta, runs the step (the graph replay) and
        # downloads H(s), Omega and eta, with H's upload and Omega's download inside the step
        info = eng.magnus_step_host(HS_, G_, DG_, H_, hb[0], hb[1], hb[2], hb[3], args.ds, allow_unconverged=True,
                                    **step_kw)
        if it >= 1:
            e2e_comm += info["magnus_terms"] + info["bch_terms"]
    e2e_s = allreduce_max(pg, time.perf_counter() - t0)
    e2e_value = allreduce_sum(pg, e2e_comm) / e2e_s
    for p in hb:
        eng.L.imsrg_pinned_free(p)
    del st, HS_, G_, DG_, H_

    # ---- per-phase event timing of eager commutators for the roofline of the dominant kernel
    dH = eng.new_op(1, H)
    dE = eng.new_op(-1)
    dR = eng.new_op(1)
    eng.build_gs_white(dH, dE)
    eng.commutator(dE, dH, dR)
    eng.profile_phases(True)
    nprof = 3
    for _ in range(nprof):
        eng.commutator(dE, dH, dR)
    phases = eng.profile_read()
    eng.profile_phases(False)
    dom = max(phases, key=lambda k: phases[k][0])
    dom_ms = phases[dom][0] / max(phases[dom][1], 1)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    bound, work = algorithmic_work(eng, args.mode, dom, bool((tune or {}).get("gemm_merged", 0)))
    traffic = None
    try:
        tr = json.load(open(os.path.join(ROOT, "profiles", "ncu_traffic.json")))
        traffic = tr.get(f"{dom}@emax{args.emax}@{args.mode}")
    except Exception:
        pass
    if bound == "tensor":
        peak = peaks.get("bf16_tflops", 1900.0)
        achieved = work / (dom_ms * 1e-3) / 1e12
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak}
    else:
        peak = peaks.get("hbm_gbs", 6800.0)
        achieved = (work or 0) / (dom_ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak}
    roof.update({"traffic": traffic, "kernel_phase": dom, "kernel_ms": dom_ms, "algorithmic": work,
                 "peak_source": "measured" if peaks else "fallback",
                 "phases_ms": {k: round(v[0] / max(v[1], 1), 4) for k, v in phases.items() if v[1]},
                 "commutator_ms": round(sum(v[0] for v in phases.values()) / nprof, 4)})
    del dH, dE, dR

    # ---- CPU restatement of the reference on the host cores (rank 0, N=1)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        dt, cores, blas, _, state = cpu_commutators(args.emax, 0, args.cpu_steps, reference=args.reference)
        cpu = {"value": args.cpu_steps / dt, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{args.cpu_steps} full [eta,H] commutators at eMax={args.emax} on the "
                         f"{state['reference'].upper()} state (FP64 restatement, OpenMP x{cores}, {blas})"}

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms_max / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "tf32" if args.mode == "tf32x3" else "bf16", "data": "synthetic",
            "config": {
                "workload": flow_workload_name(args, b.norbits),
                "emax": args.emax, "ds": args.ds,
                "step": "one Magnus step, one CUDA-graph replay",
                "precision": f"{args.mode}: " + ("TF32-compensated" if args.mode == "tf32x3" else "split-BF16") +
                             " tcgen05 channel GEMMs, FP32 accumulate, FP32 gathers, FP64 operators, E0 and norms",
                "parallelism": f"replicas x{world}",
                "l2": "inputs larger than L2 (0.27 GiB per operator; the recoupling input X 0.73 GiB)",
                "reference_state": hf_rec, "autotune": tune,
                "timed": timed, "warmup_E0": e0_steps,
                "fp64_commutators_per_s": fp64_rate * world if fp64_rate else None,
                "speedup_vs_fp64": value / (fp64_rate * world) if fp64_rate else None, **cmp,
            },
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 3 * nbytes,
                    "d2h_bytes_per_step": 3 * nbytes, "steps": args.e2e_steps, "commutators": e2e_comm},
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": launches_all,
        }
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
