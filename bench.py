#!/usr/bin/env python
"""Benchmark of the GB300 IMSRG(2) commutator engine.

Workload (one "step"): one full two-body-truncated commutator [eta, H] at eMax=10
(132 j-orbits, 16O-like reference, 132 (J,parity,Tz) channels, 88 cross-coupled
channels), eta the White generator of a seeded synthetic Hamiltonian -- the unit of
the reference's Magnus/BCH loop (src/IMSRG_MAGNUS.f90:207-219).

Prints one JSON line.  `value` is mixed-precision (split-BF16 tcgen05) commutators/s
with operators resident in HBM; `e2e` is the same metric through the C ABI with the
operators uploaded from / downloaded to pinned host memory every step.  With
--impl reference the CPU restatement of the reference algorithm (FP64, OpenMP on all
host cores, BLAS dgemm) is timed on the same workload instead.
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
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = f"/tmp/imsrg_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for k, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(k)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


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


def cpu_commutators(emax: int, n_warm: int, n_steps: int, seed: int = 1):
    """Time the CPU restatement of the reference on one [eta, H] commutator per step."""
    from oracle import oracle as orc
    from imsrg_gb300 import Engine, make_basis
    b = make_basis(emax)
    host = Engine(b, device=-1)
    H = host.synthetic_hamiltonian(seed=seed)
    o = orc.Oracle(b)
    cores = os.cpu_count() or 1
    orc.set_threads(cores)
    addr, ilp64, blas_name, keep = find_blas_dgemm()
    if addr:
        orc.use_blas_dgemm(addr, ilp64)
    eta = o.white(H, 1)
    for _ in range(n_warm):
        o.commutator(eta, -1, H, 1, 1)
    t = time.perf_counter()
    for _ in range(n_steps):
        o.commutator(eta, -1, H, 1, 1)
    dt = time.perf_counter() - t
    return dt, cores, blas_name, keep


# ---------------------------------------------------------------- roofline bookkeeping
def algorithmic_work(eng, mode: str, phase: str):
    """Algorithmic bytes (or FLOPs) of one launch of a phase at this basis."""
    S = {"bf16x3": 3, "bf16x6": 6, "fp64": 1}[mode]          # slice products per GEMM
    slices = {"bf16x3": 2, "bf16x6": 3, "fp64": 1}[mode]
    info = eng.block_info()
    A = eng.basis.nholes
    P = eng.basis.norbits - A
    n2b = eng.slab - (1 + A * A + P * P + P * A)
    cc = eng.cc_info()
    if phase == "recouple":   # read Z once (FP32) + read and write the 2b part of RES (FP64)
        return "hbm", eng.wcc_size * 4 + 2 * 8 * n2b
    if phase == "c122":       # read L and R once, write the 2b part of RES
        return "hbm", 2 * 8 * eng.slab + 8 * n2b
    if phase == "ph_gemm":    # Z written once in FP32 (the product itself is K<=90)
        return "hbm", eng.wcc_size * 4
    if phase == "pphh_gemm":  # sum 2 M N K over the K = npp products, times slice products
        f = 0
        for q in range(eng.nblocks):
            np_, nb, nh = int(info["npp"][q]), int(info["nph"][q]), int(info["nhh"][q])
            if np_ == 0:
                continue
            f += 2 * np_ * np_ * np_ + 2 * nh * nh * np_ + 2 * 2 * np_ * nh * np_
            f += 2 * nb * nb * np_ + 2 * 2 * np_ * nb * np_ + 2 * 2 * nb * nh * np_
        return "tensor", f * S
    if phase == "pandya":     # two operators read, LCC and RCC written once
        return "hbm", 2 * 8 * eng.slab + 2 * 2 * slices * int((cc["rlen"] * cc["nph"]).sum())
    return None, None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--emax", type=int, default=10)
    ap.add_argument("--mode", default="bf16x6", choices=["bf16x3", "bf16x6"])
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--flow-steps", type=int, default=3)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    world, rank, local, pg = dist_setup()

    if args.impl == "reference":
        if rank != 0:
            return
        dt, cores, blas, _ = cpu_commutators(args.emax, args.warmup, args.steps)
        v = args.steps / dt
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"one [eta,H] IMSRG(2) commutator, eMax={args.emax}", "emax": args.emax,
                       "path": "CPU restatement of the reference (FP64, OpenMP)", "blas": blas},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} full commutators at eMax={args.emax}"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }), flush=True)
        return

    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300.flow import magnus_decouple
    import numpy as np

    b = make_basis(args.emax)
    eng = Engine(b, device=local, precision=args.mode)
    H = eng.synthetic_hamiltonian(seed=1)
    dH = eng.new_op(1, H)
    dE = eng.new_op(-1)
    dR = eng.new_op(1)
    eng.build_gs_white(dH, dE)

    # ---- device-resident timing (the headline value)
    for _ in range(max(args.warmup, 3)):
        eng.commutator(dE, dH, dR)
    eng.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(pg)
    eng.synchronize()
    l0 = eng.launch_count()
    eng.timer_begin()
    for _ in range(args.steps):
        eng.commutator(dE, dH, dR)
    ms = eng.timer_end()
    eng.synchronize()
    launches = eng.launch_count() - l0
    barrier(pg)
    clk = clocks.stop()
    ms_max = allreduce_max(pg, ms)
    launches_all = int(allreduce_sum(pg, launches))
    value = world * args.steps / (ms_max * 1e-3)

    # ---- plain FP64 GPU path on the same inputs
    eng64 = Engine(b, device=local, precision="fp64")
    dH64 = eng64.new_op(1, H)
    dE64 = eng64.new_op(-1)
    dR64 = eng64.new_op(1)
    eng64.build_gs_white(dH64, dE64)
    eng64.commutator(dE64, dH64, dR64)
    eng64.timer_begin()
    for _ in range(args.fp64_steps):
        eng64.commutator(dE64, dH64, dR64)
    ms64 = eng64.timer_end() / args.fp64_steps
    fp64_rate = 1e3 / ms64
    R_mixed, R_64 = dR.download(), dR64.download()
    comm_dE0 = abs(R_mixed[0] - R_64[0])
    comm_rel = float(np.max(np.abs(R_mixed - R_64)) / np.max(np.abs(R_64)))
    del dH64, dE64, dR64

    # ---- end to end through the C ABI: pinned host operators in, result out, every step
    nbytes = 8 * eng.slab
    hbuf = []
    for _ in range(3):
        p = C.c_void_p()
        eng._ck(eng.L.imsrg_pinned_alloc(nbytes, C.byref(p)))
        hbuf.append(p)
    hE = np.ctypeslib.as_array(C.cast(hbuf[0], C.POINTER(C.c_double)), shape=(eng.slab,))
    hH = np.ctypeslib.as_array(C.cast(hbuf[1], C.POINTER(C.c_double)), shape=(eng.slab,))
    hE[:] = dE.download()
    hH[:] = H
    e2e_steps = max(3, args.steps // 2)
    for it in range(e2e_steps + 1):
        if it == 1:
            barrier(pg)
            t0 = time.perf_counter()
        eng._ck(eng.L.imsrg_op_upload_slab(eng.h, dE.h, hbuf[0]))
        eng._ck(eng.L.imsrg_op_upload_slab(eng.h, dH.h, hbuf[1]))
        eng.commutator(dE, dH, dR)
        eng._ck(eng.L.imsrg_op_download_slab(eng.h, dR.h, hbuf[2]))
    e2e_s = allreduce_max(pg, time.perf_counter() - t0)
    e2e_value = world * e2e_steps / e2e_s
    for p in hbuf:
        eng.L.imsrg_pinned_free(p)

    # ---- per-phase event timing (separate pass) for the roofline of the dominant kernel
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
    bound, work = algorithmic_work(eng, args.mode, dom)
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
    roof.update({"traffic": traffic, "kernel_phase": dom, "kernel_ms": dom_ms,
                 "algorithmic": work, "peak_source": "measured" if peaks else "fallback",
                 "phases_ms": {k: round(v[0] / max(v[1], 1), 4) for k, v in phases.items() if v[1]}})

    # ---- |dE0| of a short Magnus flow, mixed vs plain FP64
    flow = {}
    if args.flow_steps > 0:
        r_mixed = magnus_decouple(eng, H, max_steps=args.flow_steps)
        eng64b = Engine(b, device=local, precision="fp64")
        r_64 = magnus_decouple(eng64b, H, max_steps=args.flow_steps)
        flow = {"flow_steps": args.flow_steps, "E0_mixed": r_mixed.E0, "E0_fp64": r_64.E0,
                "dE0_keV": abs(r_mixed.E0 - r_64.E0) * 1e3}
        del eng64b

    # ---- CPU restatement of the reference on the host cores (rank 0, N=1)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        dt, cores, blas, _ = cpu_commutators(args.emax, 0, args.cpu_steps)
        cpu = {"value": args.cpu_steps / dt, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{args.cpu_steps} full [eta,H] commutators at eMax={args.emax} "
                         f"(FP64 restatement, OpenMP x{cores}, {blas})"}

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {
                "workload": f"one [eta,H] IMSRG(2) commutator, eMax={args.emax} (132 orbits, 16O-like), "
                            "seeded synthetic Hamiltonian + White generator",
                "emax": args.emax, "precision": f"{args.mode}: split-BF16 tcgen05 channel GEMMs, FP32 accumulate, "
                                                "FP32 gathers, FP64 operators and E0",
                "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (0.27 GiB operators, 0.78 GiB Z)",
                "fp64_commutators_per_s": fp64_rate * world, "speedup_vs_fp64": value / (fp64_rate * world),
                "commutator_dE0_keV": comm_dE0 * 1e3, "commutator_max_rel_err": comm_rel, **flow,
            },
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * nbytes, "d2h_bytes_per_step": nbytes},
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": launches_all,
        }
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
