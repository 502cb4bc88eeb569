"""Magnus-expansion IMSRG flow on the GB300 engine.

Restates magnus_decouple (src/IMSRG_MAGNUS.f90:15-128): eta(0) from the generator,
then per step MAGNUS_EXPAND -> euler_step -> BCH_EXPAND from the bare Hamiltonian ->
generator -> MBPT(2) convergence measure.  Every operator stays on the device; only
scalars (norms, E0, MBPT2) come back to the host.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

from .engine import CONV, Engine


def omega_checkpoint_name(prefix: str, s: float) -> str:
    """File name of the Omega checkpoint at flow parameter s, as write_omega_checkpoint builds it
    (src/basic_IMSRG.f90:3215-3251): the prefix cut after 'hwHO0' and two more characters (or
    after 'hw' and two more), then '_s' and s in six characters with three decimals."""
    k = prefix.find("hwHO0")
    cut = k + 7 if k >= 0 else prefix.find("hw") + 4
    if cut < 4:
        raise ValueError("the prefix names no hw value")
    txt = f"{s:6.3f}".strip()
    if s < 10.0:
        txt += "0"
    return f"{prefix[:cut]}_s{txt}.bin"


def latest_omega_checkpoint(directory: str, prefix: str, ds: float = 0.5, s_top: float = 95.5):
    """(path, s) of the newest checkpoint, searched from s = 95.5 down in steps of ds as
    read_omega_checkpoint does (src/basic_IMSRG.f90:3300-3330), or None."""
    s = s_top
    while s > 1.0:
        path = os.path.join(directory, omega_checkpoint_name(prefix, s))
        if os.path.exists(path):
            return path, s
        s -= ds
    return None


def checkpoint_interval(emax: int) -> int:
    """Steps between checkpoints (src/IMSRG_MAGNUS.f90:55-61)."""
    return 12 if emax == 14 else (4 if emax > 14 else 24)


@dataclass
class FlowResult:
    steps: list = field(default_factory=list)  # (step, s, E0, E0 + MBPT2, |MBPT2|, magnus terms, bch terms)

    @property
    def E0(self) -> float:
        return self.steps[-1][2] if self.steps else float("nan")


def magnus_decouple(eng: Engine, H0: np.ndarray, ds: float = 0.5, s_max: float | None = None,
                    max_steps: int | None = None, crit_stop: float = float(np.float32(1e-6)),
                    bch_max_terms: int = 40, bch_conv: float = CONV, generator: str = "white",
                    ops: dict | None = None, graph: bool = False, checkpoint: tuple | None = None,
                    checkpoint_every: int | None = None) -> FlowResult:
    """Flow the Hamiltonian H0 (host slab, herm +1) to s_max / max_steps / |MBPT2| < crit.

    graph=True runs each step as one replay of the CUDA graph of imsrg_magnus_step
    (same operators as the eager step, bit for bit).

    checkpoint=(directory, prefix) follows the reference's checkpointing: on entry the newest
    Omega checkpoint is read, H(s) rebuilt by BCH_EXPAND and the flow resumes there; every
    checkpoint_every steps (default: the reference's interval for eMax) Omega is written at
    the start of the step, the first one after a restart skipped, and the file written
    checkpoint_every steps earlier removed."""
    gens = {"white": eng.build_gs_white, "atan": eng.build_gs_atan, "w2": eng.build_gs_w2}
    if generator not in gens:
        raise ValueError(f"generator must be one of {sorted(gens)}")
    if graph and generator != "white":
        raise ValueError("the CUDA-graph step builds the White generator; use graph=False for atan / w2")
    build = gens[generator]
    HS = eng.new_op(1, H0)          # evolved Hamiltonian
    H = eng.new_op(1)               # bare Hamiltonian
    eng.copy_sq_op(HS, H)
    G = eng.new_op(-1)              # Omega
    DG = eng.new_op(-1)             # eta, then dOmega
    build(HS, DG)
    res = FlowResult()
    s, steps = 0.0, 0
    chk = checkpoint_every or checkpoint_interval(eng.basis.eMax)
    first = False
    found = latest_omega_checkpoint(checkpoint[0], checkpoint[1], ds) if checkpoint else None
    if found:  # checkpoint restart (src/IMSRG_MAGNUS.f90:73-84)
        eng.read_omega_checkpoint(G, found[0])
        eng.bch_expand(HS, G, H, bch_max_terms, bch_conv)
        build(HS, DG)
        s = found[1]
        steps = int(round(s / ds))
        first = True
    e2 = eng.mbpt2(HS)
    crit = abs(e2)
    res.steps.append((steps, s, HS.E0, HS.E0 + e2, crit, 0, 0))
    while crit > crit_stop:
        if max_steps is not None and steps >= max_steps:
            break
        if s_max is not None and s >= s_max - 1e-12:
            break
        steps += 1
        if checkpoint and steps % chk == 0:
            if first:
                first = False
            else:
                eng.write_omega_checkpoint(G, os.path.join(checkpoint[0], omega_checkpoint_name(checkpoint[1], s)))
                old = os.path.join(checkpoint[0], omega_checkpoint_name(checkpoint[1], s - chk * ds)) \
                    if s - chk * ds > 0 else None
                if old and os.path.exists(old):
                    os.remove(old)
        if graph:
            info = eng.magnus_step(HS, G, DG, H, ds, bch_max_terms, bch_conv, graph=True)
            s += ds
            e2, e0, nm, nb = info["mbpt2"], info["E0"], info["magnus_terms"], info["bch_terms"]
        else:
            nm = eng.magnus_expand(DG, G)
            s = eng.euler_step(G, DG, s, ds)
            nb = eng.bch_expand(HS, G, H, bch_max_terms, bch_conv)
            build(HS, DG)
            e2 = eng.mbpt2(HS)
            e0 = HS.E0
        crit = abs(e2)
        res.steps.append((steps, s, e0, e0 + e2, crit, nm, nb))
    if ops is not None:
        ops.update(HS=HS, G=G)
    return res


def magnus_triples(eng: Engine, H0: np.ndarray, G, E0: float, kind: str = "y", prefix: str | None = None,
                   output_dir: str = ".") -> tuple:
    """The driver's triples step after the flow (src/main_IMSRG.f90:294-318): restore_triples of
    the flow's starting Hamiltonian H0 (host slab) and Omega G (device operator), kind 'y', or of
    CR_EXPAND(Omega, H0) and Omega, kind 'C' (completely renormalised).  Returns
    (E0, E0 + correction); with prefix set, writes them to <output_dir>/<prefix>_magnus_triples.dat
    or _magnus_cr_triples.dat as the reference does ('(2(e15.7))')."""
    if kind not in ("y", "C"):
        raise ValueError("kind must be 'y' or 'C'")
    H = eng.new_op(1, H0)
    if kind == "C":
        CR = eng.new_op(1)
        eng.cr_expand(CR, G, H, 14, CONV)
        H = CR
    corr, _ = eng.restore_triples(H, G)
    if prefix is not None:
        name = f"{prefix.strip()}_magnus_triples.dat" if kind == "y" else f"{prefix.strip()}_magnus_cr_triples.dat"
        with open(os.path.join(output_dir, name), "w") as f:
            f.write(f"{_e15_7(E0)}{_e15_7(E0 + corr)}\n")
    return E0, E0 + corr


def _e15_7(x: float) -> str:
    """Fortran's e15.7 edit descriptor: 0.ddddddd E+xx, right-justified in 15 columns."""
    if x == 0.0:
        return f"{'0.0000000E+00':>15}"
    exp = int(np.floor(np.log10(abs(x)))) + 1
    v = round(abs(x) / 10.0 ** exp, 7)
    if v >= 1.0:  # rounding carried into a new digit
        v /= 10.0
        exp += 1
    s = f"{'-' if x < 0 else ''}0.{int(round(v * 1e7)):07d}E{'+' if exp >= 0 else '-'}{abs(exp):02d}"
    return f"{s:>15}"
