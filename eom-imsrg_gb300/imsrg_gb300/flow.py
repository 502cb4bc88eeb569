"""Magnus-expansion IMSRG flow on the GB300 engine.

Restates magnus_decouple (src/IMSRG_MAGNUS.f90:15-128): eta(0) from the generator,
then per step MAGNUS_EXPAND -> euler_step -> BCH_EXPAND from the bare Hamiltonian ->
generator -> MBPT(2) convergence measure.  Every operator stays on the device; only
scalars (norms, E0, MBPT2) come back to the host.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .engine import CONV, Engine


@dataclass
class FlowResult:
    steps: list = field(default_factory=list)  # (step, s, E0, E0 + MBPT2, |MBPT2|, magnus terms, bch terms)

    @property
    def E0(self) -> float:
        return self.steps[-1][2] if self.steps else float("nan")


def magnus_decouple(eng: Engine, H0: np.ndarray, ds: float = 0.5, s_max: float | None = None,
                    max_steps: int | None = None, crit_stop: float = float(np.float32(1e-6)),
                    bch_max_terms: int = 40, bch_conv: float = CONV, generator: str = "white",
                    ops: dict | None = None, graph: bool = False) -> FlowResult:
    """Flow the Hamiltonian H0 (host slab, herm +1) to s_max / max_steps / |MBPT2| < crit.

    graph=True runs each step as one replay of the CUDA graph of imsrg_magnus_step
    (same operators as the eager step, bit for bit)."""
    if generator != "white":
        raise ValueError("only the White generator is implemented")
    HS = eng.new_op(1, H0)          # evolved Hamiltonian
    H = eng.new_op(1)               # bare Hamiltonian
    eng.copy_sq_op(HS, H)
    G = eng.new_op(-1)              # Omega
    DG = eng.new_op(-1)             # eta, then dOmega
    eng.build_gs_white(HS, DG)
    res = FlowResult()
    s, steps = 0.0, 0
    e2 = eng.mbpt2(HS)
    crit = abs(e2)
    res.steps.append((0, s, HS.E0, HS.E0 + e2, crit, 0, 0))
    while crit > crit_stop:
        if max_steps is not None and steps >= max_steps:
            break
        if s_max is not None and s >= s_max - 1e-12:
            break
        steps += 1
        if graph:
            info = eng.magnus_step(HS, G, DG, H, ds, bch_max_terms, bch_conv, graph=True)
            s += ds
            e2, e0, nm, nb = info["mbpt2"], info["E0"], info["magnus_terms"], info["bch_terms"]
        else:
            nm = eng.magnus_expand(DG, G)
            s = eng.euler_step(G, DG, s, ds)
            nb = eng.bch_expand(HS, G, H, bch_max_terms, bch_conv)
            eng.build_gs_white(HS, DG)
            e2 = eng.mbpt2(HS)
            e0 = HS.E0
        crit = abs(e2)
        res.steps.append((steps, s, e0, e0 + e2, crit, nm, nb))
    if ops is not None:
        ops.update(HS=HS, G=G)
    return res
