"""Adjoint derivatives of the Magnus-flow ground-state energy, dE0/dtheta.

The Hamiltonian is H(theta) = H0 + sum_k theta_k V_k (slabs in the reference's sq_op
layout).  The flow is the loop of magnus_decouple (src/IMSRG_MAGNUS.f90:47-110) with the
White generator: per step MAGNUS_EXPAND (:620-691), euler_step (:754-764) and BCH_EXPAND
(:149-234) from the bare H, then build_gs_white (src/generators.f90:4-106).  E0 is the
zero-body part of H(s) after the last step.

The derivative is taken by reverse mode through that program with the numbers of nested
commutators of every series fixed by a first (planning) pass -- the reference's early
exits make E0 piecewise smooth in theta, and a fixed plan is the smooth branch the finite
differences see.  The reverse sweep keeps Omega(s) after every step as checkpoints and
recomputes the BCH and Magnus terms of one step at a time (about one forward pass of
extra commutators); each nested commutator is reversed with imsrg_commutator_vjp, the
generator with imsrg_white_vjp.  dE0/dtheta_k = <Hbar, V_k> in the slab inner product.

The backend is the device engine (EngineBackend); any object with the same methods can
drive the same algorithm.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .engine import CONV

# MAGNUS_EXPAND coefficients, the literals of src/IMSRG_MAGNUS.f90:646
MAGNUS_COF = (1.0, -0.5, .0833333333, 0.0, -0.00138888888, 0.0, 3.306878e-5)


class EngineBackend:
    """Device operators of one Engine (FP64 commutators) behind the adjoint's interface."""

    def __init__(self, eng):
        self.eng = eng
        self.slab = eng.slab

    def new(self, herm: int, slab: np.ndarray | None = None):
        return self.eng.new_op(herm, slab)

    def download(self, x) -> np.ndarray:
        return x.download()

    def copy(self, x):
        y = self.eng.new_op(x.herm)
        self.eng.copy_sq_op(x, y)
        return y

    def axpby(self, A, a: float, B, b: float, out):
        self.eng.add_sq_op(A, float(a), B, float(b), out)

    def dot(self, A, B) -> float:
        return self.eng.dot(A, B)

    def e0(self, x) -> float:
        return x.E0

    def commutator(self, L, R, herm_res: int, e0: bool):
        out = self.eng.new_op(herm_res)
        self.eng.commutator(L, R, out, e0)
        return out

    def commutator_vjp(self, L, R, RESb, Lb, Rb, e0: bool):
        self.eng.commutator_vjp(L, R, RESb, Lb, Rb, e0)

    def white(self, H):
        eta = self.eng.new_op(-1)
        self.eng.build_gs_white(H, eta)
        return eta

    def white_vjp(self, H, ETAb, Hb):
        self.eng.white_vjp(H, ETAb, Hb)

    def magnus_expand(self, DG, G) -> int:
        return self.eng.magnus_expand(DG, G)

    def bch_expand(self, HS, G, H, max_terms: int, conv: float) -> int:
        return self.eng.bch_expand(HS, G, H, max_terms, conv)

    def synchronize(self):
        self.eng.synchronize()


@dataclass
class FlowPlan:
    """Nested commutators per step: magnus[k] for step k (from Omega_k), bch[k] for H(s_k+1)."""
    magnus: list = field(default_factory=list)
    bch: list = field(default_factory=list)

    @property
    def commutators(self) -> int:
        return int(sum(self.magnus) + sum(self.bch))


def channel_perturbations(eng, K: int, sigma: float = 0.1, seed: int = 1) -> list:
    """K seeded random hermitian two-body operators (slabs): N(0, sigma) MeV on every
    stored (J, parity, Tz) channel element, symmetric square blocks, zero for pairs of
    identical orbits at odd J (Pauli), no zero- or one-body part."""
    rng = np.random.default_rng(seed)
    info = eng.block_info()
    A = eng.basis.nholes
    P = eng.basis.norbits - A
    ncls = np.stack([info["npp"], info["nph"], info["nhh"]], axis=1)
    sea1, sea2 = (0, 0, 0, 1, 2, 1), (0, 1, 2, 1, 2, 2)
    square = (True, False, False, True, True, False)
    pairs = {}
    out = []
    for _ in range(K):
        v = np.zeros(eng.slab)
        o = 1 + A * A + P * P + P * A
        for q in range(eng.nblocks):
            Jodd = (int(info["lamJ"][q]) // 2) % 2 == 1
            for g in range(6):
                n1, n2 = int(ncls[q][sea1[g]]), int(ncls[q][sea2[g]])
                if n1 * n2:
                    X = rng.normal(0.0, sigma, size=(n1, n2))
                    if square[g]:
                        X = np.triu(X) + np.triu(X, 1).T
                    if Jodd:
                        for side, c in ((0, sea1[g]), (1, sea2[g])):
                            if (q, c) not in pairs:
                                pairs[(q, c)] = eng.block_pairs(q, c)
                            pr = pairs[(q, c)]
                            same = pr[:, 0] == pr[:, 1]
                            if side == 0:
                                X[same, :] = 0.0
                            else:
                                X[:, same] = 0.0
                    v[o:o + n1 * n2] = X.reshape(-1, order="F")
                o += n1 * n2
        out.append(v)
    return out


class MagnusFlowAdjoint:
    """E0 of a fixed-length Magnus flow of H(theta) = H0 + sum_k theta_k V_k and its gradient.

    steps Magnus steps of size ds (s_end = steps * ds); BCH_EXPAND keeps adding terms until
    the term norm drops below bch_conv (at most bch_max_terms), as in the reference."""

    def __init__(self, backend, H0: np.ndarray, V: list, ds: float = 0.5, steps: int = 60,
                 bch_max_terms: int = 40, bch_conv: float = CONV):
        self.be = backend
        self.ds = float(ds)
        self.steps = int(steps)
        self.bch_max_terms = int(bch_max_terms)
        self.bch_conv = float(bch_conv)
        self.H0 = backend.new(1, np.ascontiguousarray(H0, dtype=np.float64))
        self.V = [backend.new(1, np.ascontiguousarray(v, dtype=np.float64)) for v in V]
        self._omegas = None
        self._H = None
        self._plan = None

    # ---------------------------------------------------------------- forward pieces
    def hamiltonian(self, theta) -> object:
        H = self.be.copy(self.H0)
        for t, v in zip(np.asarray(theta, dtype=np.float64), self.V):
            if t != 0.0:
                self.be.axpby(H, 1.0, v, float(t), H)
        return H

    def _bch(self, G, H, nterms: int):
        """H(s) = sum_n ad_G^n(H) / n! with nterms nested commutators; returns (HS, terms, coefs)."""
        be = self.be
        terms, coefs = [H], [1.0]
        HS = be.copy(H)
        coef = 1.0
        for n in range(1, nterms + 1):
            coef = coef / float(n)
            A = be.commutator(G, terms[-1], 1, True)
            be.axpby(HS, 1.0, A, coef, HS)
            terms.append(A)
            coefs.append(coef)
        return HS, terms, coefs

    def _magnus(self, eta, G, nterms: int):
        """dOmega = sum_j cof_j ad_G^j(eta) with nterms nested commutators; returns (dOmega, terms)."""
        be = self.be
        terms = [eta]
        DG = be.copy(eta)
        for j in range(1, nterms + 1):
            B = be.commutator(G, terms[-1], -1, False)
            be.axpby(DG, 1.0, B, MAGNUS_COF[j], DG)
            terms.append(B)
        return DG, terms

    def plan(self, theta) -> FlowPlan:
        """Term counts of every series from the reference's own early exits at theta."""
        be = self.be
        H = self.hamiltonian(theta)
        DG = be.white(H)
        G = be.new(-1)
        plan = FlowPlan()
        for _ in range(self.steps):
            plan.magnus.append(be.magnus_expand(DG, G))
            be.axpby(G, 1.0, DG, self.ds, G)
            HS = be.new(1)
            plan.bch.append(be.bch_expand(HS, G, H, self.bch_max_terms, self.bch_conv))
            DG = be.white(HS)
        self._plan = plan
        return plan

    def forward(self, theta, plan: FlowPlan | None = None) -> float:
        """E0 after the flow with the term counts of `plan` (default: planned at theta);
        keeps Omega after every step for gradient()."""
        be = self.be
        if plan is None:
            plan = self.plan(theta) if self._plan is None else self._plan
        if len(plan.magnus) != self.steps:
            raise ValueError("plan does not match the number of steps")
        H = self.hamiltonian(theta)
        HS = H
        G = be.new(-1)
        omegas = [be.copy(G)]
        for k in range(self.steps):
            eta = be.white(HS)
            dG, _ = self._magnus(eta, G, plan.magnus[k])
            be.axpby(G, 1.0, dG, self.ds, G)
            omegas.append(be.copy(G))
            HS, _, _ = self._bch(G, H, plan.bch[k])
        self._omegas, self._H, self._plan = omegas, H, plan
        return be.e0(HS)

    # ---------------------------------------------------------------- reverse sweep
    def _bch_vjp(self, G, terms, coefs, HSb, Gb, Hb):
        """Gb += d<HSb, HS>/dG and Hb += d<HSb, HS>/dH for HS = sum_n coef_n ad_G^n(H)."""
        be = self.be
        T = len(terms) - 1
        Ab = be.new(1)
        be.axpby(Ab, 0.0, HSb, coefs[T], Ab)
        for n in range(T, 0, -1):
            prev = be.new(1)
            be.commutator_vjp(G, terms[n - 1], Ab, Gb, prev, True)
            be.axpby(prev, 1.0, HSb, coefs[n - 1], prev)
            Ab = prev
        be.axpby(Hb, 1.0, Ab, 1.0, Hb)

    def _magnus_vjp(self, G, terms, dGb, Gb):
        """Gb += d<dGb, dOmega>/dG; returns d<dGb, dOmega>/deta."""
        be = self.be
        m = len(terms) - 1
        Bb = be.new(-1)
        be.axpby(Bb, 0.0, dGb, MAGNUS_COF[m], Bb)
        for j in range(m, 0, -1):
            prev = be.new(-1)
            be.commutator_vjp(G, terms[j - 1], Bb, Gb, prev, False)
            be.axpby(prev, 1.0, dGb, MAGNUS_COF[j - 1], prev)
            Bb = prev
        return Bb

    def gradient_H(self):
        """Cotangent of the bare Hamiltonian slab, d E0 / d H (after forward())."""
        if self._omegas is None:
            raise RuntimeError("call forward() first")
        be, plan, om, H = self.be, self._plan, self._omegas, self._H
        N = self.steps
        Hb = be.new(1)
        Gb = be.new(-1)
        seed = np.zeros(be.slab)
        seed[0] = 1.0
        HSb = be.new(1, seed)
        if N == 0:
            return HSb
        _, terms, coefs = self._bch(om[N], H, plan.bch[N - 1])
        for k in range(N, 0, -1):
            # H(s_k) = BCH(Omega_k, H)
            self._bch_vjp(om[k], terms, coefs, HSb, Gb, Hb)
            # Omega_k = Omega_{k-1} + ds * MAGNUS_EXPAND(eta(H(s_{k-1})), Omega_{k-1})
            if k == 1:
                HSp, terms, coefs = H, None, None
            else:
                HSp, terms, coefs = self._bch(om[k - 1], H, plan.bch[k - 2])
            eta = be.white(HSp)
            _, bterms = self._magnus(eta, om[k - 1], plan.magnus[k - 1])
            dGb = be.new(-1)
            be.axpby(dGb, 0.0, Gb, self.ds, dGb)
            etab = self._magnus_vjp(om[k - 1], bterms, dGb, Gb)
            HSb = be.new(1)
            be.white_vjp(HSp, etab, HSb)
        be.axpby(Hb, 1.0, HSb, 1.0, Hb)   # H(s_0) = H
        return Hb

    def gradient(self) -> np.ndarray:
        """dE0/dtheta_k = <dE0/dH, V_k> (after forward())."""
        Hb = self.gradient_H()
        return np.array([self.be.dot(Hb, v) for v in self.V])


_FLOW_FN = None


def flow_energy(theta, flow: MagnusFlowAdjoint):
    """E0(theta) as a differentiable torch scalar: forward runs the flow on the device and
    keeps its checkpoints, backward runs the adjoint sweep (torch.autograd.Function)."""
    global _FLOW_FN
    import torch
    if _FLOW_FN is None:
        class _FlowE0(torch.autograd.Function):
            @staticmethod
            def forward(ctx, th, fl):
                e0 = fl.forward(th.detach().to("cpu", torch.float64).numpy())
                ctx.flow = fl
                ctx.th_meta = (th.dtype, th.device)
                return torch.tensor(e0, dtype=th.dtype, device=th.device)

            @staticmethod
            def backward(ctx, g):
                dtype, device = ctx.th_meta
                grad = torch.as_tensor(ctx.flow.gradient(), dtype=dtype, device=device)
                return g * grad, None

        _FLOW_FN = _FlowE0
    return _FLOW_FN.apply(theta, flow)
