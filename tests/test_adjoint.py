"""Reverse mode of the commutator, the generator and the Magnus flow, on the CPU.

The oracle's transposes (oracle/oracle.cpp, reverse-mode section) are checked against its
forward routines: for the bilinear commutator, <Cb, [dL, R]> = <Lb, dL> and
<Cb, [L, dR]> = <Rb, dR> for independent random directions, on hermitian and on arbitrary
slabs; the White generator's transpose against central differences.  The product's flow
adjoint (imsrg_gb300.adjoint) is run over an oracle-backed backend and checked against
central finite differences of the same fixed-plan flow.
"""
import numpy as np
import pytest

from helpers import rel_err


class OracleOp:
    def __init__(self, a, herm):
        self.a = a
        self.herm = herm


class OracleBackend:
    """The adjoint's backend interface over the CPU oracle (test-only)."""

    def __init__(self, o):
        self.o = o
        self.slab = o.slab

    def new(self, herm, slab=None):
        return OracleOp(np.zeros(self.slab) if slab is None else np.array(slab, dtype=np.float64), herm)

    def download(self, x):
        return x.a.copy()

    def copy(self, x):
        return OracleOp(x.a.copy(), x.herm)

    def axpby(self, A, a, B, b, out):
        out.a[:] = A.a * a + B.a * b

    def dot(self, A, B):
        return float(A.a @ B.a)

    def e0(self, x):
        return float(x.a[0])

    def commutator(self, L, R, herm_res, e0):
        return OracleOp(self.o.commutator_e0(L.a, L.herm, R.a, R.herm, herm_res, e0), herm_res)

    def commutator_vjp(self, L, R, RESb, Lb, Rb, e0):
        lb, rb = self.o.commutator_vjp(L.a, L.herm, R.a, R.herm, RESb.herm, e0, RESb.a)
        Lb.a += lb
        Rb.a += rb

    def white(self, H):
        return OracleOp(self.o.white(H.a, H.herm), -1)

    def white_vjp(self, H, ETAb, Hb):
        Hb.a += self.o.white_vjp(H.a, H.herm, ETAb.a)

    def magnus_expand(self, DG, G):
        return self.o.magnus_expand(DG.a, G.a)

    def bch_expand(self, HS, G, H, max_terms, conv):
        hs, n = self.o.bch_expand(G.a, H.a, max_terms, conv)
        if n < 0:
            raise RuntimeError("BCH did not converge")
        HS.a[:] = hs
        HS.herm = H.herm
        return n


HERMS = [(-1, 1, 1, True), (-1, -1, -1, False), (1, 1, -1, True), (1, -1, 1, False)]


@pytest.mark.parametrize("emax", [2, 4])
@pytest.mark.parametrize("hL,hR,hRES,e0", HERMS)
def test_commutator_transpose(oracles, emax, hL, hR, hRES, e0):
    o = oracles(emax)
    rng = np.random.default_rng(emax * 10 + hL + 2 * hR)
    for valid in (True, False):
        if valid:
            L, R, Cb = o.random(3, hL), o.random(4, hR), o.random(5, hRES)
            dL, dR = o.random(6, hL), o.random(7, hR)
        else:
            L, R, Cb, dL, dR = (rng.standard_normal(o.slab) for _ in range(5))
        Lb, Rb = o.commutator_vjp(L, hL, R, hR, hRES, e0, Cb)
        fL = Cb @ o.commutator_e0(dL, hL, R, hR, hRES, e0)
        fR = Cb @ o.commutator_e0(L, hL, dR, hR, hRES, e0)
        assert abs(Lb @ dL - fL) <= 1e-12 * max(abs(fL), 1.0)
        assert abs(Rb @ dR - fR) <= 1e-12 * max(abs(fR), 1.0)


@pytest.mark.parametrize("emax", [2, 4])
def test_white_transpose_vs_fd(oracles, emax):
    from imsrg_gb300 import Engine, make_basis
    o = oracles(emax)
    H = Engine(make_basis(emax), device=-1).synthetic_hamiltonian(seed=2)
    rng = np.random.default_rng(emax)
    Eb = rng.standard_normal(o.slab)
    D = o.random(7, 1) * 1e-2
    Hb = o.white_vjp(H, 1, Eb)
    h = 1e-4
    fd = (Eb @ o.white(H + h * D, 1) - Eb @ o.white(H - h * D, 1)) / (2 * h)
    assert abs(fd - Hb @ D) <= 1e-8 * abs(fd)


def test_channel_perturbations_are_hermitian(oracles):
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300.adjoint import channel_perturbations
    from helpers import sections
    o = oracles(4)
    eng = Engine(make_basis(4), device=-1)
    V = channel_perturbations(eng, 3, sigma=0.1, seed=5)
    info = eng.block_info()
    ncls = np.stack([info["npp"], info["nph"], info["nhh"]], axis=1)
    sea1, sea2 = (0, 0, 0, 1, 2, 1), (0, 1, 2, 1, 2, 2)
    for v in V:
        e0, one, two = sections(o, v)
        assert e0 == 0.0 and not one.any()
        off = 0
        for q in range(eng.nblocks):
            for g in range(6):
                n1, n2 = int(ncls[q][sea1[g]]), int(ncls[q][sea2[g]])
                X = two[off:off + n1 * n2].reshape(n1, n2, order="F")
                if g in (0, 3, 4):
                    assert np.array_equal(X, X.T)
                off += n1 * n2
        assert 0.05 < np.std(two[two != 0.0]) < 0.2
        # the oracle sees a hermitian operator: its commutator with itself vanishes
        assert np.max(np.abs(o.commutator(v, 1, v, 1))) < 1e-12
    assert not np.allclose(V[0], V[1])


def test_flow_gradient_matches_central_differences(oracles):
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300.adjoint import MagnusFlowAdjoint, channel_perturbations
    o = oracles(2)
    eng = Engine(make_basis(2), device=-1)
    H0 = eng.synthetic_hamiltonian(seed=3)
    V = channel_perturbations(eng, 3, sigma=0.1, seed=4)
    fl = MagnusFlowAdjoint(OracleBackend(o), H0, V, ds=0.5, steps=4, bch_conv=1e-10)
    theta = np.zeros(3)
    plan = fl.plan(theta)
    assert plan.commutators > 0
    e0 = fl.forward(theta, plan)
    g = fl.gradient()
    h = 1e-4
    fd = np.zeros(3)
    for k in range(3):
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd[k] = (fl.forward(tp, plan) - fl.forward(tm, plan)) / (2 * h)
    assert np.isfinite(e0)
    assert rel_err(g, fd) < 1e-6, (g, fd)
