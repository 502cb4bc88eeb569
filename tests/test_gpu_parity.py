"""FP64 GPU path against the CPU oracle, piece by piece, through the C ABI.

Bar: 1e-10 relative (max abs difference over the max magnitude of the array group),
the tolerance the plain FP64 path is held to against the reference restatement.
"""
import numpy as np
import pytest

from helpers import rel_err, sections

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _ops(o, eng, seed, hL, hR, scale=1.0):
    L = o.random(seed, hL) * scale
    R = o.random(seed + 1, hR) * scale
    return L, R, eng.new_op(hL, L), eng.new_op(hR, R)


def _check(name, x, ref, o, tol=TOL):
    e0, ob, tb = sections(o, x)
    r0, rob, rtb = sections(o, ref)
    assert abs(e0 - r0) <= tol * max(1.0, abs(r0)), (name, "E0", e0, r0)
    assert rel_err(ob, rob) <= tol, (name, "1b", rel_err(ob, rob))
    assert rel_err(tb, rtb) <= tol, (name, "2b", rel_err(tb, rtb))


@pytest.mark.parametrize("emax", [2, 4, 6])
@pytest.mark.parametrize("hL,hR", [(-1, 1), (1, 1), (-1, -1)])
def test_pieces(oracles, engines, emax, hL, hR):
    o, eng = oracles(emax), engines(emax)
    hRES = -hL * hR
    L, R, dL, dR = _ops(o, eng, 100 + emax, hL, hR)
    # 0-body
    assert abs(eng.commutator_110(dL, dR) - o.commutator_110(L, hL, R, hR)) <= TOL * max(1, abs(o.commutator_110(L, hL, R, hR)))
    assert abs(eng.commutator_220(dL, dR) - o.commutator_220(L, hL, R, hR)) <= TOL * max(1, abs(o.commutator_220(L, hL, R, hR)))
    # 111 assigns the one-body part; 121 accumulates; 122 assigns the two-body part
    start = o.random(7, hRES)
    ref = start.copy()
    dRES = eng.new_op(hRES, start)
    o.commutator_111(L, hL, R, hR, ref, hRES)
    eng.commutator_111(dL, dR, dRES)
    _check("111", dRES.download(), ref, o)
    o.commutator_121(L, hL, R, hR, ref, hRES)
    eng.commutator_121(dL, dR, dRES)
    _check("121", dRES.download(), ref, o)
    o.commutator_122(L, hL, R, hR, ref, hRES)
    eng.commutator_122(dL, dR, dRES)
    _check("122", dRES.download(), ref, o)
    # 222_pp_hh fills w1/w2 and accumulates; 221 reads them
    w1, w2 = o.new(), o.new()
    dw1, dw2 = eng.new_op(1), eng.new_op(1)
    o.commutator_222_pp_hh(L, hL, R, hR, ref, hRES, w1, w2)
    eng.commutator_222_pp_hh(dL, dR, dRES, dw1, dw2)
    _check("pphh w1", dw1.download(), w1, o)
    _check("pphh w2", dw2.download(), w2, o)
    _check("pphh", dRES.download(), ref, o)
    o.commutator_221(L, hL, R, hR, ref, hRES, w1, w2)
    eng.commutator_221(dL, dR, dRES, dw1, dw2)
    _check("221", dRES.download(), ref, o)
    # Pandya transforms and the particle-hole channel
    LCC, RCC = o.calculate_cross_coupled(L, hL), o.calculate_cross_coupled(R, hR)
    dLCC, dRCC, dWCC = eng.new_cc(0), eng.new_cc(0), eng.new_cc(1)
    eng.calculate_cross_coupled(dL, dLCC)
    eng.calculate_cross_coupled(dR, dRCC)
    assert rel_err(dLCC.download(), LCC) <= TOL and rel_err(dRCC.download(), RCC) <= TOL
    WCC = o.commutator_222_ph(LCC, hL, RCC, hR, ref, hRES)
    eng.commutator_222_ph(dLCC, dRCC, dRES, dWCC)
    assert rel_err(dWCC.download(), WCC) <= TOL
    _check("222_ph", dRES.download(), ref, o)


@pytest.mark.parametrize("emax", [2, 4, 6])
def test_full_commutator(oracles, engines, emax):
    o, eng = oracles(emax), engines(emax)
    L, R, dL, dR = _ops(o, eng, 300 + emax, -1, 1)
    ref = o.commutator(L, -1, R, 1, 1)
    dRES = eng.new_op(1)
    eng.commutator(dL, dR, dRES)
    _check("full", dRES.download(), ref, o)


@pytest.mark.parametrize("emax", [2, 4])
def test_generator_norms_flow(oracles, engines, emax):
    o, eng = oracles(emax), engines(emax)
    H = eng.synthetic_hamiltonian(seed=5)
    dH = eng.new_op(1, H)
    dE = eng.new_op(-1)
    eng.build_gs_white(dH, dE)
    eta = o.white(H, 1)
    _check("white", dE.download(), eta, o)
    assert abs(eng.mat_frob_norm(dE) - o.frob(eta)) <= 1e-12 * o.frob(eta)
    assert abs(eng.mbpt2(dH) - o.mbpt2(H, 1)) <= 1e-12 * abs(o.mbpt2(H, 1))
    # one Magnus step: dOmega from eta, Euler step, BCH rebuild of H(s)
    G = o.random(9, -1) * 1e-3
    dG = eng.new_op(-1, G)
    DG = eta.copy()
    used = o.magnus_expand(DG, G)
    dDG = eng.new_op(-1, eta)
    assert eng.magnus_expand(dDG, dG) == used
    _check("magnus", dDG.download(), DG, o)
    HS, n = o.bch_expand(G, H)
    dHS = eng.new_op(1)
    assert eng.bch_expand(dHS, dG, dH) == n
    _check("bch", dHS.download(), HS, o)


@pytest.mark.parametrize("emax", [2, 4])
def test_cr_expand(oracles, engines, emax):
    """CR_EXPAND (src/IMSRG_MAGNUS.f90:532-617) against the oracle: same terms, 1e-10."""
    o, eng = oracles(emax), engines(emax)
    G = o.random(81, -1) * 0.05
    H = o.random(82, 1)
    ref, n = o.cr_expand(G, H, 14, 1e-6)
    dG, dH, dHS = eng.new_op(-1, G), eng.new_op(1, H), eng.new_op(1)
    assert eng.cr_expand(dHS, dG, dH, 14, 1e-6) == n
    assert rel_err(dHS.download(), ref) < TOL
    # the capped series ends without an error
    assert eng.cr_expand(dHS, eng.new_op(-1, G * 40), dH, 14, 1e-30) == 13


@pytest.mark.parametrize("emax", [2, 4])
def test_quadrupoles(oracles, engines, emax):
    """restore_quadrupoles and BCH_EXPAND with quads = 'y' (src/IMSRG_MAGNUS.f90:149-234, 908-1132)
    against the oracle, FP64, 1e-10."""
    o, eng = oracles(emax), engines(emax)
    X, OM = o.random(93, 1), o.random(94, -1) * 0.02
    dX, dOM, dQ = eng.new_op(1, X), eng.new_op(-1, OM), eng.new_op(1)
    eng.restore_quadrupoles(dX, dOM, dQ)
    assert rel_err(dQ.download(), o.restore_quadrupoles(X, 1, OM, -1)) < TOL
    ref, n = o.bch_expand_quads(OM, X, 40, 1e-6)
    dHS = eng.new_op(1)
    assert eng.bch_expand_quads(dHS, dOM, dX, 40, 1e-6) == n
    assert rel_err(dHS.download(), ref) < TOL
