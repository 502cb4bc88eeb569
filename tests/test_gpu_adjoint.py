"""Device reverse mode (imsrg_commutator_vjp, imsrg_white_vjp, imsrg_dot_sq_op) against the
oracle's transposes, and the device adjoint of the Magnus flow against central finite
differences of the FP64 forward flow and against the same adjoint run on the oracle."""
import numpy as np
import pytest

from helpers import rel_err
from test_adjoint import OracleBackend

pytestmark = pytest.mark.gpu

HERMS = [(-1, 1, 1, True), (-1, -1, -1, False), (1, 1, -1, True)]
TOL = 1e-10


@pytest.mark.parametrize("emax", [2, 4])
@pytest.mark.parametrize("hL,hR,hRES,e0", HERMS)
def test_commutator_vjp_matches_oracle(oracles, engines, emax, hL, hR, hRES, e0):
    o, eng = oracles(emax), engines(emax)
    rng = np.random.default_rng(3 + emax)
    for valid in (True, False):
        if valid:
            L, R, Cb = o.random(11, hL), o.random(12, hR), o.random(13, hRES)
        else:
            L, R, Cb = (rng.standard_normal(o.slab) for _ in range(3))
        Lb_ref, Rb_ref = o.commutator_vjp(L, hL, R, hR, hRES, e0, Cb)
        dL, dR, dC = eng.new_op(hL, L), eng.new_op(hR, R), eng.new_op(hRES, Cb)
        dLb, dRb = eng.new_op(hL), eng.new_op(hR)
        eng.commutator_vjp(dL, dR, dC, dLb, dRb, e0)
        assert rel_err(dLb.download(), Lb_ref) < TOL
        assert rel_err(dRb.download(), Rb_ref) < TOL
        # outputs accumulate
        eng.commutator_vjp(dL, dR, dC, dLb, dRb, e0)
        assert rel_err(dLb.download(), 2 * Lb_ref) < TOL


@pytest.mark.parametrize("emax", [2, 4])
def test_white_vjp_and_dot_match_oracle(oracles, engines, emax):
    o, eng = oracles(emax), engines(emax)
    H = eng.synthetic_hamiltonian(seed=8)
    Eb = np.random.default_rng(emax).standard_normal(o.slab)
    ref = o.white_vjp(H, 1, Eb)
    dH, dEb, dHb = eng.new_op(1, H), eng.new_op(-1, Eb), eng.new_op(1)
    eng.white_vjp(dH, dEb, dHb)
    assert rel_err(dHb.download(), ref) < TOL
    assert abs(eng.dot(dH, dEb) - H @ Eb) <= 1e-12 * np.abs(H).sum() * np.abs(Eb).max()


def _flow(eng, backend, steps, K=3):
    from imsrg_gb300.adjoint import MagnusFlowAdjoint, channel_perturbations
    H0 = eng.synthetic_hamiltonian(seed=3)
    V = channel_perturbations(eng, K, sigma=0.1, seed=4)
    return MagnusFlowAdjoint(backend, H0, V, ds=0.5, steps=steps)


def test_flow_gradient_device(oracles, engines):
    from imsrg_gb300.adjoint import EngineBackend
    eng = engines(4)
    fl = _flow(eng, EngineBackend(eng), steps=3)
    theta = np.zeros(3)
    plan = fl.plan(theta)
    e0 = fl.forward(theta, plan)
    g = fl.gradient()
    h = 1e-4
    fd = np.zeros(3)
    for k in range(3):
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd[k] = (fl.forward(tp, plan) - fl.forward(tm, plan)) / (2 * h)
    assert rel_err(g, fd) < 1e-7, (g, fd)
    # the same adjoint over the oracle
    flo = _flow(eng, OracleBackend(oracles(4)), steps=3)
    assert abs(flo.forward(theta, plan) - e0) <= 1e-10 * abs(e0)
    assert rel_err(flo.gradient(), g) < 1e-9


def test_flow_energy_autograd(engines):
    torch = pytest.importorskip("torch")
    from imsrg_gb300.adjoint import EngineBackend, flow_energy
    eng = engines(2)
    fl = _flow(eng, EngineBackend(eng), steps=4, K=2)
    theta = torch.zeros(2, dtype=torch.float64, requires_grad=True)
    E = flow_energy(theta, fl)
    E.backward()
    assert theta.grad is not None
    assert rel_err(theta.grad.numpy(), fl.gradient()) < 1e-12
    assert abs(E.item() - fl.forward(np.zeros(2))) <= 1e-12 * abs(E.item())
