"""The Adams integrator of the traditional flow (the Shampine-Gordon code of src/adams_ode.f90)
on problems with known solutions, and the ODE flow driven by the oracle's derivative.

The reference's code is a restatement of a published algorithm (Shampine and Gordon 1975); its
behaviour is pinned here by what the algorithm guarantees: the local error control at
relerr = abserr = 1e-6 reproduces exp(-t), a harmonic oscillator and a stiff-free linear system
to that tolerance, raises order and step on smooth problems, and continues across successive
output points (iflag = 2) without restarting."""
import numpy as np
import pytest


def test_exponential_decay_and_continuation():
    from imsrg_gb300.ode import AdamsIntegrator
    integ = AdamsIntegrator(lambda t, y: -y, 1, 1e-6, 1e-6)
    y, t = np.array([1.0]), 0.0
    for k in range(1, 21):
        y, t, iflag = integ.integrate(t, 0.1 * k, y)
        assert iflag == 2 and abs(t - 0.1 * k) < 1e-15
        assert abs(y[0] - np.exp(-t)) < 2e-5
    # continuation: far fewer evaluations than 20 fresh starts, orders above 1 reached
    assert integ.evaluations < 150 and integ.kold > 2


def test_oscillator_and_linear_system():
    from imsrg_gb300.ode import AdamsIntegrator
    A = np.array([[0.0, 1.0, 0.0], [-4.0, 0.0, 0.5], [0.0, -0.5, -0.1]])
    w, V = np.linalg.eig(A)
    y0 = np.array([1.0, 0.0, 0.3])
    integ = AdamsIntegrator(lambda t, y: A @ y, 3, 1e-6, 1e-6)
    y, t = y0.copy(), 0.0
    for k in range(1, 31):
        y, t, _ = integ.integrate(t, 0.2 * k, y)
    exact = (V @ np.diag(np.exp(w * t)) @ np.linalg.solve(V, y0)).real
    assert np.abs(y - exact).max() < 1e-4


def test_ode_flow_oracle_derivative_matches_magnus_endpoint(oracles, built_lib):
    """The ODE flow with the oracle's derivative (white generator, full commutator) and the
    Magnus flow decouple the same Hamiltonian to the same E0 (to the integrator's tolerance)."""
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300.ode import AdamsIntegrator
    o = oracles(2)
    eng = Engine(make_basis(2), device=-1)
    H0 = eng.synthetic_hamiltonian(seed=4)

    def deriv(s, y):
        H = eng.repackage(y, 1)
        return eng.vectorize(o.commutator(o.white(H, 1), -1, H, 1))

    integ = AdamsIntegrator(deriv, eng.neq, 1e-6, 1e-6)
    y, s = eng.vectorize(H0), 0.0
    for k in range(1, 101):
        y, s, iflag = integ.integrate(s, 0.1 * k, y)
        assert iflag == 2
    H = eng.repackage(y, 1)
    # the Magnus flow (oracle) to the same s
    G, DG = o.new(), o.white(H0, 1)
    for _ in range(20):
        o.magnus_expand(DG, G)
        G += 0.5 * DG
        HS, _ = o.bch_expand(G, H0, 40, 1e-10)
        DG = o.white(HS, 1)
    assert abs(H[0] - HS[0]) < 1e-3 * abs(H0[0] - HS[0]) + 1e-4
