"""The traditional flow (decouple_hamiltonian, src/IMSRG_ODE.f90:9-178) with the device derivative
against the same Adams integrator driven by the oracle's derivative: same intervals, same
number of derivative evaluations, H(s) to 1e-9."""
import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("emax", [2, 4])
def test_ode_flow_matches_oracle_derivative(oracles, engines, emax, tmp_path):
    from imsrg_gb300.ode import decouple_hamiltonian
    o, eng = oracles(emax), engines(emax)
    H0 = eng.synthetic_hamiltonian(seed=5)
    ops = {}
    res = decouple_hamiltonian(eng, H0, max_steps=30, ops=ops, prefix="t", output_dir=str(tmp_path))

    def oracle_derivative(s, y):
        H = eng.repackage(y, 1)
        return eng.vectorize(o.commutator(o.white(H, 1), -1, H, 1))

    ref = decouple_hamiltonian(eng, H0, max_steps=30, derivative=oracle_derivative)
    assert len(res.steps) == len(ref.steps) and res.evaluations == ref.evaluations
    for a, b in zip(res.steps, ref.steps):
        assert a[0] == b[0] and abs(a[1] - b[1]) < 1e-12
        assert abs(a[2] - b[2]) <= 1e-9 * abs(b[2])
    lines = (tmp_path / "t_0bflow.dat").read_text().splitlines()
    assert len(lines) == len(res.steps) and len(lines[0]) == 6 + 4 * 17 and len(lines[1]) == 6 + 4 * 15
    assert res.steps[-1][2] < res.steps[0][2]
