"""The oracle's own restatement of the synthetic input against the library's generator.

The CPU legs of the benchmark build their Hamiltonian with the oracle alone (no product
library loaded), so the two generators must agree bit for bit: the me2j record loop and
proton-neutron conversion (src/interaction_IO.f90:320-555) and the HO kinetic energy with its
FP32 intermediates (src/basic_IMSRG.f90:2093-2191), from the same seeded stream.  The library
side runs in a host-only context (no GPU).
"""
import numpy as np
import pytest


@pytest.mark.parametrize("emax", [2, 4, 6])
@pytest.mark.parametrize("seed,v_scale", [(1, 1.0), (7, 0.3)])
def test_oracle_synthetic_equals_library(built_lib, oracles, emax, seed, v_scale):
    from imsrg_gb300 import Engine, make_basis
    host = Engine(make_basis(emax), device=-1)
    ref = host.synthetic_bare_hamiltonian(seed=seed, v_scale=v_scale)
    got = oracles(emax).synthetic_bare_hamiltonian(seed=seed, v_scale=v_scale)
    assert got.shape == ref.shape
    assert np.array_equal(got, ref)
    assert np.count_nonzero(got) > 0.05 * got.size


def test_oracle_hf_of_own_input_is_stable(oracles):
    """calc_HF of the oracle's own input: converged, E_HF finite, and H in the HF basis is
    Hermitian in its one-body part (the CPU baseline's starting state)."""
    o = oracles(4)
    H, D, e_hf, iters = o.calc_hf(o.synthetic_bare_hamiltonian(seed=1))
    assert np.isfinite(e_hf) and 0 < iters < 1000
    assert np.allclose(D.T @ D, np.eye(D.shape[0]), atol=1e-10)
    assert np.isfinite(H).all()
