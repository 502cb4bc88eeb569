"""Hartree-Fock and normal ordering on the device against the oracle's restatement.

imsrg_calc_hf / imsrg_calc_ho / imsrg_sqop_to_hf / imsrg_transform_2b_to_hf /
imsrg_normal_order follow calc_HF, calc_HO, sqop_to_HF, transform_2b_to_HF
(src/HF_mod.f90:14-209, 567-692) and normal_order (src/basic_IMSRG.f90:2419-2550).  The
device builds the mean-field tensor and changes the two-body basis; the self-consistency loop
runs on the host.  Same iteration count, coefficients and operators as the oracle to 1e-10;
at eMax=10 the size-independent properties (f_ph = 0, orthogonality, round trip).
"""
import numpy as np
import pytest

from helpers import rel_err
from test_hf_oracle import _channel_norms, _particle_rotation

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("emax", [2, 4])
def test_calc_hf_matches_oracle(oracles, engines, emax):
    o, eng = oracles(emax), engines(emax)
    bare = eng.synthetic_bare_hamiltonian(seed=5)
    ref, Dref, E, it = o.calc_hf(bare)
    H = eng.new_op(1, bare)
    D, info = eng.calc_hf(H)
    assert info["iterations"] == it and info["crit"] <= 1e-6
    assert abs(info["e_hf"] - E) <= 1e-10 * abs(E)
    assert np.abs(D - Dref).max() < 1e-10
    assert rel_err(H.download(), ref) < 1e-10


@pytest.mark.parametrize("emax", [2, 4])
def test_calc_ho_and_normal_order_match_oracle(oracles, engines, emax):
    o, eng = oracles(emax), engines(emax)
    bare = eng.synthetic_bare_hamiltonian(seed=6)
    H = eng.new_op(1, bare)
    D, info = eng.calc_ho(H)
    assert info["iterations"] == 0 and np.array_equal(D, np.eye(o.basis.norbits))
    ho = eng.synthetic_hamiltonian(seed=6)
    assert abs(info["e_hf"] - ho[0]) <= 1e-12 * abs(ho[0])
    assert rel_err(H.download(), ho) < 1e-12
    # a random hermitian operator
    R = o.random(17, 1)
    op = eng.new_op(1, R)
    eng.normal_order(op)
    assert rel_err(op.download(), o.normal_order(R, 1)) < 1e-12


@pytest.mark.parametrize("emax", [2, 4])
def test_transform_and_sqop_to_hf_match_oracle(oracles, engines, emax):
    o, eng = oracles(emax), engines(emax)
    bare = eng.synthetic_bare_hamiltonian(seed=7)
    _, D, _, _ = o.calc_hf(bare)
    if emax > 2:
        D = D @ _particle_rotation(o, 3)  # any block-diagonal orthogonal matrix will do
    R = o.random(19, 1)
    op = eng.new_op(1, R)
    eng.transform_2b_to_hf(op, D)
    assert rel_err(op.download(), o.transform_2b_to_hf(R, D)) < 1e-12
    op = eng.new_op(1, R)
    eng.sqop_to_hf(op, D)
    assert rel_err(op.download(), o.sqop_to_hf(R, D)) < 1e-12


def test_calc_hf_iteration_limit(engines):
    from imsrg_gb300._lib import ImsrgError
    eng = engines(2)
    bare = eng.synthetic_bare_hamiltonian(seed=5)
    H = eng.new_op(1, bare)
    with pytest.raises(ImsrgError) as e:
        eng.calc_hf(H, max_iter=1)
    assert e.value.code == 4
    assert np.array_equal(H.download(), bare)


def test_calc_hf_emax10_properties(built_lib):
    from imsrg_gb300 import Engine, make_basis
    basis = make_basis(10)
    eng = Engine(basis, device=0)
    bare = eng.synthetic_bare_hamiltonian(seed=1)
    ho = eng.synthetic_hamiltonian(seed=1)
    H = eng.new_op(1, bare)
    D, info = eng.calc_hf(H)
    hf = H.download()
    b = basis
    A, P = b.nholes, b.norbits - b.nholes
    assert info["iterations"] > 2 and info["e_hf"] == hf[0] and hf[0] < ho[0]
    assert np.allclose(D.T @ D, np.eye(b.norbits), atol=1e-13)
    fpp = hf[1 + A * A:1 + A * A + P * P]
    fph = hf[1 + A * A + P * P:1 + A * A + P * P + P * A]
    assert np.abs(fph).max() < 1e-12 * np.abs(fpp).max()
    n0, n1 = _channel_norms(eng, bare), _channel_norms(eng, hf)
    assert np.allclose(n0, n1, rtol=1e-11, atol=1e-12 * n0.max())
    eng.transform_2b_to_hf(H, D.T)
    off = 1 + A * A + P * P + P * A
    assert rel_err(H.download()[off:], bare[off:]) < 1e-12
