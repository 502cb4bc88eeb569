"""Flat operator vectors (vectorize / repackage, src/basic_IMSRG.f90:3929-4053) and the
Omega checkpoint file layout (src/basic_IMSRG.f90:3215-3407), on the CPU."""
import numpy as np
import pytest


@pytest.mark.parametrize("emax", [2, 4])
def test_vectorize_matches_oracle_and_round_trips(built_lib, oracles, emax):
    from imsrg_gb300 import Engine, make_basis
    o = oracles(emax)
    eng = Engine(make_basis(emax), device=-1)
    info = eng.block_info()
    b = eng.basis
    A, P = b.nholes, b.norbits - b.nholes
    neq = 1 + A * A + A * P + P * P
    for q in range(eng.nblocks):
        nh, np_, nb = int(info["nhh"][q]), int(info["npp"][q]), int(info["nph"][q])
        neq += (nh * nh + nh + nb * nb + nb + np_ * np_ + np_) // 2 + nb * np_ + nh * np_ + nh * nb
    assert eng.neq == neq
    for herm in (1, -1):
        X = o.random(30 + herm, herm)
        v = eng.vectorize(X)
        assert v.size == neq and np.array_equal(v, o.vectorize(X))
        assert np.array_equal(eng.repackage(v, herm), X)
    with pytest.raises(ValueError):
        eng.repackage(np.zeros(neq + 1))


def test_checkpoint_names_follow_the_reference():
    from imsrg_gb300.flow import omega_checkpoint_name
    p = "chi2b_srg0625_eMax08_hwHO020"
    assert omega_checkpoint_name(p, 12.5) == "chi2b_srg0625_eMax08_hwHO020_s12.500.bin"
    assert omega_checkpoint_name(p, 2.5) == "chi2b_srg0625_eMax08_hwHO020_s2.5000.bin"
    assert omega_checkpoint_name("synth_eMax10_hw20_x", 24.0) == "synth_eMax10_hw20_s24.000.bin"


def test_fortran_e15_7_format():
    from imsrg_gb300.flow import _e15_7
    assert _e15_7(-12.3456789) == " -0.1234568E+02"
    assert _e15_7(123.45678949) == "  0.1234568E+03"
    assert _e15_7(9.99999999) == "  0.1000000E+02"
    assert _e15_7(-0.000123456789) == " -0.1234568E-03"
    assert _e15_7(0.0) == "  0.0000000E+00"


def test_fortran_e_formats():
    from imsrg_gb300.ode import _e_fmt
    assert _e_fmt(114.357603550025, 17, 9) == "  0.114357604E+03"
    assert _e_fmt(-0.0001234, 15, 7) == " -0.1234000E-03"
