"""me2j interaction records: the format and read_me2j_interaction's conversion
(src/interaction_IO.f90:282-557) on the CPU.

The synthetic Hamiltonian is built from seeded me2j record values through the same
conversion, so converting those values reproduces its two-body part exactly; a file written
in the me2j layout reads back to the values rounded to the format's 7 decimals; the records of
a larger file that fall outside the basis are skipped."""
import numpy as np
import pytest

from helpers import rel_err


def _two_body(eng, slab):
    b = eng.basis
    A, P = b.nholes, b.norbits - b.nholes
    return slab[1 + A * A + P * P + P * A:]


@pytest.mark.parametrize("emax", [2, 4])
def test_synthetic_values_reproduce_the_hamiltonian(built_lib, emax):
    from imsrg_gb300 import Engine, make_basis
    eng = Engine(make_basis(emax), device=-1)
    vals = eng.synthetic_me2j_values(seed=5)
    assert vals.size % 4 == 0 and np.count_nonzero(vals) > vals.size // 2
    slab = eng.me2j_to_slab(vals, emax, htype=0)  # the synthetic H has no c.m. term
    assert np.array_equal(_two_body(eng, slab), _two_body(eng, eng.synthetic_bare_hamiltonian(seed=5)))


def test_file_round_trip(built_lib, tmp_path):
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300.me2j import read_me2j, write_me2j
    eng = Engine(make_basis(4), device=-1)
    vals = eng.synthetic_me2j_values(seed=6)
    path = str(tmp_path / "synthetic_eMax04_hwHO020.me2j.gz")
    write_me2j(path, vals)
    back = read_me2j(path)
    assert back.size == vals.size and np.abs(back - np.round(vals, 7)).max() < 1e-12
    slab = eng.me2j_to_slab(back, 4, htype=0)
    ref = eng.synthetic_bare_hamiltonian(seed=6)
    assert rel_err(_two_body(eng, slab), _two_body(eng, ref)) < 1e-6


def test_larger_file_restricted_to_the_basis(built_lib, oracles):
    """Records of an eMax=4 file read into the eMax=2 basis give the same elements as in the
    eMax=4 basis"""
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300._lib import ImsrgError
    big, small = Engine(make_basis(4), device=-1), Engine(make_basis(2), device=-1)
    vals = big.synthetic_me2j_values(seed=7)
    V4, V2 = big.me2j_to_slab(vals, 4), small.me2j_to_slab(vals, 4)
    o4, o2 = oracles(4), oracles(2)
    b2 = small.basis
    # hk order: the eMax=2 orbits are the first ones of the eMax=4 basis
    n = b2.norbits
    checked = 0
    for a in range(n):
        for b in range(n):
            for c in range(n):
                for d in range(n):
                    for J in range(0, 2 * int(b2.jj.max()) + 1, 2):
                        v2 = o2.v_elem(V2, 1, a, b, c, d, J)
                        assert abs(v2 - o4.v_elem(V4, 1, a, b, c, d, J)) < 1e-13
                        checked += v2 != 0.0
    assert checked > 100
    with pytest.raises(ImsrgError) as e:
        small.me2j_to_slab(vals[:-4], 4)
    assert e.value.code == 5


def test_centre_of_mass_term_matches_oracle(built_lib, oracles):
    """htype 1 adds -p1.p2 hw/A to every element (p1_p2, src/basic_IMSRG.f90:4445-4504)"""
    from imsrg_gb300 import Engine, make_basis
    emax = 2
    o, eng = oracles(emax), Engine(make_basis(emax), device=-1)
    b = eng.basis
    zero = np.zeros(eng.synthetic_me2j_values(seed=1).size)
    com = eng.me2j_to_slab(zero, emax, htype=1)
    assert not np.any(_two_body(eng, eng.me2j_to_slab(zero, emax, htype=0)))
    f = -b.hw / (b.Aprot + b.Aneut)
    n, checked = b.norbits, 0
    for a in range(n):
        for bb in range(n):
            for c in range(n):
                for d in range(n):
                    if (b.ll[a] + b.ll[bb]) % 2 != (b.ll[c] + b.ll[d]) % 2 or b.itzp[a] + b.itzp[bb] != b.itzp[c] + b.itzp[d]:
                        continue
                    for J in range(abs(b.jj[a] - b.jj[bb]), b.jj[a] + b.jj[bb] + 1, 2):
                        if not abs(b.jj[c] - b.jj[d]) <= J <= b.jj[c] + b.jj[d]:
                            continue
                        ref = f * o.p1_p2(a, bb, c, d, J)
                        # v_elem adds sqrt(2) for identical orbits; p1_p2 is normalised
                        norm = np.sqrt((1.0 + (a == bb)) * (1.0 + (c == d)))
                        assert abs(o.v_elem(com, 1, a, bb, c, d, J) - ref * norm) < 1e-13, (a, bb, c, d, J)
                        checked += ref != 0.0
    assert checked > 50
    # p.p and r.r share their angular structure: their elements are never both zero by symmetry alone
    assert any(o.r1_r2(0, 2, 0, 2, J) != 0.0 for J in (0, 2, 4))
