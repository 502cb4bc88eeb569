"""The perturbative triples correction on the device (restore_triples,
src/IMSRG_MAGNUS.f90:767-902) against the oracle's restatement, FP64, 1e-10 relative: for a
random Omega at eMax 2, 4 and 6, and for the Omega and H(s) of a Magnus flow (the reference's
'trips' option), with H(s) from BCH_EXPAND and from CR_EXPAND (src/main_IMSRG.f90:296-315)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("emax", [2, 4, 6])
def test_triples_match_oracle(oracles, engines, emax):
    o, eng = oracles(emax), engines(emax)
    H = eng.synthetic_hamiltonian(seed=1)
    OM = o.random(5, -1) * 0.05
    ref = o.restore_triples(H, OM)
    e3, items = eng.restore_triples(eng.new_op(1, H), eng.new_op(-1, OM))
    ch = o.three_channels()
    assert items == int((ch["nppp"].astype(np.int64) * ch["nhhh"]).sum())
    assert abs(e3 - ref) <= 1e-10 * abs(ref)


def test_triples_after_flow(oracles, engines):
    from imsrg_gb300.flow import magnus_decouple
    o, eng = oracles(4), engines(4)
    bare = eng.synthetic_bare_hamiltonian(seed=3)
    Hop = eng.new_op(1, bare)
    eng.calc_hf(Hop)
    H0 = Hop.download()
    ops = {}
    magnus_decouple(eng, H0, max_steps=40, ops=ops)
    G = ops["G"]
    OM = G.download()
    e3, _ = eng.restore_triples(eng.new_op(1, H0), G)
    ref = o.restore_triples(H0, OM)
    assert e3 < 0.0 and abs(e3 - ref) <= 1e-10 * abs(ref)
    # the completely renormalised form: H replaced by CR_EXPAND(Omega, H0)
    CR = eng.new_op(1)
    eng.cr_expand(CR, G, eng.new_op(1, H0), 14)
    cr_ref, _ = o.cr_expand(OM, H0, 14)
    e3cr, _ = eng.restore_triples(CR, G)
    assert abs(e3cr - o.restore_triples(cr_ref, OM)) <= 1e-10 * abs(e3cr)


def test_magnus_triples_files(engines, tmp_path):
    """The driver's output files: E0 and E0 + correction in e15.7."""
    from imsrg_gb300.flow import magnus_decouple, magnus_triples
    eng = engines(2)
    H0 = eng.synthetic_hamiltonian(seed=2)
    ops = {}
    res = magnus_decouple(eng, H0, max_steps=10, ops=ops)
    E0, Et = magnus_triples(eng, H0, ops["G"], res.E0, "y", prefix="t", output_dir=str(tmp_path))
    E0c, Ec = magnus_triples(eng, H0, ops["G"], res.E0, "C", prefix="t", output_dir=str(tmp_path))
    assert E0 == E0c == res.E0 and Et < E0 and Ec < E0
    for name, v in (("t_magnus_triples.dat", Et), ("t_magnus_cr_triples.dat", Ec)):
        line = (tmp_path / name).read_text().rstrip("\n")
        assert len(line) == 30
        assert abs(float(line[15:]) - v) <= 1e-6 * abs(v)
