"""The atan, atanxx and w2 generators on the device (build_gs_atan / build_gs_atanxx /
build_gs_w2, src/generators.f90:109-374) against the oracle, FP64, 1e-10 relative; and an
eager Magnus flow driven by w2, the reference driver's default generator."""
import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.mark.parametrize("emax", [2, 4])
def test_generators_match_oracle(oracles, engines, emax):
    o, eng = oracles(emax), engines(emax)
    assert eng.precision == "fp64"
    H = o.random(61, 1)
    H2 = o.random(62, 1)
    dH, dH2, dE = eng.new_op(1, H), eng.new_op(1, H2), eng.new_op(-1)
    eng.build_gs_atan(dH, dE)
    assert rel_err(dE.download(), o.atan(H, 1)) < TOL
    eng.build_gs_atanxx(dH, dH2, dE)
    assert rel_err(dE.download(), o.atanxx(H, H2, 1)) < TOL
    eng.build_gs_w2(dH, dE)
    assert rel_err(dE.download(), o.w2(H, 1)) < TOL
    assert dE.herm == -1


def test_w2_flow_matches_oracle(oracles, engines):
    from imsrg_gb300.flow import magnus_decouple
    o, eng = oracles(4), engines(4)
    H = eng.synthetic_hamiltonian(seed=12)
    ops = {}
    res = magnus_decouple(eng, H, max_steps=3, bch_conv=1e-6, generator="w2", ops=ops)
    G = o.new()
    DG = o.w2(H, 1)
    for _ in range(3):
        o.magnus_expand(DG, G)
        G += 0.5 * DG
        HS, _ = o.bch_expand(G, H, 40, 1e-6)
        DG = o.w2(HS, 1)
    assert abs(res.E0 - HS[0]) <= TOL * abs(HS[0])
    assert rel_err(ops["HS"].download(), HS) < TOL
    assert rel_err(ops["G"].download(), G) < TOL
    with pytest.raises(ValueError):
        magnus_decouple(eng, H, max_steps=1, generator="w2", graph=True)
