"""Mixed-precision (split-BF16 on tcgen05, FP32 gathers) against the FP64 oracle.

The mixed path is held to FP32-level agreement: 3-slice BF16 (6 products) to 2e-5
relative per array group, 2-slice (3 products) to 2e-3.
"""
import numpy as np
import pytest

from helpers import rel_err, sections

pytestmark = pytest.mark.gpu
TOL = {"bf16x6": 2e-5, "bf16x3": 2e-3}


@pytest.fixture(scope="module")
def mixed_engines(built_lib):
    from imsrg_gb300 import Engine, make_basis
    cache = {}

    def get(emax, mode):
        key = (emax, mode)
        if key not in cache:
            cache[key] = Engine(make_basis(emax), device=0, precision=mode)
        return cache[key]
    return get


@pytest.mark.parametrize("mode", ["bf16x6", "bf16x3"])
@pytest.mark.parametrize("emax", [2, 4])
def test_tc_pphh_intermediates(oracles, mixed_engines, emax, mode):
    o, eng = oracles(emax), mixed_engines(emax, mode)
    L, R = o.random(501, -1), o.random(502, 1)
    dL, dR = eng.new_op(-1, L), eng.new_op(1, R)
    w1, w2, ref = o.new(), o.new(), o.new()
    o.commutator_222_pp_hh(L, -1, R, 1, ref, 1, w1, w2)
    dw1, dw2, dRES = eng.new_op(1), eng.new_op(1), eng.new_op(1)
    eng.commutator_222_pp_hh(dL, dR, dRES, dw1, dw2)
    eng.synchronize()
    assert rel_err(dw1.download(), w1) <= TOL[mode]
    assert rel_err(dw2.download(), w2) <= TOL[mode]
    assert rel_err(dRES.download(), ref) <= TOL[mode]


@pytest.mark.parametrize("mode", ["bf16x6", "bf16x3"])
@pytest.mark.parametrize("emax", [2, 4, 6])
def test_mixed_full_commutator(oracles, mixed_engines, emax, mode):
    o, eng = oracles(emax), mixed_engines(emax, mode)
    L, R = o.random(601 + emax, -1), o.random(602 + emax, 1)
    ref = o.commutator(L, -1, R, 1, 1)
    dL, dR, dRES = eng.new_op(-1, L), eng.new_op(1, R), eng.new_op(1)
    eng.commutator(dL, dR, dRES)
    eng.synchronize()
    got = dRES.download()
    e0, ob, tb = sections(o, got)
    r0, rob, rtb = sections(o, ref)
    assert abs(e0 - r0) <= TOL[mode] * max(1.0, abs(r0))
    assert rel_err(ob, rob) <= TOL[mode]
    assert rel_err(tb, rtb) <= TOL[mode]
