"""Mixed-precision (split operands on tcgen05, FP32 gathers) against the FP64 oracle.

The mixed path is held to FP32-level agreement.  The tolerances (largest error per array
group relative to that group's largest element) are about ten times the errors observed on
GB300 at each eMax: 3-slice BF16 (6 products) and TF32-compensated (3 products) carry ~24 and
~22 operand bits and end up at the FP32 level of the gathers; 2-slice BF16 (3 products)
carries ~16 bits in the ladder products.
"""
import numpy as np
import pytest

from helpers import rel_err, sections

pytestmark = pytest.mark.gpu
TOL = {("bf16x6", 2): 6e-6, ("bf16x6", 4): 5e-6, ("bf16x6", 6): 2e-5,
       ("bf16x3", 2): 9e-5, ("bf16x3", 4): 6e-5, ("bf16x3", 6): 5e-5,
       ("tf32x3", 2): 6e-6, ("tf32x3", 4): 5e-6, ("tf32x3", 6): 2e-5}
MODES = ["bf16x6", "bf16x3", "tf32x3"]


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


@pytest.mark.parametrize("mode", MODES)
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
    print(f"eMax={emax} {mode} pphh: w1 {rel_err(dw1.download(), w1):.2e} w2 {rel_err(dw2.download(), w2):.2e} "
          f"RES {rel_err(dRES.download(), ref):.2e}")
    assert rel_err(dw1.download(), w1) <= TOL[mode, emax]
    assert rel_err(dw2.download(), w2) <= TOL[mode, emax]
    assert rel_err(dRES.download(), ref) <= TOL[mode, emax]


@pytest.mark.parametrize("mode", MODES)
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
    print(f"eMax={emax} {mode} mixed [L,R]: E0 {abs(e0 - r0) / max(1.0, abs(r0)):.2e} 1b {rel_err(ob, rob):.2e} "
          f"2b {rel_err(tb, rtb):.2e}")
    assert abs(e0 - r0) <= TOL[mode, emax] * max(1.0, abs(r0))
    assert rel_err(ob, rob) <= TOL[mode, emax]
    assert rel_err(tb, rtb) <= TOL[mode, emax]
