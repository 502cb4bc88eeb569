"""The launch-configuration autotuner of the mixed commutator (imsrg_autotune).

Every candidate configuration computes the same commutator: the 122 sub-block partition
and the GEMM tile shape and order change how work is spread over the GPU, not what any
output element sums (each output tile accumulates its K blocks in the same order).  So the result after tuning is bit-identical to the one
before, and a Magnus step replayed from the re-captured graph still equals the eager step.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["bf16x6", "bf16x3"])
def test_autotune_keeps_results_and_reports_choice(built_lib, oracles, mode):
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300._lib import ImsrgError
    o = oracles(4)
    eng = Engine(make_basis(4), device=0, precision=mode)
    A, B = o.random(21, -1), o.random(22, 1)
    dA, dB, dR = eng.new_op(-1, A), eng.new_op(1, B), eng.new_op(1)
    eng.commutator(dA, dB, dR)
    before = dR.download()
    info = eng.autotune(dA, dB, dR)
    assert (info["tiny_cap"], info["small_cap"]) in {(32, 256), (64, 256), (32, 512), (64, 512), (64, 1024)}
    assert info["gemm_order"] in (0, 1) and info["recouple_ctas"] > 0
    assert info["gemm_wmax"] in (128, 256) and info["gemm_narrow"] in (0, 1)
    assert info["recouple_kind"] == 1 and info["recouple_min_blocks"] in (4, 6, 8)
    assert info["gemm_merged"] in (0, 1)
    assert info["ms_before"] > 0 and info["ms_after"] > 0
    eng.commutator(dA, dB, dR)
    assert np.array_equal(dR.download(), before)
    # every other choice of each knob, applied with imsrg_set_tuning, still gives the same bits
    for change in ({"recouple_min_blocks": 4 if info["recouple_min_blocks"] != 4 else 8, "recouple_ctas": 152 * 8},
                   {"gemm_merged": 1 - info["gemm_merged"]}, {"gemm_narrow": 1 - info["gemm_narrow"]},
                   {"gemm_order": 1 - info["gemm_order"]},
                   {"gemm_wmax": 384 - info["gemm_wmax"]} if mode == "bf16x3" else {},
                   {"gemm_merged": 0, "gemm_wmax_x": 384 - max(info["gemm_wmax_x"], 128),
                    "gemm_narrow_x": 1 - info["gemm_narrow_x"]} if mode == "bf16x3" else {},
                   {"tiny_cap": 16, "small_cap": 128}):
        cfg = dict(info)
        cfg.update(change)
        eng.set_tuning(cfg)
        eng.commutator(dA, dB, dR)
        assert np.array_equal(dR.download(), before), change
    eng.set_tuning(info)
    # graph replay after tuning equals the eager step
    H = eng.synthetic_hamiltonian(seed=3)
    states = []
    for _ in range(2):
        st = (eng.new_op(1, H), eng.new_op(-1), eng.new_op(-1), eng.new_op(1, H))
        eng.build_gs_white(st[0], st[2])
        states.append(st)
    for _ in range(2):
        eng.magnus_step(*states[0], 0.5, 11, 1e-8, graph=False, allow_unconverged=True)
        eng.magnus_step(*states[1], 0.5, 11, 1e-8, graph=True, allow_unconverged=True)
    for x, y in zip(states[0], states[1]):
        assert np.array_equal(x.download(), y.download())
    e64 = Engine(make_basis(2), device=0)
    a = e64.new_op(-1)
    with pytest.raises(ImsrgError) as e:
        e64.autotune(a, e64.new_op(1), e64.new_op(1))
    assert e.value.code == 6
