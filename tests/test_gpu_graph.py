"""The Magnus step replayed from a CUDA graph (imsrg_magnus_step).

A step is the loop body of magnus_decouple (src/IMSRG_MAGNUS.f90:47-110).  The graph
replay must give the eager step's operators bit for bit (same kernels, same order, early
exits of MAGNUS_EXPAND / BCH_EXPAND decided on the device with the reference's tests), and
the FP64 step must follow the oracle's restatement of the same loop to 1e-10.
"""
import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu

DS = 0.5


def _state(eng, H):
    dH = eng.new_op(1, H)
    HS = eng.new_op(1, H)
    G = eng.new_op(-1)
    DG = eng.new_op(-1)
    eng.build_gs_white(HS, DG)
    return HS, G, DG, dH


@pytest.mark.parametrize("precision", ["fp64", "bf16x6"])
def test_graph_step_equals_eager(built_lib, precision):
    from imsrg_gb300 import Engine, make_basis
    eng = Engine(make_basis(4), device=0, precision=precision)
    H = eng.synthetic_hamiltonian(seed=3)
    eager, graph = _state(eng, H), _state(eng, H)
    c0 = eng.magnus_step_counters()
    ie, ig = [], []
    for _ in range(4):
        ie.append(eng.magnus_step(*eager, DS, 11, 1e-8, graph=False, allow_unconverged=True))
        ig.append(eng.magnus_step(*graph, DS, 11, 1e-8, graph=True, allow_unconverged=True))
    for a, b in zip(ie, ig):
        for k in ("E0", "mbpt2", "magnus_terms", "bch_terms", "bch_converged"):
            assert a[k] == b[k], (k, a, b)
    assert ig[0]["graph_rebuilt"] and not any(i["graph_rebuilt"] for i in ig[1:])
    assert ig[-1]["magnus_terms"] > 0 and ig[-1]["bch_terms"] > 1
    for x, y in zip(eager, graph):
        assert np.array_equal(x.download(), y.download())
    c1 = eng.magnus_step_counters()
    assert c1["steps"] - c0["steps"] == 4
    assert c1["commutators"] - c0["commutators"] == sum(i["magnus_terms"] + i["bch_terms"] for i in ig)
    assert c1["kernels"] > c0["kernels"]


@pytest.mark.parametrize("reference", ["ho", "hf"])
def test_graph_flow_matches_oracle(built_lib, oracles, reference):
    from imsrg_gb300 import Engine, make_basis
    o = oracles(4)
    eng = Engine(make_basis(4), device=0, precision="fp64")
    if reference == "hf":  # calc_HF first, as the reference's driver does with hartree_fock set
        bare = eng.synthetic_bare_hamiltonian(seed=4)
        Hop = eng.new_op(1, bare)
        eng.calc_hf(Hop)
        H = Hop.download()
        assert rel_err(H, o.calc_hf(bare)[0]) < 1e-10
    else:
        H = eng.synthetic_hamiltonian(seed=4)
    HS, G, DG, dH = _state(eng, H)
    oG = o.new()
    oDG = o.white(H, 1)
    for step in range(3):
        info = eng.magnus_step(HS, G, DG, dH, DS, 40, 1e-6, graph=True)
        used = o.magnus_expand(oDG, oG)
        oG += DS * oDG
        oHS, n = o.bch_expand(oG, H, 40, 1e-6)
        oDG = o.white(oHS, 1)
        assert info["magnus_terms"] == used and info["bch_terms"] == n
        assert abs(info["E0"] - oHS[0]) <= 1e-10 * abs(oHS[0])
        assert abs(info["mbpt2"] - o.mbpt2(oHS, 1)) <= 1e-10 * abs(o.mbpt2(oHS, 1))
        assert rel_err(HS.download(), oHS) < 1e-10
        assert rel_err(G.download(), oG) < 1e-10
        assert rel_err(DG.download(), oDG) < 1e-10


def test_graph_unconverged_and_async(built_lib):
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300._lib import ImsrgError
    eng = Engine(make_basis(2), device=0, precision="fp64")
    H = eng.synthetic_hamiltonian(seed=6)
    eager, graph = _state(eng, H), _state(eng, H)
    # two BCH terms cannot reach 1e-30: both paths finish the step and report it
    a = eng.magnus_step(*eager, DS, 3, 1e-30, graph=False, allow_unconverged=True)
    b = eng.magnus_step(*graph, DS, 3, 1e-30, graph=True, allow_unconverged=True)
    assert not a["bch_converged"] and not b["bch_converged"] and a["bch_terms"] == b["bch_terms"] == 2
    for x, y in zip(eager, graph):
        assert np.array_equal(x.download(), y.download())
    with pytest.raises(ImsrgError):
        eng.magnus_step(*graph, DS, 3, 1e-30, graph=True)
    # enqueue-only replays, then the device counters
    c0 = eng.magnus_step_counters()
    e2, g2 = _state(eng, H), _state(eng, H)
    for _ in range(3):
        eng.magnus_step(*e2, DS, 40, 1e-6, graph=False)
        eng.magnus_step(*g2, DS, 40, 1e-6, graph=True, wait=False)
    eng.synchronize()
    for x, y in zip(e2, g2):
        assert np.array_equal(x.download(), y.download())
    c1 = eng.magnus_step_counters()
    assert c1["steps"] - c0["steps"] == 3 and c1["unconverged"] == c0["unconverged"]
    with pytest.raises(ValueError):
        eng.magnus_step(*e2, DS, 40, 1e-6, graph=False, wait=False)
    with pytest.raises(ImsrgError):
        eng.magnus_step(e2[0], e2[0], e2[2], e2[3], DS, 40, 1e-6)
