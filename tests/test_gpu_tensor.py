"""Device scalar-tensor commutator and BCH_TENSOR against the oracle (FP64, 1e-10 relative).

The oracle's tensor commutator is pinned against the reference's J-coupled known answers in
tests/test_tensor_oracle.py; here every piece (TS_111 ... TS_222_ph) and the full commutator of
the device path are compared with the oracle on the same seeded operators."""
import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-10
PIECES = [1 | 8, 2, 4, 16, 32, 64, 127]


@pytest.mark.parametrize("emax,rank", [(2, 4), (4, 4), (4, 2), (4, 0)])
@pytest.mark.parametrize("hA,hB", [(-1, 1), (-1, -1), (1, 1), (1, -1)])
def test_tensor_commutator_pieces(oracles, engines, emax, rank, hA, hB):
    from oracle.oracle import TensorOracle
    o, eng = oracles(emax), engines(emax)
    t = TensorOracle(o, rank, 0)
    A, B = o.random(21, hA), t.random(22, hB)
    dA = eng.new_op(hA, A)
    dB = eng.new_tensor(rank, 0, hB, B)
    for pieces in PIECES:
        ref = t.commutator(A, hA, B, hB, pieces)
        dR = eng.new_tensor(rank, 0, -hA * hB)
        eng.tensor_commutator(dA, dB, dR, pieces)
        assert rel_err(dR.download(), ref) < TOL, pieces


def test_bch_tensor_matches_oracle(oracles, engines):
    from oracle.oracle import TensorOracle
    o, eng = oracles(4), engines(4)
    t = TensorOracle(o, 4, 0)
    G = o.random(31, -1) * 2e-3
    Q = t.random(32, 1)
    ref, n = t.bch(G, Q, 30, 1e-8)
    dG = eng.new_op(-1, G)
    dQ = eng.new_tensor(4, 0, 1, Q)
    assert eng.bch_tensor(dG, dQ, 30, 1e-8) == n
    assert rel_err(dQ.download(), ref) < TOL
    assert abs(dQ.frob() - t.frob(ref)) <= 1e-12 * t.frob(ref)


@pytest.mark.parametrize("mode,tol", [("bf16x6", 2e-6), ("bf16x3", 2e-5), ("tf32x3", 2e-6)])
@pytest.mark.parametrize("emax,rank", [(4, 4), (4, 2)])
def test_tensor_ladder_on_tensor_cores(oracles, emax, rank, mode, tol):
    """In a mixed mode the ladder's products through pp pairs and the cross-coupled products of
    the particle-hole term run as split-BF16 or TF32-compensated tcgen05 GEMMs (FP32
    accumulate); the rest of the tensor commutator stays FP64."""
    from imsrg_gb300 import Engine, make_basis
    from oracle.oracle import TensorOracle
    o = oracles(emax)
    t = TensorOracle(o, rank, 0)
    eng = Engine(make_basis(emax), device=0, precision=mode)
    A, B = o.random(23, -1), t.random(24, 1)
    dA = eng.new_op(-1, A)
    dB = eng.new_tensor(rank, 0, 1, B)
    for pieces in (32, 64, 127):
        ref = t.commutator(A, -1, B, 1, pieces)
        dR = eng.new_tensor(rank, 0, 1)
        eng.tensor_commutator(dA, dB, dR, pieces)
        err = rel_err(dR.download(), ref)
        assert err < tol, (pieces, err)
        assert err > 0.0  # the products did run in reduced precision
