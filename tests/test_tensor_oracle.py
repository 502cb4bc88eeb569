"""Known-answer pin of the oracle's scalar-tensor commutator (BCH_TENSOR's building block).

The reference tests TS_commutator_* against its own J-coupled expressions
scalar_tensor_1body_comm / scalar_tensor_2body_comm (src/brute_force_testing.f90:912-1056,
2159-2247, 3223-3393).  The oracle restates both; here every one-body element and a seeded
sample of two-body elements agree to 1e-10 for random operators (scalar anti-hermitian, as
Omega in BCH_TENSOR, and hermitian, as H in the EOM product; tensor hermitian or
anti-hermitian; ranks 0, 1 and 2).
"""
import numpy as np
import pytest


def _tensor(oracles, emax, rank):
    from oracle.oracle import TensorOracle
    o = oracles(emax)
    return o, TensorOracle(o, rank, 0)


def _samples(o, rank, n, seed):
    b = o.basis
    N = b.norbits
    jj, ll, tz = np.array(b.jj), np.array(b.ll), np.array(b.itzp)
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        a, bb, c, d = (int(x) for x in rng.integers(0, N, 4))
        if (ll[a] + ll[bb]) % 2 != (ll[c] + ll[d]) % 2 or tz[a] + tz[bb] != tz[c] + tz[d]:
            continue
        for J1 in range(abs(jj[a] - jj[bb]), jj[a] + jj[bb] + 1, 2):
            for J2 in range(abs(jj[c] - jj[d]), jj[c] + jj[d] + 1, 2):
                if abs(J1 - J2) <= rank <= J1 + J2:
                    out.append((a, bb, c, d, J1, J2))
    return out


@pytest.mark.parametrize("emax,rank,hA,hB,n2", [(2, 4, -1, 1, 25), (2, 2, -1, -1, 25), (4, 4, -1, 1, 6),
                                                (2, 0, 1, 1, 25), (2, 2, 1, -1, 25), (2, 4, 1, 1, 25)])
def test_scalar_tensor_commutator_known_answers(oracles, emax, rank, hA, hB, n2):
    o, t = _tensor(oracles, emax, rank)
    A, B = o.random(3, hA), t.random(4, hB)
    RES = t.commutator(A, hA, B, hB)
    hR = -hA * hB
    N = o.basis.norbits
    scale = max(np.abs(RES).max(), 1.0)
    for a in range(N):
        for b in range(N):
            assert abs(t.f_elem(RES, hR, a, b) - t.bf1(A, hA, B, hB, a, b)) <= 1e-10 * scale, (a, b)
    for (a, b, c, d, J1, J2) in _samples(o, rank, n2, seed=emax + rank):
        ref = t.bf2(A, hA, B, hB, a, b, c, d, J1, J2)
        assert abs(t.elem(RES, hR, a, b, c, d, J1, J2) - ref) <= 1e-10 * scale, (a, b, c, d, J1, J2)


def test_tensor_pieces_compose(oracles):
    o, t = _tensor(oracles, 2, 4)
    A, B = o.random(5, -1), t.random(6, 1)
    full = t.commutator(A, -1, B, 1)
    parts = np.zeros_like(full)
    # 111 and 122 assign; the rest accumulate onto them
    parts += t.commutator(A, -1, B, 1, 1 | 8)
    for m in (2, 4, 16, 32, 64):
        parts += t.commutator(A, -1, B, 1, m)
    assert np.allclose(parts, full, rtol=0, atol=1e-10 * np.abs(full).max())


def test_bch_tensor_first_order(oracles):
    o, t = _tensor(oracles, 2, 4)
    G = o.random(7, -1) * 1e-4
    Q = t.random(8, 1)
    out, n = t.bch(G * 0.0, Q)
    assert n == 1 and np.array_equal(out, Q)
    out, n = t.bch(G, Q, conv=1e-12)
    assert n >= 2
    lin = Q + t.commutator(G, -1, Q, 1)
    assert np.abs(out - lin).max() < 1e-5 * np.abs(Q).max()
    assert np.abs(out - Q).max() > 1e-6


@pytest.mark.parametrize("emax,rank", [(2, 4), (4, 2), (4, 4), (10, 4)])
def test_device_tensor_layout_matches_oracle(built_lib, oracles, emax, rank):
    from imsrg_gb300 import Engine, make_basis
    eng = Engine(make_basis(emax), device=-1)
    slab, nb = eng.tensor_sizes(rank, 0)
    if emax > 4:  # the oracle is not run at this size: the layout only has to build
        assert slab > eng.slab and nb > 0
        return
    o, t = _tensor(oracles, emax, rank)
    assert (slab, nb) == (t.slab, t.nblocks)
    info, ref = eng.tensor_block_info(rank, 0), t.block_info()
    for k in ("J1", "J2", "Tz", "P1"):
        assert np.array_equal(info[k], ref[k])
