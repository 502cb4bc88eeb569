"""EOM-IMSRG ladder operators in the oracle (calculate_excited_states, src/EOM_IMSRG.f90:13-595).

The EOM product of matvec_nonzeroX_prod is [H, X] for an excitation operator X of rank lambda,
read back on its particle-hole and pp-hh amplitudes.  The reference tests its EOM_TS_commutator_*
routines against the J-coupled expressions EOM_scalar_tensor_1body_comm / _2body_comm
(src/brute_force_testing.f90:1467-1624, 2348-2437, 3601-3709); the oracle restates both
expressions and computes the product through two general scalar-tensor commutators.  Here every
one-body amplitude and a seeded sample of two-body amplitudes agree to 1e-10, for positive and
negative parity, and the amplitude vector round-trips through unwrap_tensor / rewrap_tensor."""
import numpy as np
import pytest


def _eom(oracles, emax, rank, dpar):
    from oracle.oracle import EomOracle
    o = oracles(emax)
    return o, EomOracle(o, rank, dpar)


def _samples(o, rank, dpar, n, seed):
    b = o.basis
    jj, ll, tz, con = (np.array(x) for x in (b.jj, b.ll, b.itzp, b.con))
    P, A = np.flatnonzero(con == 0), np.flatnonzero(con == 1)
    rng = np.random.default_rng(seed)
    out, k = [], 0
    while k < n:
        a, bb = (int(x) for x in rng.choice(P, 2))
        c, d = (int(x) for x in rng.choice(A, 2))
        if (ll[a] + ll[bb] + dpar // 2) % 2 != (ll[c] + ll[d]) % 2 or tz[a] + tz[bb] != tz[c] + tz[d]:
            continue
        k += 1
        for J1 in range(abs(jj[a] - jj[bb]), jj[a] + jj[bb] + 1, 2):
            for J2 in range(abs(jj[c] - jj[d]), jj[c] + jj[d] + 1, 2):
                if abs(J1 - J2) <= rank <= J1 + J2:
                    out.append((a, bb, c, d, J1, J2))
    return out


@pytest.mark.parametrize("rank,dpar", [(0, 0), (2, 0), (4, 0), (2, 2), (6, 2)])
def test_eom_product_known_answers(oracles, rank, dpar):
    o, e = _eom(oracles, 2, rank, dpar)
    b = o.basis
    H = o.random(31, 1)
    v = np.random.default_rng(rank + dpar).standard_normal(e.n)
    X = e.unwrap(v)
    Y = e.unwrap(e.matvec(H, v))
    A, P = b.nholes, b.norbits - b.nholes
    off = 1 + A * A + P * P
    parts, holes = np.flatnonzero(np.array(b.con) == 0), np.flatnonzero(np.array(b.con) == 1)
    scale = max(np.abs(Y).max(), 1.0)
    n1 = 0
    for ip, p in enumerate(parts):
        for ih, h in enumerate(holes):
            ref = e.bf1(H, X, int(p), int(h))
            assert abs(Y[off + ip + ih * P] - ref) <= 1e-10 * scale, (p, h)
            n1 += ref != 0.0
    assert n1 == e.n1b
    for (a, bb, c, d, J1, J2) in _samples(o, rank, dpar, 10, seed=7 + rank):
        ref = e.bf2(H, X, a, bb, c, d, J1, J2)
        assert abs(e.pphh(Y, a, bb, c, d, J1, J2) - ref) <= 1e-10 * scale, (a, bb, c, d, J1, J2)


@pytest.mark.parametrize("rank,dpar", [(2, 0), (2, 2)])
def test_amplitude_vector_round_trip(oracles, rank, dpar):
    o, e = _eom(oracles, 4, rank, dpar)
    m = e.amplitude_map()
    assert len(np.unique(m["pos"])) == e.n and np.all(m["kind"][:e.n1b] == 0) and np.all(m["kind"][e.n1b:] > 0)
    v = np.random.default_rng(3).standard_normal(e.n)
    X = e.unwrap(v)
    assert np.array_equal(e.rewrap(X), v)
    # only fph and the pp-hh arrays are written (plus the transposed copies of J1 == J2 blocks)
    mirrors = m["mirror"][m["mirror"] >= 0]
    assert np.count_nonzero(X) == e.n + len(mirrors)
    assert np.array_equal(X[mirrors], v[m["mirror"] >= 0])


def test_decoupled_product_is_symmetric(oracles):
    """With the off-diagonal parts of H removed (f_ph and the pp-hh two-body arrays) the EOM
    matrix is symmetric, the case the reference's symmetric Lanczos (dsaupd) assumes."""
    o, e = _eom(oracles, 2, 2, 0)
    H = o.random(32, 1)
    Hd = H.copy()
    od = o.white(H, 1) != 0.0
    od[0] = False
    Hd[od] = 0.0
    M = e.matrix(Hd)
    assert np.abs(M - M.T).max() <= 1e-12 * np.abs(M).max()
    Mf = e.matrix(H)
    assert np.abs(Mf - Mf.T).max() > 1e-3 * np.abs(Mf).max()


@pytest.mark.parametrize("emax,rank,dpar", [(2, 0, 0), (2, 4, 0), (4, 2, 0), (4, 2, 2), (4, 6, 2)])
def test_library_amplitude_map_matches_oracle(built_lib, oracles, emax, rank, dpar):
    """imsrg_eom_amplitude_map (host-only context) equals the oracle's unwrap_tensor order."""
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300.eom import LadderSpace
    eng = Engine(make_basis(emax), device=-1)
    space = LadderSpace(eng, rank, dpar)
    _, e = _eom(oracles, emax, rank, dpar)
    assert (space.n, space.n1b) == (e.n, e.n1b)
    got, ref = space.amplitude_map(), e.amplitude_map()
    for k in ("pos", "kind", "phase", "mirror"):
        assert np.array_equal(got[k], ref[k]), k
