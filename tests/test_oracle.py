"""The CPU oracle against the reference's own known-answer tests.

The reference pins its commutators only with brute-force formulas
(test_scalar_scalar_commutator, src/brute_force_testing.f90:483-607, tolerances
1e-10 for 0b/1b and 1e-6 for 2b); these tests run the same comparison on the oracle,
plus standard angular-momentum identities for its 6j / 9j symbols.
"""
import json
import os

import numpy as np
import pytest

from imsrg_gb300.basis import ho_orbits, make_basis
from oracle.oracle import Oracle, lib

HERE = os.path.dirname(os.path.abspath(__file__))


def test_hk_bases_match_reference_files():
    gold = json.load(open(os.path.join(HERE, "golden", "hk_bases.json")))
    for e in range(3, 15):
        mine = [list(o) for o in ho_orbits(e)]
        ref = [[r[0], r[1], r[2], r[3], int(round(r[4]))] for r in gold[f"hk{e}"]]
        assert mine == ref, f"hk{e}"
    b = make_basis(10)
    assert list(b.con[:30]) == gold["hole_scheme_8_8"]


def test_sixj_identities():
    L = lib()
    # {a b 0; d e f} = (-1)^(a+e+f) delta_ab delta_de / sqrt((2a+1)(2d+1))
    for a in (1, 3, 5, 7):
        for d in (1, 3, 5):
            for f in range(abs(a - d), a + d + 1, 2):
                v = L.orc_sixj(a, a, 0, d, d, f)
                ref = (-1) ** ((a + d + f) // 2) / np.sqrt((a + 1) * (d + 1))
                assert abs(v - ref) < 1e-13
    # orthogonality: sum_x (2x+1)(2f+1) {a b x; c d f}{a b x; c d g} = delta_fg
    for (a, b, c, d) in [(1, 3, 5, 3), (5, 5, 3, 7), (9, 7, 5, 11), (11, 13, 9, 15)]:
        fs = [f for f in range(0, 40, 2) if abs(a - d) <= f <= a + d and abs(b - c) <= f <= b + c]
        xs = [x for x in range(0, 40, 2) if abs(a - b) <= x <= a + b and abs(c - d) <= x <= c + d]
        for f in fs:
            for g in fs:
                s = sum((x + 1) * (f + 1) * L.orc_sixj(a, b, x, c, d, f) * L.orc_sixj(a, b, x, c, d, g) for x in xs)
                assert abs(s - (1.0 if f == g else 0.0)) < 1e-12


def test_ninej_reduces_to_sixj():
    L = lib()
    # {a b c; d e f; g h 0} = delta_cf delta_gh (-1)^(b+c+d+g) / sqrt((2c+1)(2g+1)) {a b c; e d g}
    rng = np.random.default_rng(3)
    checked = 0
    for _ in range(400):
        a, b, d, e = (int(x) for x in 2 * rng.integers(0, 5, 4) + 1)
        c = int(rng.integers(abs(a - b) // 2, (a + b) // 2 + 1)) * 2
        g = int(rng.integers(abs(a - d) // 2, (a + d) // 2 + 1)) * 2
        if not (abs(d - e) <= c <= d + e and abs(b - e) <= g <= b + e):
            continue
        v = L.orc_ninej(a, b, c, d, e, c, g, g, 0)
        ref = (-1) ** ((b + c + d + g) // 2) / np.sqrt((c + 1) * (g + 1)) * L.orc_sixj(a, b, c, e, d, g)
        assert abs(v - ref) < 1e-12
        checked += 1
    assert checked > 50


@pytest.mark.parametrize("hA,hB", [(-1, 1), (1, 1), (-1, -1)])
def test_commutator_vs_brute_force_emax2_all_elements(oracles, hA, hB):
    o = oracles(2)
    b = o.basis
    A = o.random(11, hA)
    B = o.random(12, hB)
    hR = -hA * hB
    RES = o.commutator(A, hA, B, hB, hR)
    assert abs(RES[0] - o.bf_0body(A, hA, B, hB)) < 1e-10 * max(1.0, abs(RES[0]))
    N = b.norbits
    for a in range(N):
        for c in range(N):
            ref = o.bf_1body(A, hA, B, hB, a, c)
            assert abs(o.f_elem(RES, hR, a, c) - ref) < 1e-10 * max(1.0, abs(ref)), (a, c)
    jj, ll, tz = b.jj, b.ll, b.itzp
    worst = 0.0
    for a in range(N):
        for bb in range(N):
            for c in range(N):
                for d in range(N):
                    if (ll[a] + ll[bb]) % 2 != (ll[c] + ll[d]) % 2 or tz[a] + tz[bb] != tz[c] + tz[d]:
                        continue
                    lo = max(abs(jj[a] - jj[bb]), abs(jj[c] - jj[d]))
                    hi = min(jj[a] + jj[bb], jj[c] + jj[d])
                    for J in range(lo, hi + 1, 2):
                        ref = o.bf_2body(A, hA, B, hB, a, bb, c, d, J)
                        worst = max(worst, abs(o.v_elem(RES, hR, a, bb, c, d, J) - ref))
    # the reference's 2b tolerance (src/brute_force_testing.f90:591); the gap comes from
    # its truncated 1/sqrt(2) literal in commutator_222_ph, which the oracle keeps
    assert worst < 1e-6


def test_commutator_vs_brute_force_emax4_sampled(oracles):
    o = oracles(4)
    b = o.basis
    hA, hB = -1, 1
    A = o.random(21, hA)
    B = o.random(22, hB)
    hR = 1
    RES = o.commutator(A, hA, B, hB, hR)
    assert abs(RES[0] - o.bf_0body(A, hA, B, hB)) < 1e-10 * max(1.0, abs(RES[0]))
    rng = np.random.default_rng(5)
    N = b.norbits
    for _ in range(50):
        a, c = (int(x) for x in rng.integers(0, N, 2))
        ref = o.bf_1body(A, hA, B, hB, a, c)
        assert abs(o.f_elem(RES, hR, a, c) - ref) < 1e-10 * max(1.0, abs(ref))
    jj, ll, tz = b.jj, b.ll, b.itzp
    done = 0
    while done < 15:
        a, bb, c, d = (int(x) for x in rng.integers(0, N, 4))
        if (ll[a] + ll[bb]) % 2 != (ll[c] + ll[d]) % 2 or tz[a] + tz[bb] != tz[c] + tz[d]:
            continue
        done += 1
        lo = max(abs(jj[a] - jj[bb]), abs(jj[c] - jj[d]))
        hi = min(jj[a] + jj[bb], jj[c] + jj[d])
        for J in range(lo, hi + 1, 2):
            ref = o.bf_2body(A, hA, B, hB, a, bb, c, d, J)
            assert abs(o.v_elem(RES, hR, a, bb, c, d, J) - ref) < 1e-6


def test_pieces_compose_to_full_commutator(oracles):
    o = oracles(4)
    L, R = o.random(31, -1), o.random(32, 1)
    full = o.commutator(L, -1, R, 1, 1)
    RES = o.new()
    w1, w2 = o.new(), o.new()
    RES[0] = o.commutator_110(L, -1, R, 1) + o.commutator_220(L, -1, R, 1)
    RCC = o.calculate_cross_coupled(R, 1)
    LCC = o.calculate_cross_coupled(L, -1)
    o.commutator_111(L, -1, R, 1, RES, 1)
    o.commutator_121(L, -1, R, 1, RES, 1)
    o.commutator_122(L, -1, R, 1, RES, 1)
    o.commutator_222_pp_hh(L, -1, R, 1, RES, 1, w1, w2)
    o.commutator_221(L, -1, R, 1, RES, 1, w1, w2)
    o.commutator_222_ph(LCC, -1, RCC, 1, RES, 1)
    assert np.array_equal(full, RES)


def test_bch_and_magnus_small(oracles):
    o = oracles(2)
    H = o.random(41, 1) * 0.05
    G = o.random(42, -1) * 0.01
    HS, n = o.bch_expand(G, H)
    assert n > 1
    # unitary transformation of a hermitian operator stays hermitian: e^G H e^-G with
    # G anti-hermitian; first-order check against H + [G,H]
    first = H + o.commutator(G, -1, H, 1, 1)
    assert np.max(np.abs(HS - first)) < 50 * np.max(np.abs(G)) ** 2 * np.max(np.abs(H)) * 100
    DG = o.random(43, -1) * 0.01
    eta = DG.copy()
    used = o.magnus_expand(DG, G)
    assert used >= 1
    assert np.max(np.abs(DG - eta)) > 0


def test_atan_generators_against_white(oracles):
    """build_gs_atan / atanxx / w2 (src/generators.f90:109-374) share White's numerators N and
    denominators E: atan = atan(2 N/E)/2 = atan(2 white)/2 element by element; atanxx with the
    numerators and denominators of one operator is atan; w2 = 1.5 atan + 0.5 atanxx(H, [atan, H])"""
    o = oracles(4)
    H = o.random(51, 1)
    w, a = o.white(H, 1), o.atan(H, 1)
    assert np.abs(w).max() > 0
    assert np.allclose(a, 0.5 * np.arctan(2 * w), rtol=1e-13, atol=1e-15)
    assert np.array_equal(o.atanxx(H, H), a)
    H2 = o.commutator(a, -1, H, 1)
    assert np.allclose(o.w2(H, 1), 1.5 * a + 0.5 * o.atanxx(H, H2), rtol=0, atol=1e-15)


def test_cr_expand_series(oracles):
    """CR_EXPAND (src/IMSRG_MAGNUS.f90:532-617): H + [G,H]/2! + [G,[G,H]]/3! + ... with the
    reference's stop (term norm times coefficient below conv) and at most 13 nested commutators."""
    o = oracles(2)
    G = o.random(71, -1) * 0.05
    H = o.random(72, 1)
    CR, n = o.cr_expand(G, H, 14, 1e-6)
    ref, ad, coef = H.copy(), H.copy(), 1.0
    for k in range(2, 15):
        coef /= k
        ad = o.commutator(G, -1, ad, 1)
        ref += coef * ad
        if o.frob(ad) * coef < 1e-6:
            break
    assert n == k - 1
    assert np.allclose(CR, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
    # capped series: no error, all 13 terms
    CR2, n2 = o.cr_expand(G * 40, H, 14, 1e-30)
    assert n2 == 13 and np.all(np.isfinite(CR2))


def test_restore_quadrupoles_structure(oracles):
    """restore_quadrupoles (src/IMSRG_MAGNUS.f90:908-1070): with a zero Omega the quadrupole BCH
    reduces to H, and its change of H(s) shrinks with Omega (at first order through the ladder
    products the reference's workspace holds in channels without pp or hh pairs, at second order
    elsewhere)."""
    o = oracles(4)
    b = o.basis
    X, OM = o.random(91, 1), o.random(92, -1) * 0.05
    Q = o.restore_quadrupoles(X, 1, OM, -1)
    ref, _ = o.bch_expand(OM, X)
    hq, _ = o.bch_expand_quads(OM, X)
    assert np.count_nonzero(Q) > 0
    assert np.abs(hq - ref).max() > 0.0
    h0, n0 = o.bch_expand_quads(OM * 0.0, X)
    assert n0 == 1 and np.array_equal(h0, X)
    # halving Omega at least halves the difference
    hq2, _ = o.bch_expand_quads(OM * 0.5, X)
    ref2, _ = o.bch_expand(OM * 0.5, X)
    r = np.abs(hq2 - ref2).max() / np.abs(hq - ref).max()
    assert 0.1 < r < 0.55
