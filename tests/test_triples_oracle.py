"""The perturbative triples correction in the oracle (restore_triples, src/IMSRG_MAGNUS.f90:767-902).

The reference has no test or golden value for it.  The restatement of its three-body element
commutator_223_single (src/commutators.f90:928-1325), nine J-coupled terms, is checked here
through properties the element must have: antisymmetry under the exchange of the two coupled
orbits of the bra (which trades terms 1-3 for terms 4-6) and of the ket, antisymmetry in
[L, R], and the correction's quadratic dependence on Omega."""
import numpy as np
import pytest


def _elements(o, n, seed):
    b = o.basis
    jj, ll, tz = np.array(b.jj), np.array(b.ll), np.array(b.itzp)
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        p, q, r, s, t, u = (int(x) for x in rng.integers(0, b.norbits, 6))
        if tz[p] + tz[q] + tz[r] != tz[s] + tz[t] + tz[u] or (ll[p] + ll[q] + ll[r] - ll[s] - ll[t] - ll[u]) % 2:
            continue
        for Jtot in range(1, 3 * int(jj.max()) + 1, 2):
            for jpq in range(abs(jj[p] - jj[q]), jj[p] + jj[q] + 1, 2):
                if not abs(jpq - jj[r]) <= Jtot <= jpq + jj[r]:
                    continue
                for jst in range(abs(jj[s] - jj[t]), jj[s] + jj[t] + 1, 2):
                    if abs(jst - jj[u]) <= Jtot <= jst + jj[u]:
                        out.append((p, q, r, s, t, u, Jtot, jpq, jst))
    return out


@pytest.mark.parametrize("emax", [2, 4])
def test_three_body_element_antisymmetry(oracles, emax):
    o = oracles(emax)
    jj = np.array(o.basis.jj)
    L, R = o.random(5, -1), o.random(6, 1)
    big = 0.0
    for (p, q, r, s, t, u, J, jpq, jst) in _elements(o, 40 if emax == 2 else 8, seed=emax):
        w = o.comm223(L, -1, R, 1, p, q, r, s, t, u, J, jpq, jst)
        tol = 1e-12 * max(abs(w), 1.0)
        assert abs(o.comm223(L, -1, R, 1, q, p, r, s, t, u, J, jpq, jst) +
                   (-1) ** ((jj[p] + jj[q] - jpq) // 2) * w) <= tol
        assert abs(o.comm223(L, -1, R, 1, p, q, r, t, s, u, J, jpq, jst) +
                   (-1) ** ((jj[s] + jj[t] - jst) // 2) * w) <= tol
        assert abs(o.comm223(R, 1, L, -1, p, q, r, s, t, u, J, jpq, jst) + w) <= tol
        big = max(big, abs(w))
    assert big > 1.0


def test_triples_quadratic_in_omega(oracles):
    from imsrg_gb300 import Engine, make_basis
    o = oracles(2)
    H = Engine(make_basis(2), device=-1).synthetic_hamiltonian(seed=1)
    OM = o.random(7, -1) * 0.05
    e1 = o.restore_triples(H, OM)
    assert e1 < 0.0
    assert abs(o.restore_triples(H, 2.0 * OM) - 4.0 * e1) <= 1e-12 * abs(e1)
    ch = o.three_channels()
    parts = sum(o.restore_triples(H, OM, q) for q in range(len(ch["J"])))
    assert abs(parts - e1) <= 1e-12 * abs(e1)
