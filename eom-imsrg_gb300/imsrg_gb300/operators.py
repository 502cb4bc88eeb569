"""Synthetic one-body observables for the BCH transformations of a flow (host input preparation).

r2_operator:  the intrinsic (1 - 1/A) r^2 operator from harmonic-oscillator radial matrix
              elements (the one-body part of initialize_rms_radius, src/operators.f90:446-477,
              which builds r^2 from the HO potential of calculate_h0_harm_osc), normal ordered:
              E0 = sum_holes (2j+1) <h|r^2|h>.  Per nucleon, <r^2> = E0 / A.
q2_operator:  a rank-2, even-parity one-body tensor  <a||r^2 Y_2||b>: the same HO radial r^2
              matrix elements (diagonal in l) times the reduced matrix element of Y_2, stored with
              the reference's tensor hermiticity f(b,a) = (-1)^((ja-jb)/2) f(a,b)
              (construct_random_rankX, src/brute_force_testing.f90:123-265).
Both are synthetic stand-ins (the reference builds its observables from the same HO pieces);
neither carries a two-body part.  With coefs = D(HO orbit, HF orbit) the one-body matrix is
moved to the Hartree-Fock basis first, F' = D^T F D, as transform_1b_to_HF and
transform_1b_to_HF_tensor do (src/HF_mod.f90:481-564, 695-758).
"""
from __future__ import annotations

import math

import numpy as np

HBARC = 197.3269788                   # MeV fm
M_NUC = float(np.float32(938.918725))  # the reference's default-real nucleon mass (src/basic_IMSRG.f90:141)


def ho_r2(na: int, nb: int, l: int) -> float:
    """<n_a l | r^2 / b^2 | n_b l> in the phase convention where the kinetic energy's
    off-diagonal elements are positive (so those of r^2 are negative)."""
    if na == nb:
        return 2 * na + l + 1.5
    if abs(na - nb) != 1:
        return 0.0
    n = max(na, nb)
    return -math.sqrt(n * (n + l + 0.5))


def threej(j1: int, j2: int, j3: int, m1: int, m2: int, m3: int) -> float:
    """Wigner 3j symbol with doubled arguments (Racah's formula)."""
    if m1 + m2 + m3 != 0 or not (abs(j1 - j2) <= j3 <= j1 + j2):
        return 0.0
    if any(abs(m) > j for m, j in ((m1, j1), (m2, j2), (m3, j3))):
        return 0.0
    if any((j + m) % 2 for m, j in ((m1, j1), (m2, j2), (m3, j3))):
        return 0.0
    f = math.factorial
    a = [(j1 + j2 - j3) // 2, (j1 - j2 + j3) // 2, (-j1 + j2 + j3) // 2]
    tri = f(a[0]) * f(a[1]) * f(a[2]) / f((j1 + j2 + j3) // 2 + 1)
    pre = math.sqrt(tri * f((j1 + m1) // 2) * f((j1 - m1) // 2) * f((j2 + m2) // 2) * f((j2 - m2) // 2) *
                    f((j3 + m3) // 2) * f((j3 - m3) // 2))
    s = 0.0
    for k in range(0, (j1 + j2 + j3) // 2 + 1):
        d = [k, (j1 + j2 - j3) // 2 - k, (j1 - m1) // 2 - k, (j2 + m2) // 2 - k, (j3 - j2 + m1) // 2 + k,
             (j3 - j1 - m2) // 2 + k]
        if min(d) < 0:
            continue
        s += (-1) ** k / (f(d[0]) * f(d[1]) * f(d[2]) * f(d[3]) * f(d[4]) * f(d[5]))
    return (-1) ** ((j1 - j2 - m3) // 2) * pre * s


def y2_reduced(la: int, ja: int, lb: int, jb: int, k: int = 2) -> float:
    """<la ja || Y_k || lb jb> (doubled j, Edmonds' convention)."""
    if (la + lb + k) % 2:
        return 0.0
    return ((-1) ** ((ja - 1) // 2) * math.sqrt((ja + 1) * (jb + 1) * (2 * k + 1) / (4 * math.pi)) *
            threej(ja, 2 * k, jb, -1, 0, 1))


def _onebody_slab(eng, size: int, f, coefs=None) -> np.ndarray:
    """A slab of `size` elements whose fhh / fpp / fph are f(orbit a, orbit b), or the
    elements of D^T F D when coefs D is given."""
    b = eng.basis
    if coefs is not None:
        N = b.norbits
        F = np.array([[f(a, c) for c in range(N)] for a in range(N)])
        D = np.asarray(coefs, dtype=np.float64)
        Fp = D.T @ F @ D
        f = lambda a, c: Fp[a, c]  # noqa: E731
    con = np.array(b.con)
    holes = [i for i in range(b.norbits) if con[i]]
    parts = [i for i in range(b.norbits) if not con[i]]
    A, P = len(holes), len(parts)
    s = np.zeros(size)
    o_hh, o_pp = 1, 1 + A * A
    o_ph = o_pp + P * P
    for i, a in enumerate(holes):
        for j, c in enumerate(holes):
            s[o_hh + i + j * A] = f(a, c)
    for i, a in enumerate(parts):
        for j, c in enumerate(parts):
            s[o_pp + i + j * P] = f(a, c)
    for i, a in enumerate(parts):
        for j, c in enumerate(holes):
            s[o_ph + i + j * P] = f(a, c)
    return s


def r2_operator(eng, coefs=None) -> np.ndarray:
    """Scalar slab of the intrinsic r^2 operator (fm^2), normal ordered w.r.t. the reference
    (in the basis of coefs when given)."""
    b = eng.basis
    A = b.Aprot + b.Aneut
    b2 = HBARC * HBARC / (M_NUC * b.hw)
    nn, ll, jj, tz, con = (np.array(x) for x in (b.nn, b.ll, b.jj, b.itzp, b.con))

    def f(a, c):
        if ll[a] != ll[c] or jj[a] != jj[c] or tz[a] != tz[c]:
            return 0.0
        return b2 * (1.0 - 1.0 / A) * ho_r2(int(nn[a]), int(nn[c]), int(ll[a]))

    s = _onebody_slab(eng, eng.slab, f, coefs)
    A_, P_ = b.nholes, b.norbits - b.nholes
    holes = [i for i in range(b.norbits) if con[i]]
    s[0] = sum((jj[h] + 1) * s[1 + k + k * A_] for k, h in enumerate(holes))
    return s


def q2_operator(eng, rank2: int = 4, coefs=None) -> np.ndarray:
    """Tensor slab (rank2 doubled, even parity) of <a||r^2 Y_2||b> (fm^2), l-diagonal radial part
    (in the basis of coefs when given)."""
    b = eng.basis
    b2 = HBARC * HBARC / (M_NUC * b.hw)
    nn, ll, jj, tz = (np.array(x) for x in (b.nn, b.ll, b.jj, b.itzp))
    k = rank2 // 2

    def g(a, c):
        if ll[a] != ll[c] or tz[a] != tz[c] or not (abs(jj[a] - jj[c]) <= rank2 <= jj[a] + jj[c]):
            return 0.0
        return b2 * ho_r2(int(nn[a]), int(nn[c]), int(ll[a])) * y2_reduced(int(ll[a]), int(jj[a]), int(ll[c]),
                                                                            int(jj[c]), k)

    def f(a, c):  # hermitian tensor: f(c,a) = (-1)^((ja-jc)/2) f(a,c)
        if a <= c:
            return g(a, c)
        return (-1) ** ((int(jj[c]) - int(jj[a])) // 2) * g(c, a)

    return _onebody_slab(eng, eng.tensor_sizes(rank2, 0)[0], f, coefs)
