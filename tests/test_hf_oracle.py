"""The oracle's Hartree-Fock restatement (src/HF_mod.f90) on the CPU.

The reference has no test that pins calc_HF: its eigenvectors come from LAPACK dsyev and are
fixed by the diagonal-positive sign rule.  The oracle uses numpy's LAPACK eigensolver the same
way, and these tests pin what does not depend on LAPACK's rounding:
  * normal_order and calc_HO agree with the library's own input preparation;
  * calc_HF ends with a diagonal Fock matrix (f_ph = 0), below the HO energy;
  * the two-body basis change is orthogonal (channel norms, round trip);
  * with a basis change that keeps holes and particles apart the reference state does not
    change, so the IMSRG(2) commutator - pinned to the reference's brute-force sums - is
    covariant: [T A, T B] = T [A, B].
"""
import numpy as np
import pytest

from helpers import rel_err


def _bare(emax, seed=5):
    from imsrg_gb300 import Engine, make_basis
    eng = Engine(make_basis(emax), device=-1)
    return eng, eng.synthetic_bare_hamiltonian(seed=seed), eng.synthetic_hamiltonian(seed=seed)


def _channel_norms(o, slab):
    """sum of squares of each channel's full (hermitian) matrix; o is an Oracle or an Engine"""
    info = o.block_info()
    b = o.basis
    A = b.nholes
    P = b.norbits - A
    off = 1 + A * A + P * P + P * A
    out = []
    for q in range(o.nblocks):
        npp, nph, nhh = int(info["npp"][q]), int(info["nph"][q]), int(info["nhh"][q])
        dims = [(npp, npp), (npp, nph), (npp, nhh), (nph, nph), (nhh, nhh), (nph, nhh)]
        s = 0.0
        for g, (n1, n2) in enumerate(dims):
            X = slab[off:off + n1 * n2]
            s += (1.0 if g in (0, 3, 4) else 2.0) * float(np.dot(X, X))
            off += n1 * n2
        out.append(s)
    return np.array(out)


def _particle_rotation(o, seed):
    """block-diagonal orthogonal D that rotates particles among themselves only"""
    rng = np.random.default_rng(seed)
    b = o.basis
    N = b.norbits
    con = np.array(b.con)
    D = np.eye(N)
    for st in o.sp_blocks():
        parts = [int(i) for i in st if con[i] == 0]
        if len(parts) < 2:
            continue
        Q, R = np.linalg.qr(rng.standard_normal((len(parts), len(parts))))
        Q = Q * np.sign(np.diag(R))[None, :]
        D[np.ix_(parts, parts)] = Q
    return D


def _one_body_to(o, op, D):
    """D^T f D on every (l, j, tz) block, without normal ordering"""
    out = op.copy()
    T = o._kin_matrix(op)
    for st in o.sp_blocks():
        ix = np.ix_(st, st)
        o._write_f(out, st, D[ix].T @ (T[ix] @ D[ix]))
    return out


@pytest.mark.parametrize("emax", [2, 4])
def test_normal_order_and_calc_ho_match_input_preparation(built_lib, oracles, emax):
    o = oracles(emax)
    eng, bare, H = _bare(emax)
    assert bare[0] == 0.0
    assert rel_err(o.normal_order(bare, 1), H) < 1e-13
    ho, D, E, it = o.calc_ho(bare)
    assert it == 0 and np.array_equal(D, np.eye(o.basis.norbits))
    assert abs(E - H[0]) <= 1e-12 * abs(H[0])
    assert rel_err(ho, H) < 1e-13


@pytest.mark.parametrize("emax", [2, 4])
def test_calc_hf_properties(built_lib, oracles, emax):
    o = oracles(emax)
    eng, bare, H = _bare(emax)
    hf, D, E, it = o.calc_hf(bare)
    b = o.basis
    A, P = b.nholes, b.norbits - b.nholes
    assert it > 2 and E == hf[0]
    assert E < H[0]  # HF lowers the energy of the HO Slater determinant
    assert np.allclose(D.T @ D, np.eye(b.norbits), atol=1e-13)
    fhh = hf[1:1 + A * A].reshape(A, A, order="F")
    fpp = hf[1 + A * A:1 + A * A + P * P].reshape(P, P, order="F")
    fph = hf[1 + A * A + P * P:1 + A * A + P * P + P * A]
    scale = np.abs(fpp).max()
    assert np.abs(fph).max() < 1e-12 * scale          # Brillouin: f_ph = 0 in the HF basis
    assert np.abs(fhh - np.diag(np.diag(fhh))).max() < 1e-12 * scale
    assert np.abs(fpp - np.diag(np.diag(fpp))).max() < 1e-12 * scale
    # the basis change is orthogonal channel by channel
    n0, n1 = _channel_norms(o, H), _channel_norms(o, hf)
    assert np.allclose(n0, n1, rtol=1e-12, atol=1e-12 * n0.max())
    # and its transpose undoes it
    back = o.transform_2b_to_hf(hf, D.T)
    assert rel_err(back[1 + A * A + P * P + P * A:], H[1 + A * A + P * P + P * A:]) < 1e-12


def test_calc_hf_iteration_limit(built_lib, oracles):
    o = oracles(2)
    _, bare, _ = _bare(2)
    with pytest.raises(RuntimeError):
        o.calc_hf(bare, max_iter=1)


@pytest.mark.parametrize("emax,seed", [(4, 11), (4, 12)])
def test_basis_change_commutes_with_commutator(built_lib, oracles, emax, seed):
    o = oracles(emax)
    D = _particle_rotation(o, seed)
    assert np.abs(D - np.eye(o.basis.norbits)).max() > 0.1
    # transform_2b_to_HF treats hermitian operators only (the reference's lower blocks are
    # plain transposes), so compare the hermitian [A, [A, B]] of hermitian A and B
    A, B = o.random(seed, 1), o.random(seed + 1, 1)

    def T(x):
        return o.transform_2b_to_hf(_one_body_to(o, x, D), D)

    def nested(X, Y):
        return o.commutator(X, 1, o.commutator(X, 1, Y, 1), -1)

    lhs = nested(T(A), T(B))
    rhs = T(nested(A, B))
    assert np.abs(rhs).max() > 1.0
    assert rel_err(lhs, rhs) < 1e-11


def test_sqop_to_hf_of_hamiltonian_is_hf_hamiltonian(built_lib, oracles):
    """sqop_to_HF of the bare Hamiltonian with calc_HF's coefficients gives calc_HF's result
    up to the mean field of the last iteration (converged to the HF tolerance)"""
    o = oracles(4)
    _, bare, _ = _bare(4)
    hf, D, E, it = o.calc_hf(bare)
    other = o.sqop_to_hf(bare, D)
    assert abs(other[0] - E) < 1e-5 * abs(E)
    assert rel_err(other[1:], hf[1:]) < 1e-5
