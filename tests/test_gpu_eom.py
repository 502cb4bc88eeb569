"""EOM-IMSRG on the device against the oracle (calculate_excited_states, src/EOM_IMSRG.f90:13-595).

The product imsrg_eom_matvec equals the oracle's restatement (itself pinned to the reference's
EOM known-answer formulas) to 1e-10 in FP64, for positive and negative parity.  The Lanczos
eigenvalues equal the eigenvalues of the dense EOM matrix: exactly symmetric when the
off-diagonal parts of H vanish (1e-9), and after a short IMSRG flow, where the reference runs it,
to the size of what the flow left undecoupled."""
import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu


def _decoupled(o, H):
    """H without f_ph and the pp-hh two-body arrays (where the White generator is nonzero)."""
    Hd = H.copy()
    od = o.white(H, 1) != 0.0
    od[0] = False
    Hd[od] = 0.0
    return Hd


@pytest.mark.parametrize("emax,rank,dpar", [(2, 0, 0), (2, 4, 0), (2, 2, 2), (4, 2, 0), (4, 6, 2)])
def test_eom_matvec_matches_oracle(oracles, engines, emax, rank, dpar):
    from imsrg_gb300.eom import LadderSpace
    from oracle.oracle import EomOracle
    o, eng = oracles(emax), engines(emax)
    assert eng.precision == "fp64"
    e = EomOracle(o, rank, dpar)
    space = LadderSpace(eng, rank, dpar)
    H = o.random(41 + rank, 1)
    dH = eng.new_op(1, H)
    rng = np.random.default_rng(rank + dpar)
    for _ in range(2):
        v = rng.standard_normal(space.n)
        assert rel_err(space.matvec(dH, v), e.matvec(H, v)) < 1e-10
    # unwrap / rewrap through the device
    X = space.unwrap(v)
    assert np.array_equal(X.download(), e.unwrap(v))
    assert np.array_equal(space.rewrap(X), v)


def test_eom_matvec_rejects_antihermitian_h(engines):
    from imsrg_gb300._lib import ImsrgError
    from imsrg_gb300.eom import LadderSpace
    eng = engines(2)
    space = LadderSpace(eng, 2, 0)
    G = eng.new_op(-1)
    with pytest.raises(ImsrgError):
        space.matvec(G, np.zeros(space.n))


@pytest.mark.parametrize("rank,dpar,nev", [(0, 0, 3), (4, 0, 4), (2, 2, 4)])
def test_lanczos_matches_dense_eigenvalues(oracles, engines, rank, dpar, nev):
    from imsrg_gb300.eom import LadderSpace
    from oracle.oracle import EomOracle
    o, eng = oracles(2), engines(2)
    e = EomOracle(o, rank, dpar)
    Hd = _decoupled(o, eng.synthetic_hamiltonian(seed=3))
    M = e.matrix(Hd)
    assert np.abs(M - M.T).max() <= 1e-12 * np.abs(M).max()
    w = np.linalg.eigvalsh(M)
    ref = np.sort(w[np.argsort(np.abs(w))[:nev]])
    space = LadderSpace(eng, rank, dpar)
    E, V, info = space.lanczos(eng.new_op(1, Hd), nev)
    assert np.abs(E - ref).max() <= 1e-9 * np.abs(w).max(), (E, ref)
    # normalised eigenvectors with small residuals
    for i in range(nev):
        assert abs(np.linalg.norm(V[:, i]) - 1.0) < 1e-12
        assert np.linalg.norm(M @ V[:, i] - E[i] * V[:, i]) < 1e-7 * np.abs(w).max()
    assert info["matvecs"] >= nev


def test_excited_states_after_flow(engines, tmp_path):
    """calculate_excited_states (J=0+) on H(s) after a Magnus flow at eMax=4: the EOM matrix is
    symmetric up to what is left of the off-diagonal parts, and the Lanczos energies agree with
    the dense eigenvalues of the device-built matrix to that level."""
    from imsrg_gb300.eom import LadderSpace, calculate_excited_states
    from imsrg_gb300.flow import magnus_decouple
    eng = engines(4)
    bare = eng.synthetic_bare_hamiltonian(seed=2)
    Hop = eng.new_op(1, bare)
    eng.calc_hf(Hop)
    ops = {}
    magnus_decouple(eng, Hop.download(), max_steps=60, ops=ops)
    HS = ops["HS"]
    rows, info = calculate_excited_states(eng, HS, 0, 0, 3, prefix="test", output_dir=str(tmp_path))
    lines = (tmp_path / "test_EOM_spec_law0.dat").read_text().splitlines()
    assert len(lines) == 3 and all(len(x) == 48 for x in lines)
    space = LadderSpace(eng, 0, 0)
    n = space.n
    M = np.zeros((n, n))
    for k in range(n):
        ek = np.zeros(n)
        ek[k] = 1.0
        M[:, k] = space.matvec(HS, ek)
    asym = np.abs(M - M.T).max() / np.abs(M).max()
    w = np.linalg.eigvals(M).real
    ref = np.sort(w[np.argsort(np.abs(w))[:3]])
    E = np.array([r[0] for r in rows])
    assert np.abs(E - ref).max() <= max(10 * asym, 1e-8) * np.abs(w).max(), (E, ref, asym)
    for dE, Etot, n1 in rows:
        assert abs(Etot - (dE + HS.E0)) < 1e-9 and 0.0 <= n1 <= 1.0 + 1e-12


@pytest.mark.parametrize("mode,tol", [("bf16x6", 1e-5), ("bf16x3", 1e-4)])
def test_eom_matvec_mixed_precision(oracles, mode, tol):
    """In the mixed modes the product's GEMMs run as FP32 SIMT tiles and the 122 / 212 sums in FP32."""
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300.eom import LadderSpace
    from oracle.oracle import EomOracle
    o = oracles(4)
    eng = Engine(make_basis(4), device=0, precision=mode)
    e = EomOracle(o, 4, 0)
    space = LadderSpace(eng, 4, 0)
    H = eng.synthetic_hamiltonian(seed=5)
    v = np.random.default_rng(9).standard_normal(space.n)
    assert rel_err(space.matvec(eng.new_op(1, H), v), e.matvec(H, v)) < tol


def test_eom_graph_follows_precision_and_h(oracles):
    """The replayed product is recaptured when the context's precision or the H operator changes."""
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300.eom import LadderSpace
    from oracle.oracle import EomOracle
    o = oracles(4)
    eng = Engine(make_basis(4), device=0)
    e = EomOracle(o, 2, 0)
    space = LadderSpace(eng, 2, 0)
    H1, H2 = eng.synthetic_hamiltonian(seed=6), eng.synthetic_hamiltonian(seed=7)
    d1, d2 = eng.new_op(1, H1), eng.new_op(1, H2)
    v = np.random.default_rng(2).standard_normal(space.n)
    r1, r2 = e.matvec(H1, v), e.matvec(H2, v)
    for _ in range(2):
        assert rel_err(space.matvec(d1, v), r1) < 1e-10
    assert rel_err(space.matvec(d2, v), r2) < 1e-10
    eng.set_precision("bf16x6")
    assert rel_err(space.matvec(d2, v), r2) < 1e-5
    eng.set_precision("fp64")
    assert rel_err(space.matvec(d2, v), r2) < 1e-10
