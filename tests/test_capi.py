"""C ABI boundary checks that need no GPU: symbols, host-only layout, input preparation."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from imsrg_gb300 import Engine, ImsrgError, make_basis
from imsrg_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "imsrg_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(imsrg_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(built_lib):
    L = C.CDLL(built_lib)
    syms = header_symbols()
    assert len(syms) >= 40
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(_lib.exported_symbols())


@pytest.mark.parametrize("emax", [2, 4, 6])
def test_host_layout_matches_oracle(built_lib, oracles, emax):
    o = oracles(emax)
    eng = Engine(make_basis(emax), device=-1)
    assert eng.slab == o.slab and eng.cc_size == o.cc_size and eng.wcc_size == o.wcc_size
    assert eng.nblocks == o.nblocks and eng.ncc == o.ncc
    a, b = eng.block_info(), o.block_info()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    for q in range(eng.nblocks):
        for cls in range(3):
            assert np.array_equal(eng.block_pairs(q, cls), o.block_pairs(q, cls))
    ca, cb = eng.cc_info(), o.cc_info()
    for k in ca:
        assert np.array_equal(ca[k], cb[k]), k


def test_emax10_layout_sizes(built_lib):
    eng = Engine(make_basis(10), device=-1)
    info = eng.block_info()
    assert eng.nblocks == 132 and eng.ncc == 88
    assert int(info["npp"].max()) == 1291 and int(info["nph"].max()) == 74 and int(info["nhh"].max()) == 5
    cc = eng.cc_info()
    assert int(cc["rlen"].max()) == 2682 and int(cc["nph"].max()) == 74


def test_synthetic_hamiltonian(built_lib, oracles):
    emax = 4
    eng = Engine(make_basis(emax), device=-1)
    o = oracles(emax)
    H = eng.synthetic_hamiltonian(seed=7)
    H2 = eng.synthetic_hamiltonian(seed=7)
    H3 = eng.synthetic_hamiltonian(seed=8)
    assert np.array_equal(H, H2) and not np.array_equal(H, H3)
    assert np.all(np.isfinite(H))
    info = o.block_info()
    b = o.basis
    A, P = b.nholes, b.norbits - b.nholes
    fhh = H[1:1 + A * A].reshape(A, A, order="F")
    fpp = H[1 + A * A:1 + A * A + P * P].reshape(P, P, order="F")
    assert np.allclose(fhh, fhh.T) and np.allclose(fpp, fpp.T)
    off = 1 + A * A + P * P + P * A
    for q in range(o.nblocks):
        npp, nph, nhh = int(info["npp"][q]), int(info["nph"][q]), int(info["nhh"][q])
        dims = [(npp, npp), (npp, nph), (npp, nhh), (nph, nph), (nhh, nhh), (nph, nhh)]
        for g, (n1, n2) in enumerate(dims):
            X = H[off:off + n1 * n2].reshape(n1, n2, order="F")
            if g in (0, 3, 4):
                assert np.allclose(X, X.T), (q, g)
            off += n1 * n2
    # kinetic energy dominates the diagonal: particles above holes
    assert fpp.diagonal().min() > fhh.diagonal().max()


def test_error_paths(built_lib):
    b = make_basis(2)
    bad = make_basis(2)
    bad.jj = bad.jj.copy()
    bad.jj[0] = 2  # 2j must be odd
    with pytest.raises(ImsrgError):
        Engine(bad, device=-1)
    eng = Engine(b, device=-1)
    with pytest.raises(ImsrgError) as e:
        eng.new_op(1)
    assert e.value.code == 6  # IMSRG_ERR_UNSUPPORTED on a host-only context
