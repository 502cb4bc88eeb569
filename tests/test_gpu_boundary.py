"""The Fortran-facing per-array boundary: imsrg_op_upload / imsrg_op_download.

A Fortran caller holds an sq_op as separate allocations, one column-major array per
(channel q, array g) (op%mat(q)%gam(g)%X, src/basic_IMSRG.f90:65-76, 623-628) plus
fhh, fph, fpp, and passes c_loc of each.  Here every array lives in its own numpy buffer in
Fortran order, the way those pointers arrive.  Uploading through the per-array call and
downloading through it must round-trip bit for bit, agree bit for bit with the slab calls,
and give bit-identical commutators.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fortran_arrays(eng, slab):
    """The slab as separate Fortran-ordered allocations: (E0, fhh, fph, fpp, [gam per (q, g)])."""
    A, N = eng.basis.nholes, eng.basis.norbits
    P = N - A
    o = 1
    fhh = slab[o:o + A * A].reshape(A, A, order="F").copy(order="F"); o += A * A
    fpp = slab[o:o + P * P].reshape(P, P, order="F").copy(order="F"); o += P * P
    fph = slab[o:o + P * A].reshape(P, A, order="F").copy(order="F"); o += P * A
    info = eng.block_info()
    gam = []
    for q in range(eng.nblocks):
        npp, nph, nhh = int(info["npp"][q]), int(info["nph"][q]), int(info["nhh"][q])
        for n1, n2 in ((npp, npp), (npp, nph), (npp, nhh), (nph, nph), (nhh, nhh), (nph, nhh)):
            n = n1 * n2
            gam.append(slab[o:o + n].reshape(n1, n2, order="F").copy(order="F") if n else None)
            o += n
    assert o == slab.size
    return slab[0], fhh, fph, fpp, gam


def _ptrs(gam):
    arr = (C.c_void_p * len(gam))()
    for k, g in enumerate(gam):
        arr[k] = g.ctypes.data if g is not None else None
    return arr


@pytest.mark.parametrize("emax", [2, 4])
def test_per_array_upload_download_round_trip(built_lib, oracles, emax):
    from imsrg_gb300 import Engine, make_basis
    eng = Engine(make_basis(emax), device=0)
    o = oracles(emax)
    slab = o.random(71 + emax, 1)
    slab[0] = -123.25
    E0, fhh, fph, fpp, gam = _fortran_arrays(eng, slab)
    pd = C.POINTER(C.c_double)
    op = eng.new_op(1)
    st = eng.L.imsrg_op_upload(eng.h, op.h, C.cast(_ptrs(gam), C.POINTER(C.c_void_p)), fhh.ctypes.data_as(pd),
                               fph.ctypes.data_as(pd), fpp.ctypes.data_as(pd), float(E0))
    assert st == 0, eng.L.imsrg_last_error(eng.h)
    assert np.array_equal(op.download(), slab)  # the slab call reads back what the array call wrote
    # download through the per-array call into fresh Fortran-ordered buffers
    _, fhh2, fph2, fpp2, gam2 = _fortran_arrays(eng, np.zeros_like(slab))
    e0 = C.c_double()
    st = eng.L.imsrg_op_download(eng.h, op.h, C.cast(_ptrs(gam2), C.POINTER(C.c_void_p)), fhh2.ctypes.data_as(pd),
                                 fph2.ctypes.data_as(pd), fpp2.ctypes.data_as(pd), C.byref(e0))
    assert st == 0, eng.L.imsrg_last_error(eng.h)
    assert e0.value == E0
    for a, b in ((fhh, fhh2), (fph, fph2), (fpp, fpp2)):
        assert np.array_equal(a, b)
    for a, b in zip(gam, gam2):
        assert (a is None and b is None) or np.array_equal(a, b)
    # same commutator as the slab-uploaded operators, bit for bit
    L = o.random(81 + emax, -1)
    dL = eng.new_op(-1, L)
    r1, r2 = eng.new_op(1), eng.new_op(1)
    eng.commutator(dL, op, r1)
    eng.commutator(dL, eng.new_op(1, slab), r2)
    assert np.array_equal(r1.download(), r2.download())


def test_per_array_upload_rejects_missing_arrays(built_lib, oracles):
    from imsrg_gb300 import Engine, make_basis
    eng = Engine(make_basis(2), device=0)
    slab = oracles(2).random(5, 1)
    E0, fhh, fph, fpp, gam = _fortran_arrays(eng, slab)
    pd = C.POINTER(C.c_double)
    op = eng.new_op(1)
    k = next(i for i, g in enumerate(gam) if g is not None)
    holes = list(gam)
    holes[k] = None  # a NULL pointer for a non-empty array
    st = eng.L.imsrg_op_upload(eng.h, op.h, C.cast(_ptrs(holes), C.POINTER(C.c_void_p)), fhh.ctypes.data_as(pd),
                               fph.ctypes.data_as(pd), fpp.ctypes.data_as(pd), float(E0))
    assert st == 1  # IMSRG_ERR_INVALID_ARGUMENT
    st = eng.L.imsrg_op_upload(eng.h, op.h, C.cast(_ptrs(gam), C.POINTER(C.c_void_p)), None,
                               fph.ctypes.data_as(pd), fpp.ctypes.data_as(pd), float(E0))
    assert st == 1
