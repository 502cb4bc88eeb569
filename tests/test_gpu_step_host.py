"""The Magnus step with the flow state in host memory (imsrg_magnus_step_host).

A Fortran driver of magnus_decouple (src/IMSRG_MAGNUS.f90:47-110) keeps H, Omega and eta in
its own arrays between steps.  imsrg_magnus_step_host uploads the step's inputs, runs the step
and downloads its outputs, with some of the copies overlapping the step inside the captured
graph.  Its results must equal, bit for bit, the plain sequence upload -> imsrg_magnus_step ->
download on the same host data, eager and captured.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DS = 0.5


def _pinned(eng, n):
    p = C.c_void_p()
    eng._ck(eng.L.imsrg_pinned_alloc(8 * n, C.byref(p)))
    return p, np.ctypeslib.as_array((C.c_double * n).from_address(p.value))


@pytest.mark.parametrize("precision,graph", [("bf16x3", True), ("bf16x3", False), ("fp64", True)])
def test_host_step_equals_upload_step_download(built_lib, precision, graph):
    from imsrg_gb300 import Engine, make_basis
    eng = Engine(make_basis(4), device=0, precision=precision)
    n = eng.slab
    H = eng.synthetic_hamiltonian(seed=5)
    HS0, G0, DG0 = eng.new_op(1, H), eng.new_op(-1), eng.new_op(-1)
    eng.build_gs_white(HS0, DG0)
    ptrs, bufs = [], []
    for _ in range(2):  # two copies of the host flow state: H, Omega, eta, H(s)
        p4, a4 = zip(*[_pinned(eng, n) for _ in range(4)])
        a4[0][:] = H
        a4[1][:] = G0.download()
        a4[2][:] = DG0.download()
        ptrs.append(p4)
        bufs.append(a4)
    # A: the plain sequence on device operators
    dA = [eng.new_op(1), eng.new_op(-1), eng.new_op(-1), eng.new_op(1)]  # HS, G, DG, H
    # B: the host step on its own workspaces
    dB = [eng.new_op(1), eng.new_op(-1), eng.new_op(-1), eng.new_op(1)]
    pa, pb = ptrs
    for step in range(3):
        for op, p in ((dA[3], pa[0]), (dA[1], pa[1]), (dA[2], pa[2])):
            eng._ck(eng.L.imsrg_op_upload_slab(eng.h, op.h, p))
        ia = eng.magnus_step(dA[0], dA[1], dA[2], dA[3], DS, 11, 1e-8, graph=graph, allow_unconverged=True)
        for op, p in ((dA[0], pa[3]), (dA[1], pa[1]), (dA[2], pa[2])):
            eng._ck(eng.L.imsrg_op_download_slab(eng.h, op.h, p))
        ib = eng.magnus_step_host(dB[0], dB[1], dB[2], dB[3], pb[3], pb[1], pb[2], pb[0], DS, 11, 1e-8, graph=graph,
                                  allow_unconverged=True)
        for k in ("E0", "mbpt2", "magnus_terms", "bch_terms", "bch_converged"):
            assert ia[k] == ib[k], (step, k, ia, ib)
        for x, y in zip(bufs[0][1:], bufs[1][1:]):  # Omega, eta, H(s)
            assert np.array_equal(x, y), step
    assert ib["magnus_terms"] > 0 and ib["bch_terms"] > 1
    for p in pa + pb:
        eng.L.imsrg_pinned_free(p)


def test_host_step_arguments(built_lib):
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300 import _lib
    eng = Engine(make_basis(2), device=0, precision="bf16x3")
    ops = [eng.new_op(1), eng.new_op(-1), eng.new_op(-1), eng.new_op(1)]
    p, _ = _pinned(eng, eng.slab)
    info = _lib.StepInfo_t()
    # a null host buffer, or one output buffer given twice, is rejected before any work
    assert eng.L.imsrg_magnus_step_host(eng.h, *[o.h for o in ops], None, p, p, p, DS, 11, 1e-8, 1, C.byref(info)) == 1
    assert eng.L.imsrg_magnus_step_host(eng.h, *[o.h for o in ops], p, p, p, p, DS, 11, 1e-8, 1, C.byref(info)) == 1
    eng.L.imsrg_pinned_free(p)
