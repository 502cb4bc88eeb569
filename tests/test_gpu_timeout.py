"""A bounded device wait that runs out, and the context afterwards.

The reference STOPs the process where a loop cannot finish (src/IMSRG_MAGNUS.f90:232).
Here every mbarrier wait of the tensor-core GEMM is bounded: on timeout the kernel records
a code, stops its other roles, waits for its own copies in flight, frees its tensor memory
and returns, and imsrg_synchronize reports IMSRG_ERR_TIMEOUT.  The test makes one wait run
out without any fault: the test switch leaves one pipeline stage unarmed (no copy issued,
nothing arrives on its barrier) under a 1 ms limit.  The same context must then compute a
correct commutator.
"""
import time

import pytest

from helpers import rel_err, sections

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["bf16x3", "bf16x6", "tf32x3"])
def test_bounded_wait_runs_out_and_context_recovers(built_lib, oracles, mode):
    from imsrg_gb300 import Engine, make_basis
    emax = 4
    o = oracles(emax)
    eng = Engine(make_basis(emax), device=0, precision=mode)
    L, R = o.random(301, -1), o.random(302, 1)
    ref = o.commutator(L, -1, R, 1, 1)
    dL, dR, dRES = eng.new_op(-1, L), eng.new_op(1, R), eng.new_op(1)
    eng.commutator(dL, dR, dRES)  # prepares the tensor-core path
    eng.synchronize()
    assert eng.L.imsrg_set_wait_limit(eng.h, 1_000_000) == 0  # 1 ms
    assert eng.L.imsrg_test_unarmed_stage(eng.h, 1) == 0
    t0 = time.perf_counter()
    assert eng.L.imsrg_commutator(eng.h, dL.h, dR.h, dRES.h, 1) == 0  # enqueued
    st = eng.L.imsrg_synchronize(eng.h)
    elapsed = time.perf_counter() - t0
    assert st == 7, (st, eng.L.imsrg_last_error(eng.h))  # IMSRG_ERR_TIMEOUT
    assert b"bounded wait ran out" in eng.L.imsrg_last_error(eng.h)
    assert elapsed < 5.0
    # the error word was consumed: the next synchronize is clean
    assert eng.L.imsrg_synchronize(eng.h) == 0
    # default limit again; the same context computes the right commutator
    assert eng.L.imsrg_set_wait_limit(eng.h, 0) == 0
    eng.commutator(dL, dR, dRES)
    eng.synchronize()
    got = dRES.download()
    tol = 2e-5
    e0, ob, tb = sections(o, got)
    r0, rob, rtb = sections(o, ref)
    assert abs(e0 - r0) <= tol * max(1.0, abs(r0))
    assert rel_err(ob, rob) <= tol and rel_err(tb, rtb) <= tol


def test_wait_limit_arguments(built_lib):
    from imsrg_gb300 import Engine, make_basis
    eng = Engine(make_basis(2), device=0)
    assert eng.L.imsrg_set_wait_limit(eng.h, -1) == 1
    assert eng.L.imsrg_set_wait_limit(eng.h, 0) == 0
    assert eng.L.imsrg_test_unarmed_stage(eng.h, 0) == 0
