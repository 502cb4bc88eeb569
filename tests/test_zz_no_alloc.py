"""imsrg_mat_frob_norm_noalloc: the norm entry point that allocates nothing.

It serves callers that must not call cudaMalloc when they need the norm (an allocator
that owns all device memory, a callback or pool that forbids new allocations, a host
driver that passes only its own buffers).  Checked through the C ABI against
imsrg_mat_frob_norm on two calls in a row with different operators, so stale scratch
from the first call would show up in the second.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_norm_matches_norm_twice(built_lib, oracles):
    torch = pytest.importorskip("torch")
    from imsrg_gb300 import Engine, make_basis
    emax = 4
    eng = Engine(make_basis(emax), device=0)
    o = oracles(emax)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    for seed, herm, scale in ((11, -1, 1.0), (12, 1, 3.5)):
        slab = o.random(seed, herm) * scale
        op = eng.new_op(herm, slab)
        ref = eng.mat_frob_norm(op)
        st = eng.L.imsrg_mat_frob_norm_noalloc(eng.h, C.c_void_p(op.device_ptr()), C.c_void_p(out.data_ptr()),
                                               C.c_void_p(0))
        assert st == 0, eng.L.imsrg_last_error(eng.h)
        torch.cuda.synchronize()
        got = float(out.cpu()[0])
        assert abs(got - ref) <= 1e-12 * ref, (got, ref)
        assert abs(got - o.frob(slab)) <= 1e-12 * ref


def test_noalloc_rejects_bad_arguments(built_lib):
    from imsrg_gb300 import Engine, make_basis
    eng = Engine(make_basis(2), device=0)
    st = eng.L.imsrg_mat_frob_norm_noalloc(eng.h, C.c_void_p(0), C.c_void_p(0), C.c_void_p(0))
    assert st == 1  # IMSRG_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("side_stream", [False, True])
def test_noalloc_norm_waits_for_queued_context_work(built_lib, oracles, side_stream):
    """The norm is ordered after work still queued on the context's own stream (a
    commutator writing the operator, no host synchronisation in between), on the legacy
    default stream and on a torch side stream; the context's next call waits for it."""
    torch = pytest.importorskip("torch")
    from imsrg_gb300 import Engine, make_basis
    emax = 4
    eng = Engine(make_basis(emax), device=0)
    o = oracles(emax)
    L, R = o.random(21, -1), o.random(22, 1)
    ref = o.frob(o.commutator(L, -1, R, 1, 1))
    dL, dR, dRES = eng.new_op(-1, L), eng.new_op(1, R), eng.new_op(1)
    res_ptr = dRES.device_ptr()
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    side = torch.cuda.Stream() if side_stream else None
    strm = C.c_void_p(side.cuda_stream if side_stream else 0)
    eng.synchronize()
    torch.cuda.synchronize()
    for k in range(3):
        eng.clear_sq_op(dRES)
        eng.commutator(dL, dR, dRES)  # queued on the context's stream
        st = eng.L.imsrg_mat_frob_norm_noalloc(eng.h, C.c_void_p(res_ptr), C.c_void_p(out.data_ptr() + 8 * k), strm)
        assert st == 0, eng.L.imsrg_last_error(eng.h)
    # the context's next call (clearing the operator) must not run before the last norm read it
    eng.clear_sq_op(dRES)
    if side_stream:
        side.synchronize()
    torch.cuda.synchronize()
    eng.synchronize()
    got = out.cpu().numpy()
    assert np.all(np.abs(got - ref) <= 1e-10 * ref), (got, ref)
    assert float(np.max(np.abs(dRES.download()))) == 0.0
