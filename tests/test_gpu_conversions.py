"""FP64 <-> FP32 conversions of the mixed-precision kernels, and NaN through the mixed path.

The mixed kernels convert with integer instructions (the hardware conversion runs on
GB300's slow FP64 pipe).  Those conversions must round to nearest even and carry NaN, Inf,
overflow and FP32 subnormals exactly as IEEE 754 binary64 <-> binary32 conversion does:
checked bit for bit against the GPU's own conversion instructions and against numpy on
random, boundary, tie and special values.  A NaN in the Hamiltonian must then surface as a
NaN (or an error status) of a mixed commutator and a mixed Magnus step, not as a finite
number.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(seed):
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 2**63, size=200000, dtype=np.uint64) | (
        rng.integers(0, 2, size=200000, dtype=np.uint64) << np.uint64(63))
    x = [bits.view(np.float64)]
    # exponents around FP32's normal, subnormal and overflow limits, many of them exact ties
    e = rng.integers(860, 1160, size=200000).astype(np.uint64)
    m = rng.integers(0, 2**52, size=200000, dtype=np.uint64)
    m[::2] &= ~np.uint64((1 << 28) - 1)
    x.append(((e << np.uint64(52)) | m).view(np.float64))
    x.append(np.array([0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan, 3.4028234663852886e38,
                       3.4028235677973362e38, 3.4028235677973366e38, 1e39, -1e39, 1.1754943508222875e-38,
                       1.401298464324817e-45, 7.006492321624085e-46, 7.006492321624087e-46,
                       2.1019476964872256e-45, 1e-46, 5e-324, -5e-324, 1.0, -1.0, 0.1, -2.5e-40]))
    x = np.concatenate(x)
    ybits = rng.integers(0, 2**32, size=x.size, dtype=np.uint64).astype(np.uint32)
    ybits[:2**16] = np.arange(2**16, dtype=np.uint32) * 97  # many FP32 subnormals
    return x, ybits.view(np.float32)


def _same_f32(a, b):
    nan = np.isnan(a) & np.isnan(b)
    return nan | (a.view(np.uint32) == b.view(np.uint32))


def _same_f64(a, b):
    nan = np.isnan(a) & np.isnan(b)
    return nan | (a.view(np.uint64) == b.view(np.uint64))


def test_integer_conversions_match_ieee(built_lib):
    from imsrg_gb300 import Engine, make_basis
    eng = Engine(make_basis(2), device=0)
    x, y = _inputs(5)
    n = x.size
    of = np.empty(2 * n, dtype=np.float32)
    od = np.empty(2 * n, dtype=np.float64)
    st = eng.L.imsrg_check_conversions(eng.h, x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p), n,
                                       of.ctypes.data_as(C.c_void_p), od.ctypes.data_as(C.c_void_p))
    assert st == 0, eng.L.imsrg_last_error(eng.h)
    with np.errstate(over="ignore"):
        ref32 = x.astype(np.float32)  # IEEE round to nearest even on the host
    ref64 = y.astype(np.float64)
    assert _same_f32(of[:n], of[n:]).all(), "f64_to_f32 differs from __double2float_rn"
    assert _same_f32(of[:n], ref32).all(), "f64_to_f32 differs from IEEE conversion"
    assert _same_f64(od[:n], od[n:]).all(), "f32_to_f64 differs from the hardware conversion"
    assert _same_f64(od[:n], ref64).all(), "f32_to_f64 differs from IEEE conversion"
    # unbiased: the rounding error of the integer conversion averages to ~0 (truncation
    # toward zero would make every error shrink |x|)
    xs = np.random.default_rng(9).normal(size=100000)
    st = eng.L.imsrg_check_conversions(eng.h, xs.ctypes.data_as(C.c_void_p), y[:xs.size].ctypes.data_as(C.c_void_p),
                                       xs.size, of[:2 * xs.size].ctypes.data_as(C.c_void_p),
                                       od[:2 * xs.size].ctypes.data_as(C.c_void_p))
    assert st == 0
    err = (of[:xs.size].astype(np.float64) - xs) / np.abs(xs)
    assert abs(err.mean()) < 5e-10
    assert np.all(np.abs(err) <= 2.0**-24 * (1 + 1e-12))


@pytest.mark.parametrize("mode", ["bf16x3", "bf16x6", "tf32x3"])
def test_nan_in_hamiltonian_reaches_the_mixed_result(built_lib, mode):
    from imsrg_gb300 import Engine, make_basis
    eng = Engine(make_basis(4), device=0, precision=mode)
    H = eng.synthetic_hamiltonian(seed=3)
    A, N = eng.basis.nholes, eng.basis.norbits
    n1 = 1 + A * A + (N - A) ** 2 + (N - A) * A  # E0 and the one-body arrays
    Hn = H.copy()
    nz = n1 + np.flatnonzero(Hn[n1:])[len(np.flatnonzero(Hn[n1:])) // 2]
    Hn[nz] = np.nan
    dH = eng.new_op(1, Hn)
    dE = eng.new_op(-1)
    eng.build_gs_white(eng.new_op(1, H), dE)  # a finite generator: the NaN enters through H only
    dRES = eng.new_op(1)
    eng.commutator(dE, dH, dRES)
    eng.synchronize()
    assert np.isnan(dRES.download()).any(), "a NaN in H vanished in the mixed commutator"
    # a Magnus step from the NaN Hamiltonian: NaN energy or a non-convergence status
    HS, G, DG = eng.new_op(1, Hn), eng.new_op(-1), eng.new_op(-1)
    eng.build_gs_white(HS, DG)
    info = eng.magnus_step(HS, G, DG, dH, 0.5, 11, 1e-8, graph=False, allow_unconverged=True)
    assert np.isnan(info["E0"]) or not info["bch_converged"]
    assert np.isnan(HS.download()).any()
