"""Python mirror of the reference's commutator interface, on the GB300 engine.

Names, argument order and assign / accumulate semantics follow the Fortran routines
(src/commutators.f90, src/cross_coupled.f90, src/generators.f90, src/IMSRG_MAGNUS.f90);
every call goes through the C ABI of libimsrg_gb300.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .basis import Basis

# reference default-real literal for the BCH / Magnus convergence tests
CONV = float(np.float32(1e-6))


class SqOp:
    """A device-resident type(sq_op) (handle owned by an Engine)."""

    def __init__(self, eng: "Engine", herm: int = 1):
        self.eng = eng
        h = C.c_void_p()
        eng._ck(eng.L.imsrg_op_create(eng.h, int(herm), C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.eng.L.imsrg_op_destroy(self.eng.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def herm(self) -> int:
        v = C.c_int32()
        self.eng._ck(self.eng.L.imsrg_op_get_herm(self.eng.h, self.h, C.byref(v)))
        return v.value

    @herm.setter
    def herm(self, v: int):
        self.eng._ck(self.eng.L.imsrg_op_set_herm(self.eng.h, self.h, int(v)))

    def upload(self, slab: np.ndarray):
        slab = np.ascontiguousarray(slab, dtype=np.float64)
        if slab.size != self.eng.slab:
            raise ValueError(f"slab has {slab.size} elements, layout needs {self.eng.slab}")
        self.eng._ck(self.eng.L.imsrg_op_upload_slab(self.eng.h, self.h, slab.ctypes.data))
        self.eng.synchronize()
        return self

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.eng.slab, np.float64)
        self.eng._ck(self.eng.L.imsrg_op_download_slab(self.eng.h, self.h, out.ctypes.data))
        return out

    def device_ptr(self) -> int:
        p = C.c_void_p()
        self.eng._ck(self.eng.L.imsrg_op_device_slab(self.eng.h, self.h, C.byref(p)))
        return p.value

    @property
    def E0(self) -> float:
        v = C.c_double()
        self.eng._ck(self.eng.L.imsrg_op_get_e0(self.eng.h, self.h, C.byref(v)))
        return v.value


class TensorOp:
    """A rank-lambda tensor operator on the device (imsrg_tensor); rank2 / dpar2 doubled."""

    def __init__(self, eng: "Engine", rank2: int, dpar2: int = 0, herm: int = 1):
        self.eng, self.rank2, self.dpar2 = eng, int(rank2), int(dpar2)
        self.slab = eng.tensor_sizes(rank2, dpar2)[0]
        h = C.c_void_p()
        eng._ck(eng.L.imsrg_tensor_create(eng.h, self.rank2, self.dpar2, int(herm), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.eng.L.imsrg_tensor_destroy(self.eng.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, slab: np.ndarray):
        slab = np.ascontiguousarray(slab, dtype=np.float64)
        if slab.size != self.slab:
            raise ValueError(f"tensor slab has {self.slab} elements, got {slab.size}")
        self.eng._ck(self.eng.L.imsrg_tensor_upload_slab(self.eng.h, self.h, slab.ctypes.data))

    def download(self) -> np.ndarray:
        out = np.empty(self.slab)
        self.eng._ck(self.eng.L.imsrg_tensor_download_slab(self.eng.h, self.h, out.ctypes.data))
        return out

    def frob(self) -> float:
        v = C.c_double()
        self.eng._ck(self.eng.L.imsrg_tensor_frob_norm(self.eng.h, self.h, C.byref(v)))
        return v.value


class CCMat:
    """A device-resident type(cc_mat): kind 0 = CCX storage, kind 1 = WCC workspace."""

    def __init__(self, eng: "Engine", kind: int = 0):
        self.eng = eng
        self.kind = kind
        h = C.c_void_p()
        eng._ck(eng.L.imsrg_cc_create(eng.h, int(kind), C.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.eng.L.imsrg_cc_destroy(self.eng.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def download(self) -> np.ndarray:
        n = self.eng.wcc_size if self.kind else self.eng.cc_size
        out = np.empty(n, np.float64)
        if n:
            self.eng._ck(self.eng.L.imsrg_cc_download(self.eng.h, self.h, out.ctypes.data))
        return out


class Engine:
    """One basis (jbas + channel layout + 6j table) on one GPU."""

    def __init__(self, basis: Basis, device: int = 0, precision: str = "fp64"):
        self.L = _lib.load()
        self.basis = basis
        arrs = basis.arrays()
        self._keep = arrs
        P = C.POINTER(C.c_int32)
        b = _lib.Basis_t(basis.norbits, *[a.ctypes.data_as(P) for a in arrs], basis.eMax, basis.lMax,
                         float(basis.hw), basis.Aprot, basis.Aneut)
        h = C.c_void_p()
        st = self.L.imsrg_ctx_create(C.byref(b), int(device), C.byref(h))
        if st != 0:
            raise _lib.ImsrgError(st, "imsrg_ctx_create failed")
        self.h = h
        slab, cc, wcc = C.c_int64(), C.c_int64(), C.c_int64()
        nb, ncc = C.c_int32(), C.c_int32()
        self._ck(self.L.imsrg_ctx_sizes(self.h, C.byref(slab), C.byref(cc), C.byref(wcc), C.byref(nb), C.byref(ncc)))
        self.slab, self.cc_size, self.wcc_size = slab.value, cc.value, wcc.value
        self.nblocks, self.ncc = nb.value, ncc.value
        self.precision = "fp64"
        if precision != "fp64":
            self.set_precision(precision)

    def _ck(self, st: int):
        if st != 0:
            msg = self.L.imsrg_last_error(self.h)
            raise _lib.ImsrgError(st, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.L.imsrg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------------- layout
    def block_info(self):
        arrs = [np.zeros(self.nblocks, np.int32) for _ in range(6)]
        P = C.POINTER(C.c_int32)
        self._ck(self.L.imsrg_block_info(self.h, *[a.ctypes.data_as(P) for a in arrs]))
        return dict(zip(("lamJ", "lamP", "lamT", "npp", "nph", "nhh"), arrs))

    def block_pairs(self, q: int, cls: int) -> np.ndarray:
        info = self.block_info()
        n = int((info["npp"], info["nph"], info["nhh"])[cls][q])
        out = np.zeros(2 * max(n, 1), np.int32)
        self._ck(self.L.imsrg_block_pairs(self.h, q, cls, out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out[: 2 * n].reshape(n, 2)

    def cc_info(self):
        arrs = [np.zeros(self.ncc, np.int32) for _ in range(3)]
        P = C.POINTER(C.c_int32)
        self._ck(self.L.imsrg_cc_info(self.h, *[a.ctypes.data_as(P) for a in arrs]))
        return dict(zip(("rlen", "nph", "J"), arrs))

    def set_precision(self, mode: str):
        self._ck(self.L.imsrg_set_precision(self.h, _lib.PREC[mode]))
        self.precision = mode

    def autotune(self, L: SqOp, R: SqOp, RES: SqOp) -> dict:
        """Pick the launch configuration of the mixed commutator on this basis (imsrg_autotune);
        RES is overwritten with [L, R]."""
        info = _lib.TuneInfo_t()
        self._ck(self.L.imsrg_autotune(self.h, L.h, R.h, RES.h, C.byref(info)))
        return {k: getattr(info, k) for k, _ in _lib.TuneInfo_t._fields_}

    def set_tuning(self, cfg: dict):
        """Apply a launch configuration (a dict as autotune() returns; imsrg_set_tuning)."""
        info = _lib.TuneInfo_t()
        for k, _ in _lib.TuneInfo_t._fields_:
            if k in cfg:
                setattr(info, k, cfg[k])
        self._ck(self.L.imsrg_set_tuning(self.h, C.byref(info)))

    def synchronize(self):
        self._ck(self.L.imsrg_synchronize(self.h))

    # ---------------------------------------------------------------- instrumentation
    def launch_count(self) -> int:
        v = C.c_int64()
        self._ck(self.L.imsrg_launch_count(self.h, C.byref(v)))
        return v.value

    def timer_begin(self):
        self._ck(self.L.imsrg_timer_begin(self.h))

    def timer_end(self) -> float:
        """Elapsed ms on the context's stream since timer_begin (synchronizes)."""
        v = C.c_float()
        self._ck(self.L.imsrg_timer_end(self.h, C.byref(v)))
        return v.value

    def profile_phases(self, enable: bool):
        self._ck(self.L.imsrg_profile_phases(self.h, 1 if enable else 0))

    def profile_read(self) -> dict:
        n = len(_lib.PHASES)
        ms = (C.c_float * n)()
        cnt = (C.c_int32 * n)()
        self._ck(self.L.imsrg_profile_read(self.h, ms, cnt))
        return {name: (ms[i], cnt[i]) for i, name in enumerate(_lib.PHASES) if i > 0}

    # ---------------------------------------------------------------- objects
    def new_op(self, herm: int = 1, slab: np.ndarray | None = None) -> SqOp:
        op = SqOp(self, herm)
        if slab is not None:
            op.upload(slab)
        return op

    def new_cc(self, kind: int = 0) -> CCMat:
        return CCMat(self, kind)

    def synthetic_hamiltonian(self, seed: int = 1, v_scale: float = 1.0) -> np.ndarray:
        out = np.zeros(self.slab, np.float64)
        self._ck(self.L.imsrg_synthetic_hamiltonian(self.h, C.c_uint64(seed), float(v_scale), out.ctypes.data))
        return out

    def synthetic_bare_hamiltonian(self, seed: int = 1, v_scale: float = 1.0) -> np.ndarray:
        """The synthetic Hamiltonian before normal ordering (kinetic energy in f, E0 = 0)."""
        out = np.zeros(self.slab, np.float64)
        self._ck(self.L.imsrg_synthetic_bare_hamiltonian(self.h, C.c_uint64(seed), float(v_scale),
                                                          out.ctypes.data))
        return out

    # ---------------------------------------------------------------- flat vectors, checkpoints
    @property
    def neq(self) -> int:
        v = C.c_int64()
        self._ck(self.L.imsrg_neq(self.h, C.byref(v)))
        return v.value

    def vectorize(self, slab: np.ndarray) -> np.ndarray:
        """vectorize (src/basic_IMSRG.f90:3929-3985) of a host slab."""
        slab = np.ascontiguousarray(slab, dtype=np.float64)
        out = np.empty(self.neq)
        self._ck(self.L.imsrg_vectorize_slab(self.h, slab.ctypes.data, out.ctypes.data))
        return out

    def repackage(self, vec: np.ndarray, herm: int = 1) -> np.ndarray:
        """repackage (src/basic_IMSRG.f90:3988-4053) into a host slab."""
        vec = np.ascontiguousarray(vec, dtype=np.float64)
        if vec.size != self.neq:
            raise ValueError(f"vector has {vec.size} values, this basis needs {self.neq}")
        out = np.zeros(self.slab)
        self._ck(self.L.imsrg_repackage_slab(self.h, vec.ctypes.data, int(herm), out.ctypes.data))
        return out

    def write_omega_checkpoint(self, G: SqOp, path: str):
        self._ck(self.L.imsrg_write_omega_checkpoint(self.h, G.h, str(path).encode()))

    def read_omega_checkpoint(self, G: SqOp, path: str):
        self._ck(self.L.imsrg_read_omega_checkpoint(self.h, G.h, str(path).encode()))

    # ---------------------------------------------------------------- me2j interaction records
    def synthetic_me2j_values(self, seed: int = 1, v_scale: float = 1.0) -> np.ndarray:
        """The synthetic interaction as me2j record values (4 per record, file order)."""
        n = C.c_int64()
        self._ck(self.L.imsrg_synthetic_me2j_values(self.h, C.c_uint64(seed), float(v_scale), None, C.byref(n)))
        out = np.zeros(n.value)
        self._ck(self.L.imsrg_synthetic_me2j_values(self.h, C.c_uint64(seed), float(v_scale), out.ctypes.data,
                                                    C.byref(n)))
        return out

    def me2j_to_slab(self, values: np.ndarray, emax_file: int, htype: int = 1,
                     slab: np.ndarray | None = None) -> np.ndarray:
        """read_me2j_interaction (src/interaction_IO.f90:282-557) of record values into the
        two-body arrays of a host slab (a new zero slab by default); htype 1 adds the
        two-body centre-of-mass term -p1.p2 hw/A."""
        values = np.ascontiguousarray(values, dtype=np.float64)
        out = np.zeros(self.slab) if slab is None else slab
        self._ck(self.L.imsrg_me2j_to_slab(self.h, values.ctypes.data, int(values.size), int(emax_file),
                                           int(htype), out.ctypes.data))
        return out

    # ---------------------------------------------------------------- Hartree-Fock
    def calc_hf(self, H: SqOp, max_iter: int = 1000):
        """calc_HF (src/HF_mod.f90:14-105): H (bare) becomes the normal-ordered HF-basis
        Hamiltonian.  Returns (D, info) with D(HO orbit, HF orbit) as an N x N array."""
        N = self.basis.norbits
        D = np.zeros(N * N)
        info = _lib.HFInfo_t()
        self._ck(self.L.imsrg_calc_hf(self.h, H.h, int(max_iter), D.ctypes.data, C.byref(info)))
        return D.reshape(N, N, order="F"), {"e_hf": info.e_hf, "crit": info.crit, "iterations": info.iterations}

    def calc_ho(self, H: SqOp):
        """calc_HO (src/HF_mod.f90:107-179): normal ordering w.r.t. the HO reference."""
        N = self.basis.norbits
        D = np.zeros(N * N)
        info = _lib.HFInfo_t()
        self._ck(self.L.imsrg_calc_ho(self.h, H.h, D.ctypes.data, C.byref(info)))
        return D.reshape(N, N, order="F"), {"e_hf": info.e_hf, "crit": info.crit, "iterations": info.iterations}

    def sqop_to_hf(self, op: SqOp, D: np.ndarray):
        """sqop_to_HF (src/HF_mod.f90:181-209) of a bare scalar operator, in place."""
        Df = np.ascontiguousarray(np.asarray(D, np.float64).ravel(order="F"))
        self._ck(self.L.imsrg_sqop_to_hf(self.h, op.h, Df.ctypes.data))

    def transform_2b_to_hf(self, op: SqOp, D: np.ndarray):
        """transform_2b_to_HF (src/HF_mod.f90:567-692), in place."""
        Df = np.ascontiguousarray(np.asarray(D, np.float64).ravel(order="F"))
        self._ck(self.L.imsrg_transform_2b_to_hf(self.h, op.h, Df.ctypes.data))

    def normal_order(self, op: SqOp):
        """normal_order (src/basic_IMSRG.f90:2419-2550), in place."""
        self._ck(self.L.imsrg_normal_order(self.h, op.h))

    # ---------------------------------------------------------------- algebra
    def copy_sq_op(self, H: SqOp, op: SqOp):
        self._ck(self.L.imsrg_copy_sq_op(self.h, H.h, op.h))

    def clear_sq_op(self, op: SqOp):
        self._ck(self.L.imsrg_clear_sq_op(self.h, op.h))

    def add_sq_op(self, A: SqOp, ax: float, B: SqOp, bx: float, Cop: SqOp):
        self._ck(self.L.imsrg_add_sq_op(self.h, A.h, float(ax), B.h, float(bx), Cop.h))

    def scale_sq_op(self, A: SqOp, ax: float):
        self._ck(self.L.imsrg_scale_sq_op(self.h, A.h, float(ax)))

    def mat_frob_norm(self, op: SqOp) -> float:
        v = C.c_double()
        self._ck(self.L.imsrg_mat_frob_norm(self.h, op.h, C.byref(v)))
        return v.value

    def mbpt2(self, H: SqOp) -> float:
        v = C.c_double()
        self._ck(self.L.imsrg_mbpt2(self.h, H.h, C.byref(v)))
        return v.value

    # ---------------------------------------------------------------- commutator pieces
    def calculate_cross_coupled(self, HS: SqOp, CCME: CCMat):
        self._ck(self.L.imsrg_calculate_cross_coupled(self.h, HS.h, CCME.h))

    def commutator_110(self, L: SqOp, R: SqOp) -> float:
        v = C.c_double()
        self._ck(self.L.imsrg_commutator_110(self.h, L.h, R.h, C.byref(v)))
        return v.value

    def commutator_220(self, L: SqOp, R: SqOp) -> float:
        v = C.c_double()
        self._ck(self.L.imsrg_commutator_220(self.h, L.h, R.h, C.byref(v)))
        return v.value

    def commutator_111(self, L: SqOp, R: SqOp, RES: SqOp):
        self._ck(self.L.imsrg_commutator_111(self.h, L.h, R.h, RES.h))

    def commutator_121(self, L: SqOp, R: SqOp, RES: SqOp):
        self._ck(self.L.imsrg_commutator_121(self.h, L.h, R.h, RES.h))

    def commutator_122(self, L: SqOp, R: SqOp, RES: SqOp):
        self._ck(self.L.imsrg_commutator_122(self.h, L.h, R.h, RES.h))

    def commutator_222_pp_hh(self, L: SqOp, R: SqOp, RES: SqOp, w1: SqOp, w2: SqOp):
        self._ck(self.L.imsrg_commutator_222_pp_hh(self.h, L.h, R.h, RES.h, w1.h, w2.h))

    def commutator_221(self, L: SqOp, R: SqOp, RES: SqOp, w1: SqOp, w2: SqOp):
        self._ck(self.L.imsrg_commutator_221(self.h, L.h, R.h, RES.h, w1.h, w2.h))

    def commutator_222_ph(self, LCC: CCMat, RCC: CCMat, RES: SqOp, WCC: CCMat):
        self._ck(self.L.imsrg_commutator_222_ph(self.h, LCC.h, RCC.h, RES.h, WCC.h))

    def commutator(self, L: SqOp, R: SqOp, RES: SqOp, e0: bool = True):
        self._ck(self.L.imsrg_commutator(self.h, L.h, R.h, RES.h, _lib.COMM_E0 if e0 else 0))

    # ---------------------------------------------------------------- generator / flow
    def build_gs_white(self, H: SqOp, ETA: SqOp):
        self._ck(self.L.imsrg_build_gs_white(self.h, H.h, ETA.h))

    def build_gs_atan(self, H: SqOp, ETA: SqOp):
        self._ck(self.L.imsrg_build_gs_atan(self.h, H.h, ETA.h))

    def build_gs_atanxx(self, Hold: SqOp, H: SqOp, ETA: SqOp):
        self._ck(self.L.imsrg_build_gs_atanxx(self.h, Hold.h, H.h, ETA.h))

    def build_gs_w2(self, H: SqOp, ETA: SqOp):
        self._ck(self.L.imsrg_build_gs_w2(self.h, H.h, ETA.h))

    def magnus_expand(self, DG: SqOp, G: SqOp) -> int:
        n = C.c_int32()
        self._ck(self.L.imsrg_magnus_expand(self.h, DG.h, G.h, C.byref(n)))
        return n.value

    def euler_step(self, G: SqOp, DG: SqOp, s: float, stp: float) -> float:
        sv = C.c_double(s)
        self._ck(self.L.imsrg_euler_step(self.h, G.h, DG.h, C.byref(sv), float(stp)))
        return sv.value

    def bch_expand(self, HS: SqOp, G: SqOp, H: SqOp, max_terms: int = 40, conv: float = CONV) -> int:
        n = C.c_int32()
        self._ck(self.L.imsrg_bch_expand(self.h, HS.h, G.h, H.h, int(max_terms), float(conv), C.byref(n)))
        return n.value

    def bch_expand_quads(self, HS: SqOp, G: SqOp, H: SqOp, max_terms: int = 40, conv: float = CONV) -> int:
        """BCH_EXPAND with quads = 'y' (src/IMSRG_MAGNUS.f90:149-234, 908-1132)."""
        n = C.c_int32()
        self._ck(self.L.imsrg_bch_expand_quads(self.h, HS.h, G.h, H.h, int(max_terms), float(conv), C.byref(n)))
        return n.value

    def restore_quadrupoles(self, X: SqOp, OM: SqOp, RES: SqOp):
        """restore_quadrupoles (src/IMSRG_MAGNUS.f90:908-1070): RES = its pp-hh arrays."""
        self._ck(self.L.imsrg_restore_quadrupoles(self.h, X.h, OM.h, RES.h))

    def restore_triples(self, H: SqOp, OM: SqOp):
        """restore_triples (src/IMSRG_MAGNUS.f90:767-902): the triples correction and the number of
        (ppp, hhh) pairs summed."""
        e3, n = C.c_double(), C.c_int64()
        self._ck(self.L.imsrg_restore_triples(self.h, H.h, OM.h, C.byref(e3), C.byref(n)))
        return e3.value, n.value

    def cr_expand(self, HS: SqOp, G: SqOp, H: SqOp, max_terms: int = 14, conv: float = CONV) -> int:
        """CR_EXPAND (src/IMSRG_MAGNUS.f90:532-617): HS = sum_n ad_G^n(H) / (n+1)!."""
        n = C.c_int32()
        self._ck(self.L.imsrg_cr_expand(self.h, HS.h, G.h, H.h, int(max_terms), float(conv), C.byref(n)))
        return n.value

    def magnus_step(self, HS: SqOp, G: SqOp, DG: SqOp, H: SqOp, ds: float, max_terms: int = 40, conv: float = CONV,
                    graph: bool = True, wait: bool = True, allow_unconverged: bool = False):
        """One step of magnus_decouple (MAGNUS_EXPAND, euler_step, BCH_EXPAND, White, MBPT2).

        graph=True replays a CUDA graph of the step; wait=False only enqueues it (graph
        mode) and returns None.  Returns a dict with E0, mbpt2 and the term counts."""
        if not wait:
            if not graph:
                raise ValueError("the eager step always waits")
            self._ck(self.L.imsrg_magnus_step(self.h, HS.h, G.h, DG.h, H.h, float(ds), int(max_terms), float(conv),
                                              1, None))
            return None
        info = _lib.StepInfo_t()
        st = self.L.imsrg_magnus_step(self.h, HS.h, G.h, DG.h, H.h, float(ds), int(max_terms), float(conv),
                                      1 if graph else 0, C.byref(info))
        if st != 0 and not (allow_unconverged and st == 4):
            self._ck(st)
        return {"E0": info.E0, "mbpt2": info.mbpt2, "magnus_terms": info.magnus_terms, "bch_terms": info.bch_terms,
                "bch_converged": bool(info.bch_converged), "graph_rebuilt": bool(info.graph_rebuilt)}

    def magnus_step_host(self, HS: SqOp, G: SqOp, DG: SqOp, H: SqOp, hs_host, g_host, dg_host, h_host, ds: float,
                         max_terms: int = 40, conv: float = CONV, graph: bool = True, allow_unconverged: bool = False):
        """One step of magnus_decouple with the flow state in pinned host slabs (pointers from
        imsrg_pinned_alloc): uploads Omega (g_host), eta (dg_host) and H (h_host), runs the step
        and downloads H(s), Omega and eta.  HS, G, DG and H are the device workspaces."""
        info = _lib.StepInfo_t()
        st = self.L.imsrg_magnus_step_host(self.h, HS.h, G.h, DG.h, H.h, hs_host, g_host, dg_host, h_host, float(ds),
                                           int(max_terms), float(conv), 1 if graph else 0, C.byref(info))
        if st != 0 and not (allow_unconverged and st == 4):
            self._ck(st)
        return {"E0": info.E0, "mbpt2": info.mbpt2, "magnus_terms": info.magnus_terms, "bch_terms": info.bch_terms,
                "bch_converged": bool(info.bch_converged), "graph_rebuilt": bool(info.graph_rebuilt)}

    # ---------------------------------------------------------------- reverse mode (FP64)
    def commutator_vjp(self, L: SqOp, R: SqOp, RESb: SqOp, Lb: SqOp, Rb: SqOp, e0: bool = True):
        """Lb += d<RESb,[L,R]>/dL, Rb += d<RESb,[L,R]>/dR (RESb.herm = herm of [L,R])."""
        self._ck(self.L.imsrg_commutator_vjp(self.h, L.h, R.h, RESb.h, Lb.h, Rb.h, _lib.COMM_E0 if e0 else 0))

    def white_vjp(self, H: SqOp, ETAb: SqOp, Hb: SqOp):
        """Hb += d<ETAb, eta(H)>/dH for the White generator."""
        self._ck(self.L.imsrg_white_vjp(self.h, H.h, ETAb.h, Hb.h))

    def dot(self, A: SqOp, B: SqOp) -> float:
        v = C.c_double()
        self._ck(self.L.imsrg_dot_sq_op(self.h, A.h, B.h, C.byref(v)))
        return v.value

    # ---------------------------------------------------------------- tensor operators
    def tensor_sizes(self, rank2: int, dpar2: int = 0):
        slab, nb = C.c_int64(), C.c_int32()
        self._ck(self.L.imsrg_tensor_sizes(self.h, int(rank2), int(dpar2), C.byref(slab), C.byref(nb)))
        return slab.value, nb.value

    def tensor_block_info(self, rank2: int, dpar2: int = 0) -> dict:
        nb = self.tensor_sizes(rank2, dpar2)[1]
        arrs = [np.zeros(nb, np.int32) for _ in range(4)]
        P = C.POINTER(C.c_int32)
        self._ck(self.L.imsrg_tensor_block_info(self.h, int(rank2), int(dpar2), *[a.ctypes.data_as(P) for a in arrs]))
        return dict(zip(("J1", "J2", "Tz", "P1"), arrs))

    def new_tensor(self, rank2: int, dpar2: int = 0, herm: int = 1, slab: np.ndarray | None = None) -> "TensorOp":
        t = TensorOp(self, rank2, dpar2, herm)
        if slab is not None:
            t.upload(slab)
        return t

    def tensor_commutator(self, L: SqOp, R: "TensorOp", RES: "TensorOp", pieces: int = 127):
        self._ck(self.L.imsrg_tensor_commutator(self.h, L.h, R.h, RES.h, int(pieces)))

    def bch_tensor(self, G: SqOp, HS: "TensorOp", max_terms: int = 30, conv: float = CONV) -> int:
        n = C.c_int32()
        self._ck(self.L.imsrg_bch_tensor(self.h, G.h, HS.h, int(max_terms), float(conv), C.byref(n)))
        return n.value

    def magnus_step_counters(self) -> dict:
        v = [C.c_int64() for _ in range(4)]
        self._ck(self.L.imsrg_magnus_step_counters(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("commutators", "kernels", "steps", "unconverged"), (x.value for x in v)))
