"""ctypes binding of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the checker
and by bench.py's cpu_baseline leg.  The product never imports this module.

Operators are numpy float64 "slabs" in the sq_op flattening described at the top of
oracle.cpp, paired with their hermiticity flag.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_bp = np.ctypeslib.ndpointer(dtype=np.int8, flags="C_CONTIGUOUS")
_lib = None


def build(force: bool = False) -> str:
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = C.CDLL(LIB_PATH)
    vp, i, d, i64, u64 = C.c_void_p, C.c_int, C.c_double, C.c_int64, C.c_uint64
    sig = {
        "orc_basis_create": (vp, [i, _ip, _ip, _ip, _ip, _ip, i, d, i, i]),
        "orc_basis_destroy": (None, [vp]),
        "orc_slab_size": (i64, [vp]),
        "orc_nblocks": (i, [vp]),
        "orc_ncc": (i, [vp]),
        "orc_cc_size": (i64, [vp]),
        "orc_wcc_size": (i64, [vp]),
        "orc_block_info": (None, [vp, _ip, _ip, _ip, _ip, _ip, _ip]),
        "orc_block_pairs": (None, [vp, i, i, _ip]),
        "orc_cc_info": (None, [vp, _ip, _ip, _ip]),
        "orc_set_num_threads": (None, [i]),
        "orc_get_max_threads": (i, []),
        "orc_set_dgemm": (None, [vp, i]),
        "orc_sixj": (d, [i] * 6),
        "orc_ninej": (d, [i] * 9),
        "orc_v_elem": (d, [vp, _dp, i, i, i, i, i, i]),
        "orc_f_elem": (d, [vp, _dp, i, i, i]),
        "orc_random_op": (None, [vp, u64, i, _dp]),
        "orc_synthetic_bare": (None, [vp, u64, d, _dp]),
        "orc_commutator_110": (d, [vp, _dp, i, _dp, i]),
        "orc_commutator_220": (d, [vp, _dp, i, _dp, i]),
        "orc_commutator_111": (None, [vp, _dp, i, _dp, i, _dp, i]),
        "orc_commutator_121": (None, [vp, _dp, i, _dp, i, _dp, i]),
        "orc_commutator_122": (None, [vp, _dp, i, _dp, i, _dp, i]),
        "orc_commutator_222_pp_hh": (None, [vp, _dp, i, _dp, i, _dp, i, _dp, _dp]),
        "orc_commutator_221": (None, [vp, _dp, i, _dp, i, _dp, i, _dp, _dp]),
        "orc_calculate_cross_coupled": (None, [vp, _dp, i, _dp]),
        "orc_commutator_222_ph": (None, [vp, _dp, i, _dp, i, _dp, i, _dp]),
        "orc_full_commutator": (None, [vp, _dp, i, _dp, i, _dp, i]),
        "orc_build_gs_white": (None, [vp, _dp, i, _dp]),
        "orc_build_gs_atanxx": (None, [vp, _dp, i, _dp, _dp]),
        "orc_commutator_e0": (None, [vp, _dp, i, _dp, i, _dp, i, i]),
        "orc_commutator_vjp": (None, [vp, _dp, i, _dp, i, i, i, _dp, _dp, _dp]),
        "orc_white_vjp": (None, [vp, _dp, i, _dp, _dp]),
        "orc_tbasis_create": (vp, [vp, i, i]),
        "orc_tbasis_destroy": (None, [vp]),
        "orc_tslab_size": (i64, [vp]),
        "orc_tnblocks": (i, [vp]),
        "orc_tblock_info": (None, [vp, _ip, _ip, _ip, _ip, _ip, _ip]),
        "orc_random_tensor": (None, [vp, u64, i, _dp]),
        "orc_tensor_commutator": (None, [vp, _dp, i, _dp, i, _dp, i]),
        "orc_tensor_elem": (d, [vp, _dp, i, i, i, i, i, i, i]),
        "orc_f_tensor_elem": (d, [vp, _dp, i, i, i]),
        "orc_tensor_frob": (d, [vp, _dp]),
        "orc_bch_tensor": (i, [vp, _dp, _dp, i, d]),
        "orc_tensor_bf1": (d, [vp, _dp, i, _dp, i, i, i]),
        "orc_tensor_bf2": (d, [vp, _dp, i, _dp, i, i, i, i, i, i, i]),
        "orc_mat_frob_norm": (d, [vp, _dp]),
        "orc_mbpt2": (d, [vp, _dp, i]),
        "orc_add_sq_op": (None, [vp, _dp, d, _dp, d, _dp]),
        "orc_magnus_expand": (i, [vp, _dp, _dp]),
        "orc_bch_expand": (i, [vp, _dp, _dp, _dp, i, d]),
        "orc_cr_expand": (i, [vp, _dp, _dp, _dp, i, d]),
        "orc_bf_0body": (d, [vp, _dp, i, _dp, i]),
        "orc_bf_1body": (d, [vp, _dp, i, _dp, i, i, i]),
        "orc_bf_2body": (d, [vp, _dp, i, _dp, i, i, i, i, i, i]),
        "orc_gamma_matrix": (None, [vp, _dp, i, _dp, _dp]),
        "orc_transform_2b_to_hf": (None, [vp, _dp, _dp]),
        "orc_normal_order": (None, [vp, _dp, i, _dp]),
        "orc_vectorize": (i64, [vp, _dp, _dp]),
        "orc_p1_p2": (d, [vp, i, i, i, i, i]),
        "orc_r1_r2": (d, [vp, i, i, i, i, i]),
        "orc_three_channels": (i, [vp, vp, vp, vp, vp, vp]),
        "orc_restore_quadrupoles": (None, [vp, _dp, i, _dp, i, _dp]),
        "orc_bch_expand_quads": (i, [vp, _dp, _dp, _dp, i, d]),
        "orc_comm223": (d, [vp, _dp, i, _dp, i] + [i] * 9),
        "orc_restore_triples": (d, [vp, _dp, _dp, i]),
        "orc_eom_create": (vp, [vp]),
        "orc_eom_destroy": (None, [vp]),
        "orc_eom_dim": (i64, [vp, C.POINTER(C.c_int64)]),
        "orc_eom_map": (None, [vp, _lp, _bp, _bp, _lp]),
        "orc_eom_unwrap": (None, [vp, vp, _dp, _dp]),
        "orc_eom_rewrap": (None, [vp, _dp, _dp]),
        "orc_eom_bf1": (d, [vp, _dp, i, _dp, i, i]),
        "orc_eom_bf2": (d, [vp, _dp, i, _dp, i, i, i, i, i, i]),
        "orc_pphh_ladder_elem": (d, [vp, _dp, i, i, i, i, i, i]),
        "orc_eom_matvec": (None, [vp, vp, _dp, _dp, _dp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def set_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


def use_blas_dgemm(addr: int, ilp64: bool) -> None:
    lib().orc_set_dgemm(C.c_void_p(addr), 1 if ilp64 else 0)


# reference default-real literal 1e-6 (src/IMSRG_MAGNUS.f90:152)
BCH_CONV = float(np.float32(1e-6))
# calc_HF's convergence test `crit > 1e-6` compares with the same default-real literal
# (src/HF_mod.f90:49)
HF_CONV = float(np.float32(1e-6))


class Oracle:
    """One basis (the reference's jbas + channel layout) on the CPU."""

    def __init__(self, basis):
        self.basis = basis
        L = lib()
        nn, ll, jj, tz, con = basis.arrays()
        self._keep = (nn, ll, jj, tz, con)
        self.h = L.orc_basis_create(nn.size, nn, ll, jj, tz, con, basis.eMax, basis.hw,
                                    basis.Aprot, basis.Aneut)
        self.L = L
        self.slab = int(L.orc_slab_size(self.h))
        self.nblocks = int(L.orc_nblocks(self.h))
        self.ncc = int(L.orc_ncc(self.h))
        self.cc_size = int(L.orc_cc_size(self.h))
        self.wcc_size = int(L.orc_wcc_size(self.h))

    def __del__(self):
        try:
            self.L.orc_basis_destroy(self.h)
        except Exception:
            pass

    # layout -------------------------------------------------------------
    def block_info(self):
        n = self.nblocks
        arrs = [np.zeros(n, np.int32) for _ in range(6)]
        self.L.orc_block_info(self.h, *arrs)
        return dict(zip(("lamJ", "lamP", "lamT", "npp", "nph", "nhh"), arrs))

    def block_pairs(self, q: int, cls: int) -> np.ndarray:
        info = self.block_info()
        n = int((info["npp"], info["nph"], info["nhh"])[cls][q])
        out = np.zeros(2 * n, np.int32)
        if n:
            self.L.orc_block_pairs(self.h, q, cls, out)
        return out.reshape(n, 2)

    def cc_info(self):
        arrs = [np.zeros(self.ncc, np.int32) for _ in range(3)]
        self.L.orc_cc_info(self.h, *arrs)
        return dict(zip(("rlen", "nph", "J"), arrs))

    def new(self) -> np.ndarray:
        return np.zeros(self.slab, np.float64)

    def random(self, seed: int, herm: int) -> np.ndarray:
        x = self.new()
        self.L.orc_random_op(self.h, seed, herm, x)
        return x

    # pieces ---------------------------------------------------------------
    def synthetic_bare_hamiltonian(self, seed: int = 1, v_scale: float = 1.0) -> np.ndarray:
        """The seeded synthetic bare Hamiltonian (me2j-layout records converted to the pn
        J-scheme, HO kinetic energy, E0 = 0): the oracle's own restatement of the input."""
        x = self.new()
        self.L.orc_synthetic_bare(self.h, seed, v_scale, x)
        return x

    def v_elem(self, op, herm, a, b, c, d, J):
        return self.L.orc_v_elem(self.h, op, herm, a, b, c, d, J)

    def f_elem(self, op, herm, a, b):
        return self.L.orc_f_elem(self.h, op, herm, a, b)

    def commutator_110(self, L, hL, R, hR):
        return self.L.orc_commutator_110(self.h, L, hL, R, hR)

    def commutator_220(self, L, hL, R, hR):
        return self.L.orc_commutator_220(self.h, L, hL, R, hR)

    def commutator_111(self, L, hL, R, hR, RES, hRES):
        self.L.orc_commutator_111(self.h, L, hL, R, hR, RES, hRES)

    def commutator_121(self, L, hL, R, hR, RES, hRES):
        self.L.orc_commutator_121(self.h, L, hL, R, hR, RES, hRES)

    def commutator_122(self, L, hL, R, hR, RES, hRES):
        self.L.orc_commutator_122(self.h, L, hL, R, hR, RES, hRES)

    def commutator_222_pp_hh(self, L, hL, R, hR, RES, hRES, w1, w2):
        self.L.orc_commutator_222_pp_hh(self.h, L, hL, R, hR, RES, hRES, w1, w2)

    def commutator_221(self, L, hL, R, hR, RES, hRES, w1, w2):
        self.L.orc_commutator_221(self.h, L, hL, R, hR, RES, hRES, w1, w2)

    def calculate_cross_coupled(self, op, herm):
        cc = np.zeros(self.cc_size, np.float64)
        self.L.orc_calculate_cross_coupled(self.h, op, herm, cc)
        return cc

    def commutator_222_ph(self, LCC, hL, RCC, hR, RES, hRES, WCC=None):
        if WCC is None:
            WCC = np.zeros(self.wcc_size, np.float64)
        self.L.orc_commutator_222_ph(self.h, LCC, hL, RCC, hR, RES, hRES, WCC)
        return WCC

    def commutator(self, L, hL, R, hR, hRES=None):
        """Full [L,R] in the reference's order; E0 assigned."""
        if hRES is None:
            hRES = -hL * hR
        RES = self.new()
        self.L.orc_full_commutator(self.h, L, hL, R, hR, RES, hRES)
        return RES

    def commutator_e0(self, L, hL, R, hR, hRES, with_e0):
        RES = self.new()
        self.L.orc_commutator_e0(self.h, L, hL, R, hR, RES, hRES, 1 if with_e0 else 0)
        return RES

    def commutator_vjp(self, L, hL, R, hR, hRES, with_e0, Cb):
        """(Lb, Rb): gradients of <Cb, [L, R]> (exact transpose of the forward routine)."""
        Lb, Rb = self.new(), self.new()
        self.L.orc_commutator_vjp(self.h, L, hL, R, hR, hRES, 1 if with_e0 else 0, Cb, Lb, Rb)
        return Lb, Rb

    def white_vjp(self, H, hH, ETAb):
        Hb = self.new()
        self.L.orc_white_vjp(self.h, H, hH, ETAb, Hb)
        return Hb

    def white(self, H, hH=1):
        ETA = self.new()
        self.L.orc_build_gs_white(self.h, H, hH, ETA)
        return ETA

    def atan(self, H, hH=1):
        """build_gs_atan (src/generators.f90:163-266)."""
        ETA = self.new()
        self.L.orc_build_gs_atanxx(self.h, H, hH, H, ETA)
        return ETA

    def atanxx(self, Hold, H, hold=1):
        """build_gs_atanxx (src/generators.f90:271-374): numerators of H, denominators of Hold."""
        ETA = self.new()
        self.L.orc_build_gs_atanxx(self.h, Hold, hold, np.ascontiguousarray(H), ETA)
        return ETA

    def w2(self, H, hH=1):
        """build_gs_w2 (src/generators.f90:109-160): 1.5 atan(H) + 0.5 atanxx(H, [atan(H), H])."""
        eta1 = self.atan(H, hH)
        H2 = self.commutator(eta1, -1, H, hH)
        eta2 = self.atanxx(H, H2, hH)
        return 1.5 * eta1 + 0.5 * eta2

    def frob(self, op):
        return self.L.orc_mat_frob_norm(self.h, op)

    def mbpt2(self, H, hH=1):
        return self.L.orc_mbpt2(self.h, H, hH)

    def magnus_expand(self, DG, G):
        """In place: DG (eta on entry) becomes dOmega.  Returns commutators used."""
        return self.L.orc_magnus_expand(self.h, DG, G)

    def bch_expand(self, G, H, max_terms=40, conv=BCH_CONV):
        HS = self.new()
        n = self.L.orc_bch_expand(self.h, HS, G, H, max_terms, conv)
        return HS, n

    def cr_expand(self, G, H, max_terms=14, conv=BCH_CONV):
        """CR_EXPAND (src/IMSRG_MAGNUS.f90:532-617): sum_n ad_G^n(H) / (n+1)!."""
        HS = self.new()
        n = self.L.orc_cr_expand(self.h, HS, G, H, max_terms, conv)
        return HS, n

    # brute force ---------------------------------------------------------
    def bf_0body(self, A, hA, B, hB):
        return self.L.orc_bf_0body(self.h, A, hA, B, hB)

    def bf_1body(self, A, hA, B, hB, a, b):
        return self.L.orc_bf_1body(self.h, A, hA, B, hB, a, b)

    def bf_2body(self, A, hA, B, hB, a, b, c, d, J):
        return self.L.orc_bf_2body(self.h, A, hA, B, hB, a, b, c, d, J)

    # ---- quadrupoles (src/IMSRG_MAGNUS.f90:908-1132)
    def restore_quadrupoles(self, X, hX, OM, hOM):
        """restore_quadrupoles: the pp-hh arrays it assigns (zero elsewhere)."""
        RES = self.new()
        self.L.orc_restore_quadrupoles(self.h, X, hX, OM, hOM, RES)
        return RES

    def bch_expand_quads(self, G, H, max_terms=40, conv=BCH_CONV):
        """BCH_EXPAND with quads = 'y'."""
        HS = self.new()
        n = self.L.orc_bch_expand_quads(self.h, HS, G, H, max_terms, conv)
        return HS, n

    # ---- perturbative triples (src/IMSRG_MAGNUS.f90:767-902)
    def three_channels(self):
        """enumerate_three_body: per channel (Jtot, Tz, parity, #ppp, #hhh)."""
        n = self.L.orc_three_channels(self.h, None, None, None, None, None)
        arrs = [np.zeros(n, np.int32) for _ in range(5)]
        self.L.orc_three_channels(self.h, *[a.ctypes.data for a in arrs])
        return dict(zip(("J", "Tz", "P", "nppp", "nhhh"), arrs))

    def comm223(self, L, hL, R, hR, p, q, r, s, t, u, Jtot, jpq, jst):
        """commutator_223_single (src/commutators.f90:928-1325)."""
        return self.L.orc_comm223(self.h, L, hL, R, hR, p, q, r, s, t, u, Jtot, jpq, jst)

    def restore_triples(self, H, OM, chan=-1):
        """restore_triples: the triples correction of H (herm +1) and Omega (herm -1)."""
        return self.L.orc_restore_triples(self.h, H, OM, int(chan))

    # ---- Hartree-Fock input preparation (src/HF_mod.f90)
    def sp_blocks(self) -> list:
        """Orbits sharing (l, j, tz), ascending: the blocks of a full_sp_block_mat."""
        b = self.basis
        groups: dict = {}
        for i in range(b.norbits):
            groups.setdefault((int(b.ll[i]), int(b.jj[i]), int(b.itzp[i])), []).append(i)
        return [np.array(v) for v in groups.values()]

    def gamma_matrix(self, H, hH, rho) -> np.ndarray:
        """gamma_matrix (src/HF_mod.f90:242-305) of a density scaled by (2j+1)."""
        N = self.basis.norbits
        out = np.zeros(N * N)
        self.L.orc_gamma_matrix(self.h, H, hH, np.ascontiguousarray(rho.ravel(order="F")), out)
        return out.reshape(N, N, order="F")

    def normal_order(self, op, herm=1) -> np.ndarray:
        """normal_order (src/basic_IMSRG.f90:2419-2550)."""
        out = np.zeros(self.slab)
        self.L.orc_normal_order(self.h, op, herm, out)
        return out

    def p1_p2(self, a, b, c, d, J) -> float:
        """p1_p2 (src/basic_IMSRG.f90:4445-4504)."""
        return self.L.orc_p1_p2(self.h, a, b, c, d, J)

    def r1_r2(self, a, b, c, d, J) -> float:
        """r1_r2 (src/basic_IMSRG.f90:4506-4565)."""
        return self.L.orc_r1_r2(self.h, a, b, c, d, J)

    def vectorize(self, op) -> np.ndarray:
        """vectorize (src/basic_IMSRG.f90:3929-3985)."""
        out = np.zeros(self.slab)  # the vector is never longer than the slab
        n = self.L.orc_vectorize(self.h, op, out)
        return out[:n].copy()

    def transform_2b_to_hf(self, op, D) -> np.ndarray:
        """transform_2b_to_HF (src/HF_mod.f90:567-692); D(HO orbit, HF orbit), N x N."""
        out = np.array(op, dtype=np.float64, copy=True)
        self.L.orc_transform_2b_to_hf(self.h, out, np.ascontiguousarray(D.ravel(order="F")))
        return out

    def _kin_matrix(self, op, herm=1) -> np.ndarray:
        """write_kin_matrix (src/HF_mod.f90:211-240): f_elem on each block's upper triangle."""
        N = self.basis.norbits
        T = np.zeros((N, N))
        for st in self.sp_blocks():
            for x in range(len(st)):
                for y in range(x, len(st)):
                    T[st[x], st[y]] = T[st[y], st[x]] = self.f_elem(op, herm, int(st[x]), int(st[y]))
        return T

    def _write_f(self, out, st, Fp) -> None:
        """The remap of transform_1b_to_HF (src/HF_mod.f90:530-560) for one block."""
        b = self.basis
        con = np.array(b.con)
        A, P = b.nholes, b.norbits - b.nholes
        loc = np.zeros(b.norbits, dtype=int)
        loc[con == 1] = np.arange(A)
        loc[con == 0] = np.arange(P)
        o_hh, o_pp = 1, 1 + A * A
        o_ph = o_pp + P * P
        for x in range(len(st)):
            for y in range(x, len(st)):
                i, j = int(st[x]), int(st[y])
                c1, c2 = con[i], con[j]
                if c1 + c2 == 0:
                    out[o_pp + loc[i] + loc[j] * P] = out[o_pp + loc[j] + loc[i] * P] = Fp[x, y]
                elif c1 + c2 == 1:
                    if c2 > c1:
                        out[o_ph + loc[i] + loc[j] * P] = Fp[x, y]
                    else:
                        out[o_ph + loc[j] + loc[i] * P] = Fp[y, x]
                else:
                    out[o_hh + loc[i] + loc[j] * A] = out[o_hh + loc[j] + loc[i] * A] = Fp[x, y]

    def _hf(self, H, max_iter, iterate):
        b = self.basis
        N = b.norbits
        jj, con = np.array(b.jj), np.array(b.con)
        blocks = self.sp_blocks()
        T = self._kin_matrix(H)
        D = [np.eye(len(st)) for st in blocks]
        eig = [np.zeros(len(st)) for st in blocks]

        def density():  # density_matrix (src/HF_mod.f90:419-446)
            rho = np.zeros((N, N))
            for k, st in enumerate(blocks):
                Dx = D[k] * con[st][None, :]
                rho[np.ix_(st, st)] = (Dx @ Dx.T) * (jj[st[0]] + 1)
            return rho

        r = 0
        if iterate:  # calc_HF main loop (src/HF_mod.f90:56-81)
            crit = 10.0
            while crit > HF_CONV:
                if r >= max_iter:
                    raise RuntimeError("Hartree-Fock did not converge")
                Vgam = self.gamma_matrix(H, 1, density())
                crit = 0.0
                for k, st in enumerate(blocks):
                    ix = np.ix_(st, st)
                    w, v = np.linalg.eigh(T[ix] + Vgam[ix], UPLO="U")  # dsyev('V','U')
                    crit += float(np.sqrt(np.sum((eig[k] - w) ** 2)))
                    D[k], eig[k] = v, w
                r += 1
        else:  # calc_HO (src/HF_mod.f90:107-179)
            Vgam = self.gamma_matrix(H, 1, density())
        out = np.array(H, dtype=np.float64, copy=True)
        Dfull = np.zeros((N, N))
        E = 0.0
        for k, st in enumerate(blocks):
            Dk = D[k]
            for i in range(len(st)):
                if Dk[i, i] < 0.0:
                    Dk[:, i] = -Dk[:, i]
            ix = np.ix_(st, st)
            F = T[ix] + Vgam[ix]
            Fp = Dk.T @ (F @ Dk)
            Tp = Dk.T @ (T[ix] @ Dk)
            Vp = Dk.T @ (Vgam[ix] @ Dk)
            self._write_f(out, st, Fp)
            # e_HF (src/HF_mod.f90:449-478)
            E += float(np.sum((np.diag(Tp) + 0.5 * np.diag(Vp)) * con[st] * (jj[st[0]] + 1.0)))
            Dfull[ix] = Dk
        out[0] = E
        out = self.transform_2b_to_hf(out, Dfull)
        return out, Dfull, E, r

    def calc_hf(self, H, max_iter: int = 10000):
        """calc_HF (src/HF_mod.f90:14-105) of a bare Hamiltonian slab (kinetic energy in the
        one-body arrays, V in the two-body arrays, E0 unused).  Returns the normal-ordered
        Hamiltonian in the HF basis, D(HO orbit, HF orbit), E_HF and the iteration count."""
        return self._hf(H, max_iter, True)

    def calc_ho(self, H):
        """calc_HO (src/HF_mod.f90:107-179): the same steps with D = 1 and no iteration."""
        return self._hf(H, 0, False)

    def sqop_to_hf(self, op, D) -> np.ndarray:
        """sqop_to_HF (src/HF_mod.f90:181-209) of a bare hermitian scalar operator."""
        out = np.array(op, dtype=np.float64, copy=True)
        T = self._kin_matrix(op)
        for st in self.sp_blocks():
            ix = np.ix_(st, st)
            Dk = D[ix]
            self._write_f(out, st, Dk.T @ (T[ix] @ Dk))
        out = self.transform_2b_to_hf(out, D)
        return self.normal_order(out, 1)


class TensorOracle:
    """Rank-lambda tensor operators of the oracle on a scalar Oracle's basis (test-only)."""

    def __init__(self, o: "Oracle", rank: int, dpar: int = 0):
        self.o, self.L, self.rank, self.dpar = o, o.L, rank, dpar
        self.h = self.L.orc_tbasis_create(o.h, rank, dpar)
        self.slab = int(self.L.orc_tslab_size(self.h))
        self.nblocks = int(self.L.orc_tnblocks(self.h))

    def __del__(self):
        try:
            self.L.orc_tbasis_destroy(self.h)
        except Exception:
            pass

    def new(self):
        return np.zeros(self.slab)

    def block_info(self):
        arrs = [np.zeros(self.nblocks, np.int32) for _ in range(6)]
        self.L.orc_tblock_info(self.h, *arrs)
        return dict(zip(("J1", "J2", "Tz", "P1", "q1", "q2"), arrs))

    def random(self, seed: int, herm: int):
        op = self.new()
        self.L.orc_random_tensor(self.h, seed, herm, op)
        return op

    def commutator(self, L, hL, R, hR, mask=127):
        """[L (scalar), R (tensor)]; RES herm = -hL*hR."""
        RES = self.new()
        self.L.orc_tensor_commutator(self.h, L, hL, R, hR, RES, mask)
        return RES

    def elem(self, op, herm, a, b, c, d, J1, J2):
        return self.L.orc_tensor_elem(self.h, op, herm, a, b, c, d, J1, J2)

    def f_elem(self, op, herm, a, b):
        return self.L.orc_f_tensor_elem(self.h, op, herm, a, b)

    def frob(self, op):
        return self.L.orc_tensor_frob(self.h, op)

    def bch(self, G, HS, max_terms=30, conv=float(np.float32(1e-6))):
        out = np.array(HS, dtype=np.float64)
        n = self.L.orc_bch_tensor(self.h, G, out, max_terms, conv)
        return out, n

    def bf1(self, A, hA, B, hB, a, b):
        return self.L.orc_tensor_bf1(self.h, A, hA, B, hB, a, b)

    def bf2(self, A, hA, B, hB, a, b, c, d, J1, J2):
        return self.L.orc_tensor_bf2(self.h, A, hA, B, hB, a, b, c, d, J1, J2)


class EomOracle:
    """EOM-IMSRG ladder operators of rank `rank` / parity change `dpar` (doubled) on a scalar
    Oracle's basis (test-only): the amplitude vector of unwrap_tensor / rewrap_tensor
    (src/EOM_IMSRG.f90:1039-1340), the known-answer formulas of the reference's EOM
    scalar-tensor test and the matrix-vector product of matvec_nonzeroX_prod (:518-556)."""

    def __init__(self, o: "Oracle", rank: int, dpar: int = 0):
        self.t = TensorOracle(o, rank, dpar)
        self.o, self.L = o, o.L
        self.m = self.L.orc_eom_create(self.t.h)
        n1b = C.c_int64()
        self.n = int(self.L.orc_eom_dim(self.m, C.byref(n1b)))
        self.n1b = int(n1b.value)

    def __del__(self):
        try:
            self.L.orc_eom_destroy(self.m)
        except Exception:
            pass

    def amplitude_map(self):
        pos, mir = np.zeros(self.n, np.int64), np.zeros(self.n, np.int64)
        kind, ph = np.zeros(self.n, np.int8), np.zeros(self.n, np.int8)
        self.L.orc_eom_map(self.m, pos, kind, ph, mir)
        return dict(pos=pos, kind=kind, phase=ph, mirror=mir)

    def unwrap(self, v):
        X = self.t.new()
        self.L.orc_eom_unwrap(self.t.h, self.m, np.ascontiguousarray(v, dtype=np.float64), X)
        return X

    def rewrap(self, X):
        v = np.zeros(self.n)
        self.L.orc_eom_rewrap(self.m, X, v)
        return v

    def bf1(self, H, X, a, b):
        return self.L.orc_eom_bf1(self.t.h, H, 1, X, a, b)

    def bf2(self, H, X, a, b, c, d, J1, J2):
        return self.L.orc_eom_bf2(self.t.h, H, 1, X, a, b, c, d, J1, J2)

    def pphh(self, X, a, b, c, d, J1, J2):
        return self.L.orc_pphh_ladder_elem(self.t.h, X, a, b, c, d, J1, J2)

    def matvec(self, H, v):
        w = np.zeros(self.n)
        self.L.orc_eom_matvec(self.t.h, self.m, H, np.ascontiguousarray(v, dtype=np.float64), w)
        return w

    def matrix(self, H):
        """The dense EOM matrix, column k = matvec of the k-th unit vector."""
        M = np.zeros((self.n, self.n))
        e = np.zeros(self.n)
        for k in range(self.n):
            e[k] = 1.0
            M[:, k] = self.matvec(H, e)
            e[k] = 0.0
        return M
