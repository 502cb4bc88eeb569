"""EOM-IMSRG excited states on the device (calculate_excited_states, src/EOM_IMSRG.f90:13-98).

A ladder space is one J^pi: rank-J excitation operators with parity change PAR (rank2 = 2J and
dpar2 = 2 PAR doubled, as in the reference).  Its amplitude vector is the one of unwrap_tensor /
rewrap_tensor, the EOM matrix-vector product is matvec_nonzeroX_prod's rewrap([H, unwrap(v)])
and the eigenvalues of smallest magnitude come from LANCZOS_DIAGONALIZE's Lanczos, all through
the C ABI (imsrg_eom_*).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .engine import Engine, SqOp, TensorOp

# the reference's tol = 1.0E-10 is a default-real literal: the FP32 value widened to FP64
EOM_TOL = float(np.float32(1e-10))
EOM_MAX_ITER = 500


class LadderSpace:
    """The ladder operators of one J^pi (imsrg_eom handle)."""

    def __init__(self, eng: Engine, rank2: int, dpar2: int = 0):
        self.eng, self.rank2, self.dpar2 = eng, int(rank2), int(dpar2)
        h = C.c_void_p()
        eng._ck(eng.L.imsrg_eom_create(eng.h, self.rank2, self.dpar2, C.byref(h)))
        self.h = h
        n, n1 = C.c_int64(), C.c_int64()
        eng._ck(eng.L.imsrg_eom_dim(eng.h, h, C.byref(n), C.byref(n1)))
        self.n, self.n1b = n.value, n1.value

    def close(self):
        if getattr(self, "h", None):
            self.eng.L.imsrg_eom_destroy(self.eng.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def amplitude_map(self) -> dict:
        pos, mir = np.zeros(self.n, np.int64), np.zeros(self.n, np.int64)
        kind, ph = np.zeros(self.n, np.int8), np.zeros(self.n, np.int8)
        self.eng._ck(self.eng.L.imsrg_eom_amplitude_map(self.eng.h, self.h, pos.ctypes.data, kind.ctypes.data,
                                                        ph.ctypes.data, mir.ctypes.data))
        return dict(pos=pos, kind=kind, phase=ph, mirror=mir)

    def matvec(self, H: SqOp, v: np.ndarray) -> np.ndarray:
        """matvec_nonzeroX_prod: rewrap([H, unwrap(v)])."""
        v = np.ascontiguousarray(v, dtype=np.float64)
        if v.size != self.n:
            raise ValueError(f"amplitude vector has {self.n} elements, got {v.size}")
        w = np.empty(self.n)
        self.eng._ck(self.eng.L.imsrg_eom_matvec(self.eng.h, self.h, H.h, v.ctypes.data, w.ctypes.data))
        return w

    def unwrap(self, v: np.ndarray) -> TensorOp:
        X = TensorOp(self.eng, self.rank2, self.dpar2, 1)
        v = np.ascontiguousarray(v, dtype=np.float64)
        self.eng._ck(self.eng.L.imsrg_eom_unwrap(self.eng.h, self.h, v.ctypes.data, X.h))
        return X

    def rewrap(self, X: TensorOp) -> np.ndarray:
        v = np.empty(self.n)
        self.eng._ck(self.eng.L.imsrg_eom_rewrap(self.eng.h, self.h, X.h, v.ctypes.data))
        return v

    def lanczos(self, H: SqOp, nev: int, tol: float = EOM_TOL, max_restarts: int = EOM_MAX_ITER,
                vectors: bool = True):
        """LANCZOS_DIAGONALIZE: the nev eigenvalues of smallest magnitude, ascending, their
        normalised amplitude vectors (columns) and the counts of products and restarts."""
        e = np.zeros(nev)
        V = np.zeros((nev, self.n)) if vectors else None
        mv, rs = C.c_int32(), C.c_int32()
        self.eng._ck(self.eng.L.imsrg_eom_lanczos(self.eng.h, self.h, H.h, int(nev), float(tol), int(max_restarts),
                                                  e.ctypes.data, V.ctypes.data if vectors else None,
                                                  C.byref(mv), C.byref(rs)))
        return e, (V.T if vectors else None), {"matvecs": mv.value, "restarts": rs.value}


def calculate_excited_states(eng: Engine, HS: SqOp, J: int, PAR: int, nstates: int, prefix: str | None = None,
                             output_dir: str = ".", lawson_beta: float = 0.0, tol: float = EOM_TOL):
    """calculate_excited_states (src/EOM_IMSRG.f90:13-98) for J (not doubled) and parity PAR
    (0 positive, 1 negative): the rows (dE, E0 + dE, n(1p1h)) of the reference's printout, where
    n(1p1h) is the squared norm of the fph amplitudes of the normalised state.  With prefix set,
    the rows are written to <output_dir>/<prefix>_EOM_spec_law<beta>.dat as the reference writes
    them ('(3(f16.9))')."""
    space = LadderSpace(eng, 2 * J, 2 * PAR)
    E, V, info = space.lanczos(HS, nstates, tol)
    E0 = HS.E0
    rows = [(float(E[i]), float(E[i] + E0), float(np.sum(V[:space.n1b, i] ** 2))) for i in range(nstates)]
    if prefix is not None:
        name = os.path.join(output_dir, f"{prefix.strip()}_EOM_spec_law{int(round(lawson_beta))}.dat")
        with open(name, "w") as f:
            for r in rows:
                f.write("".join(f"{x:16.9f}" for x in r) + "\n")
    return rows, info
