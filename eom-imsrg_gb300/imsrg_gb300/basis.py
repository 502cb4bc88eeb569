"""Single-particle j-scheme bases for the IMSRG(2) engine.

The reference reads its harmonic-oscillator orbits from ``sp_inputs/hk<eMax>.sps``
(``read_sp_basis``, src/basic_IMSRG.f90:192-382) and marks the occupied ones from the
``hole_scheme_hk`` table (``find_holes``, src/basic_IMSRG.f90:385-440).  The ``hk`` files
list orbits by shell e = 2n + l, then by l ascending, then 2j ascending, then 2tz = -1
(proton) before +1 (neutron); this module regenerates exactly that order, so no data
file is needed on the machine that runs the engine.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

HBARC = 197.326968
# src/basic_IMSRG.f90:141 declares m_nuc with a default-real (FP32) literal
M_NUC = float(np.float32(938.918725))


@dataclass
class Basis:
    """The reference's ``type(spd)`` fields that the commutator engine needs."""

    nn: np.ndarray
    ll: np.ndarray
    jj: np.ndarray      # 2*j
    itzp: np.ndarray    # 2*tz (-1 proton, +1 neutron)
    con: np.ndarray     # 1 hole, 0 particle
    e: np.ndarray       # shell energy label from the sps file (2n+l)
    eMax: int
    lMax: int
    hw: float = 20.0
    Aprot: int = 8
    Aneut: int = 8
    name: str = field(default="")

    @property
    def norbits(self) -> int:
        return int(self.nn.size)

    @property
    def nholes(self) -> int:
        return int(self.con.sum())

    @property
    def jtotal_max(self) -> int:
        return int(self.jj.max())

    def arrays(self):
        """int32 arrays (nn, ll, jj, itzp, con) in orbit order."""
        return tuple(np.ascontiguousarray(x, dtype=np.int32) for x in
                     (self.nn, self.ll, self.jj, self.itzp, self.con))


def ho_orbits(emax: int, lmax: int | None = None):
    """Orbit list (n, l, 2j, 2tz, e) in the order of the reference's hk*.sps files."""
    out = []
    for e in range(emax + 1):
        for l in range(e % 2, e + 1, 2):
            if lmax is not None and l > lmax:
                continue
            n = (e - l) // 2
            for j2 in (2 * l - 1, 2 * l + 1):
                if j2 < 1:
                    continue
                for tz in (-1, 1):
                    out.append((n, l, j2, tz, e))
    return out


# Shell-model filling used for the closed-shell references the configurations name.
# (Z, N) -> number of leading hk orbits that are holes; the "8 8" row of hole_scheme_hk
# marks the first six orbits (0s1/2 and 0p for protons and neutrons).
_CLOSED = {(2, 2): 2, (8, 8): 6}


def closed_shell_con(norb: int, Z: int, N: int) -> np.ndarray:
    if (Z, N) not in _CLOSED:
        raise ValueError(f"no closed-shell hole pattern for Z={Z}, N={N}")
    con = np.zeros(norb, dtype=np.int32)
    con[: _CLOSED[(Z, N)]] = 1
    return con


def make_basis(emax: int, Z: int = 8, N: int = 8, hw: float = 20.0, lmax: int | None = None) -> Basis:
    orb = ho_orbits(emax, lmax)
    a = np.array(orb, dtype=np.int32)
    con = closed_shell_con(len(orb), Z, N)
    return Basis(nn=a[:, 0].copy(), ll=a[:, 1].copy(), jj=a[:, 2].copy(), itzp=a[:, 3].copy(),
                 con=con, e=a[:, 4].astype(np.float64), eMax=emax,
                 lMax=int(a[:, 1].max()) if lmax is None else lmax, hw=hw, Aprot=Z, Aneut=N,
                 name=f"hk{emax}")
