"""GB300-native IMSRG(2) commutator engine (drop-in for the EOM-IMSRG hot path)."""
from .basis import Basis, ho_orbits, make_basis
from .engine import CONV, CCMat, Engine, SqOp
from ._lib import ImsrgError

__all__ = ["Basis", "ho_orbits", "make_basis", "Engine", "SqOp", "CCMat", "CONV", "ImsrgError"]
