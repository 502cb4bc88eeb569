"""Omega checkpoints on the device: write_omega_checkpoint / read_omega_checkpoint and the
checkpoint restart of magnus_decouple (src/IMSRG_MAGNUS.f90:62-97, src/basic_IMSRG.f90:3215-3407).

A flow that restarts from the newest checkpoint rebuilds H(s) = BCH(Omega, H) as the
uninterrupted flow did at that step, so both end with the same operators.  Not bit for bit:
repackage, like the reference's, writes the diagonal of a square array as herm x itself, which
flips the sign of the round-off left on the diagonal of the anti-hermitian Omega.
"""
import os

import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu

PREFIX = "synthetic_eMax04_hwHO020"


def test_checkpoint_file_round_trip(built_lib, oracles, tmp_path):
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300._lib import ImsrgError
    o = oracles(4)
    eng = Engine(make_basis(4), device=0)
    X = o.random(41, -1)
    G = eng.new_op(-1, X)
    path = str(tmp_path / "omega.bin")
    eng.write_omega_checkpoint(G, path)
    assert os.path.getsize(path) == 8 * eng.neq
    assert np.array_equal(np.fromfile(path, dtype=np.float64), o.vectorize(X))
    G2 = eng.new_op(-1)
    eng.read_omega_checkpoint(G2, path)
    assert np.array_equal(G2.download(), X)
    with open(path, "r+b") as f:
        f.truncate(8 * (eng.neq - 1))
    with pytest.raises(ImsrgError) as e:
        eng.read_omega_checkpoint(G2, path)
    assert e.value.code == 5


def test_flow_restart_from_checkpoint(built_lib, tmp_path):
    from imsrg_gb300 import Engine, make_basis
    from imsrg_gb300.flow import magnus_decouple, omega_checkpoint_name
    eng = Engine(make_basis(4), device=0)
    H = eng.synthetic_hamiltonian(seed=9)
    d = str(tmp_path)
    ops_a = {}
    ra = magnus_decouple(eng, H, max_steps=10, checkpoint=(d, PREFIX), checkpoint_every=4, ops=ops_a)
    # written at the start of steps 4 and 8 (s = 1.5, 3.5); the older one removed
    assert not os.path.exists(os.path.join(d, omega_checkpoint_name(PREFIX, 1.5)))
    assert os.path.exists(os.path.join(d, omega_checkpoint_name(PREFIX, 3.5)))
    ops_b = {}
    rb = magnus_decouple(eng, H, max_steps=10, checkpoint=(d, PREFIX), checkpoint_every=4, ops=ops_b)
    assert rb.steps[0][0] == 7 and rb.steps[0][1] == 3.5 and rb.steps[-1][0] == 10
    assert abs(rb.steps[-1][2] - ra.steps[-1][2]) <= 1e-12 * abs(ra.steps[-1][2])
    for k in ("HS", "G"):
        assert rel_err(ops_b[k].download(), ops_a[k].download()) < 1e-12
