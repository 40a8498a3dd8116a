"""CPU check of the oracle's velocity-Verlet step against its defining
equations (no GPU).

Verlet::make_step (mdcraft/solver/stepper/verlet.cxx:36-48) is
step_one_coords (verlet.cxx:71-78: v += f/m dt/2, r += v dt), the force
stages at the new positions, then step_one_velocities (verlet.cxx:80-85:
v += f/m dt/2). Atoms with tag 0 are skipped. Restated in numpy in the same
operation order (no fused multiply-adds), one step of the oracle agrees bit
for bit in positions and velocities. Its new forces equal an independent
evaluation at the drifted positions to 1e-12.
"""
import numpy as np
import pytest

from mdcraft_gb300 import workloads as W
from oracle import mdref as R
from tests.test_oracle_gradients import _oracle_atoms, _solver


def _forces(atoms, box, p):
    a = atoms.copy()
    d = R.Domain(*box)
    for k in range(3):
        d.set_periodic(k, True)
    nl = R.VerletList(a, d, threads=1)
    nl.update(-1.0)
    s = _solver(p, d)
    s.prepare(a)
    s.stages(a, nl)
    return a, nl, s, d


@pytest.mark.parametrize("make", [lambda: W.lj_argon_fcc(ncell=5, jitter=0.02, T=300.0),
                                  lambda: W.eam_cu_fcc(ncell=5, T=900.0)], ids=["lj_argon", "eam_cu"])
def test_make_step_is_velocity_verlet(make):
    atoms, box, _, p = make()
    a0 = _oracle_atoms(atoms)
    a0["tag"][7] = 0  # skipped by both half-steps
    a, nl, s, d = _forces(a0, box, p)
    dt = p["dt"]
    r, v, f, m = a["r"].copy(), a["v"].copy(), a["f"].copy(), a["m"][:, None]
    live = (a["tag"] != 0)[:, None]
    v_half = np.where(live, v + f / m * dt * 0.5, v)
    r1 = np.where(live, r + v_half * dt, r)

    s.make_step(a, nl, dt)

    assert np.array_equal(a["r"], r1)
    # the new forces are those of the drifted positions (a fresh list there
    # may sum in another order)
    b = a0.copy()
    b["r"] = r1
    b_eval, _, _, _ = _forces(b, box, p)
    scale = np.max(np.abs(b_eval["f"]))
    assert np.max(np.abs(a["f"] - b_eval["f"])) <= 1e-12 * scale
    v1 = np.where(live, v_half + a["f"] / m * 0.5 * dt, v_half)
    assert np.array_equal(a["v"], v1)
    assert np.array_equal(a["r"][7], r[7]) and np.array_equal(a["v"][7], v[7])
