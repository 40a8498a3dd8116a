"""The mixed form's rebuild test is VerletList::decide's half-skin test in
FP64 (mdcraft/neibs/verlet-list.cxx:135-154): a step of the device loop
rebuilds exactly when |shortest(r - r_saved)|^2 > (skin/2)^2 holds in the
reference's FP64 operation order on the positions the drift produced.

Displacements are placed one position-ulp either side of the threshold (an
FP32 test, or any test with a safety margin, rebuilds on both sides), and a
hot EAM run driven by the device loop is compared with the same run driven
step by step from the host through the FP64 decide."""
from fractions import Fraction

import numpy as np
import pytest

import mdcraft_gb300 as mdg
from mdcraft_gb300 import workloads as W
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu

RC, RNS, DT = 0.5, 0.55, 0.002
BOX = (0.0, 6.0, 0.0, 6.0, 0.0, 6.0)


def _fma(a, b, c):
    """fma(a, b, c) of IEEE doubles, correctly rounded."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _trig():
    skin = RNS - RC
    return (0.25 * skin) * skin


def _need(r1, r0):
    """decide's displacement test for one atom in the reference's order
    (Domain::shortest is a no-op here: displacements are far below L/2)."""
    d = [r1[k] - r0[k] for k in range(3)]
    return ((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]) > _trig()


def _velocity_for(x0, target):
    """A velocity v with fma(v, DT, x0) == target (the mixed drift's update
    of a force-free atom)."""
    v = float((Fraction(target) - Fraction(x0)) / Fraction(DT))
    for _ in range(64):
        got = _fma(v, DT, x0)
        if got == target:
            return v
        v = np.nextafter(v, np.inf if got < target else -np.inf)
    raise AssertionError("no velocity lands on the target position")


def _straddle(x0, direction):
    """Positions x0 + t*direction one ulp either side of the half-skin
    threshold: (last position that does not trigger, first that does)."""
    u = np.asarray(direction, dtype=np.float64)
    u = u / np.linalg.norm(u)
    t = np.sqrt(_trig())
    below = above = None
    for k in range(-400, 400):
        tk = t * (1.0 + k * 2.0 ** -50)
        r1 = [float(x0[a] + tk * u[a]) if u[a] != 0.0 else float(x0[a]) for a in range(3)]
        if _need(r1, x0):
            if above is None:
                above = r1
        else:
            below = r1
    assert below is not None and above is not None
    return below, above


def _gas(moving_r0, moving_v):
    """Force-free LJ gas: the moving atom plus static atoms more than rns
    from every other atom."""
    static = [(3.0, 3.0, 3.0), (4.5, 1.5, 4.5), (1.5, 4.5, 1.5), (4.5, 4.5, 1.5)]
    a = W.new_atoms(1 + len(static))
    a["r"][0] = moving_r0
    a["v"][0] = moving_v
    for k, p in enumerate(static):
        a["r"][k + 1] = p
    a["m"] = 39.948
    a["rcut"] = RC
    a["rns"] = RNS
    a["uid"] = np.arange(1, len(a) + 1)
    return a


CASES = [((0.5, 0.5, 0.5), (1.0, 0.0, 0.0)),
         ((0.0078125, 2.0, 2.0), (1.0, 0.0, 0.0)),
         ((0.75, 0.75, 0.75), (1.0, 1.0, 0.0)),
         ((1.25, 2.5, 0.625), (0.3, -0.5, 0.8))]


@pytest.mark.parametrize("case", CASES, ids=["x_at_half", "x_near_zero", "diagonal_xy", "oblique"])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_rebuild_exactly_at_half_skin(case, precision):
    x0, direction = case
    for r_target, expect_hint in zip(_straddle(x0, direction), (False, True)):
        v = [(_velocity_for(x0[a], r_target[a]) if r_target[a] != x0[a] else 0.0) for a in range(3)]
        atoms = _gas(x0, v)
        dg = mdg.Domain(*BOX)
        for k in range(3):
            dg.set_periodic(k, True)
        s = mdg.System(H.ctx(), dg, atoms)
        nl = mdg.VerletList(s)
        nl.update(-1.0)
        pot = mdg.LJsCut(1.0, 0.3, RC)
        sol = mdg.Single(pot, periodic=True, precision=precision)
        sol.prepare(s)
        sol.stages(s)
        rb0 = nl.rebuilds()
        mdg.Verlet(sol).run(s, DT, 1)
        r1 = s.positions()[0]
        expected = _need([float(x) for x in r1], list(x0))
        if precision == "mixed":
            # the mixed drift lands exactly on the chosen position
            assert [float(x) for x in r1] == r_target
            assert expected == expect_hint
        assert (nl.rebuilds() - rb0) == int(expected), (precision, x0, direction, r1, expected)


def test_device_loop_rebuilds_where_host_fp64_decide_does():
    """A hot EAM Cu run (many rebuilds): the device loop (mdg_run, its drift
    deciding) and the reference driver loop from the host (make_step, FP64
    decide(), update(-1)) rebuild on the same steps and end bit-identical."""
    atoms, box, per, p = W.eam_cu_fcc(ncell=8, seed=21, T=2500.0, jitter=0.02)
    steps = 120
    runs = {}
    for mode in ("device", "host"):
        _, g = H.make_pair(atoms, box, (1, 1, 1), p, precision="mixed")
        g["nl"].update(-1.0)
        g["solver"].prepare(g["sys"])
        g["solver"].stages(g["sys"])
        rb0 = g["nl"].rebuilds()
        if mode == "device":
            g["stepper"].run(g["sys"], p["dt"], steps)
            trace = None
        else:
            trace = []
            for k in range(steps):
                g["stepper"].make_step(g["sys"], p["dt"])
                if g["nl"].decide():
                    g["nl"].update(-1.0)
                    trace.append(k)
        runs[mode] = (g["nl"].rebuilds() - rb0, g["sys"].positions(), g["sys"].velocities(), trace)
    nd, rd, vd, _ = runs["device"]
    nh, rh, vh, trace = runs["host"]
    assert nh >= 5, f"the run should rebuild often (host loop rebuilt {nh} times)"
    assert nd == nh, (nd, nh, trace)
    assert np.array_equal(rd, rh)
    assert np.array_equal(vd, vh)
