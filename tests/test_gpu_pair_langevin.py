"""GPU parity of the tabulated Pair and LJs potentials (mdcraft/solver/
potential/pair.cxx, LJs.cxx), of Multi solvers that mix potential types (multi.cxx:28-151), and
of the Langevin thermostat (mdcraft/solver/thermostat/langevin.cxx:29-42)
against the CPU oracle.

Bars: FP64 forces/energies within 1e-10 relative of the oracle (the
thermostat's normals come from the same Philox stream; its cos/sin/log
differ from the host's by an ulp, hence 1e-10 on positions after steps);
mixed-precision forces within ||dF||_2/||F||_2 <= 1e-5 of FP64."""
import numpy as np
import pytest

import mdcraft_gb300 as mdg
from oracle import mdref as R
from tests import gpu_helpers as H
from tests import mdsupport as S

pytestmark = pytest.mark.gpu

FP64_REL = 1e-10
MIXED_L2 = 1e-5


def _fcc(n, a, seed, mass=26.9815, jitter=0.02):
    atoms, box = S.make_fcc_bulk(n, n, n, a, mass, mdg.ATOM_DTYPE)
    rng = np.random.default_rng(seed)
    atoms["r"] += rng.normal(0.0, jitter * a, size=(len(atoms), 3))
    atoms["v"] = rng.normal(0.0, 0.5, size=(len(atoms), 3))
    return atoms, box


def _spec_pots(spec):
    """(oracle potential, device potential) for ('pair'|'eam'|'lj', table)."""
    kind, t = spec
    if kind == "pair":
        return R.Pair(t["rcut"], t["Vpar"], t["Nr1"], t["dr"]), mdg.Pair(t["rcut"], t["Vpar"], t["Nr1"], t["dr"])
    if kind == "eam":
        args = (t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
        return R.EAM(*args), mdg.EAM(*args)
    if kind == "ljs":
        return R.LJs(*t), mdg.LJs(*t)
    return R.LJsCut(*t), mdg.LJsCut(*t)


def _build(atoms, box, pots, rc, precision="fp64", thermo=None):
    """pots: a single spec (Single) or {(i, j): spec} (Multi, 2 kinds)."""
    atoms = atoms.copy()
    atoms["rcut"] = rc
    atoms["rns"] = rc + 0.05
    do, dg = H.domains(box, (1, 1, 1))
    keep = []
    if isinstance(pots, dict):
        so = R.Solver(None, periodic=do, threads=R.hardware_threads(), nkinds=2)
        sg = mdg.Multi(2, periodic=True, precision=precision)
        for (i, j), spec in pots.items():
            po, pg = _spec_pots(spec)
            so.add_potential(i, j, po)
            sg.add_potential(i, j, pg)
            keep.append((po, pg))
    else:
        po, pg = _spec_pots(pots)
        so = R.Solver(po, periodic=do, threads=R.hardware_threads())
        sg = mdg.Single(pg, periodic=True, precision=precision)
        keep.append((po, pg))
    if thermo is not None:
        th_o = R.Thermostat(*thermo)
        so.set_thermostat(th_o)
        th_g = mdg.Compound(*[mdg.Langevin(**t) for t in thermo])
        sg.set_thermostat(th_g)
        keep.append((th_o, th_g))
    ao = H.to_oracle_atoms(atoms)
    nlo = R.VerletList(ao, do, threads=R.hardware_threads())
    sysg = mdg.System(H.ctx(), dg, atoms)
    nlg = mdg.VerletList(sysg)
    return dict(atoms=ao, nl=nlo, solver=so, dom=do, keep=keep), dict(sys=sysg, nl=nlg, solver=sg, dom=dg)


def _forces_both(o, g):
    o["nl"].update(-1.0)
    g["nl"].update(-1.0)
    for fn in ("prepare", "stages", "virials"):
        getattr(o["solver"], fn)(o["atoms"]) if fn == "prepare" else getattr(o["solver"], fn)(o["atoms"], o["nl"])
        getattr(g["solver"], fn)(g["sys"])
    return o["atoms"], g["sys"].download()


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _nial_multi():
    al = S.al2009()
    t = S.nialpair()
    return {(0, 0): ("eam", al), (1, 1): ("eam", al), (0, 1): ("pair", t)}, max(al["rcut"], t["rcut"])


def test_pair_single_fp64_matches_oracle():
    t = S.nialpair()
    atoms, box = _fcc(5, 0.405, 1)
    o, g = _build(atoms, box, ("pair", t), t["rcut"])
    ao, ag = _forces_both(o, g)
    assert np.abs(ao["f"]).max() > 1.0
    assert _rel(ag["f"], ao["f"]) < FP64_REL
    assert _rel(ag["Ep"], ao["Ep"]) < FP64_REL
    assert _rel(ag["V"], ao["V"]) < FP64_REL


def test_pair_single_mixed_within_tolerance():
    t = S.nialpair()
    atoms, box = _fcc(6, 0.405, 2)
    o, g = _build(atoms, box, ("pair", t), t["rcut"], precision="mixed")
    ao, _ = _forces_both(o, g)
    fg = g["sys"].forces()
    _, l2 = H.force_error(fg, ao["f"])
    assert l2 < MIXED_L2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multi_eam_with_pair_cross_term(precision):
    pots, rc = _nial_multi()
    atoms, box = _fcc(5, 0.405, 3)
    atoms["kind"] = (np.arange(len(atoms)) % 4 == 0).astype(np.uint16)
    o, g = _build(atoms, box, pots, rc, precision=precision)
    ao, ag = _forces_both(o, g)
    if precision == "fp64":
        assert _rel(ag["f"], ao["f"]) < FP64_REL
        assert _rel(ag["Ep"], ao["Ep"]) < FP64_REL
        assert _rel(ag["Em"], ao["Em"]) < FP64_REL
    else:
        _, l2 = H.force_error(g["sys"].forces(), ao["f"])
        assert l2 < MIXED_L2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multi_eam_with_ljcut_cross_term(precision):
    al = S.al2009()
    lj = (0.5, 0.26, 0.55)
    pots = {(0, 0): ("eam", al), (1, 1): ("eam", al), (0, 1): ("lj", lj)}
    atoms, box = _fcc(5, 0.405, 4)
    atoms["kind"] = (np.arange(len(atoms)) % 2).astype(np.uint16)
    o, g = _build(atoms, box, pots, max(al["rcut"], lj[2]), precision=precision)
    ao, ag = _forces_both(o, g)
    if precision == "fp64":
        assert _rel(ag["f"], ao["f"]) < FP64_REL
    else:
        _, l2 = H.force_error(g["sys"].forces(), ao["f"])
        assert l2 < MIXED_L2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multi_ljcut_with_pair(precision):
    t = S.nialpair()
    lj = (0.5, 0.26, 0.55)
    pots = {(0, 0): ("lj", lj), (1, 1): ("pair", t), (0, 1): ("pair", t)}
    atoms, box = _fcc(5, 0.405, 5)
    atoms["kind"] = (np.arange(len(atoms)) % 3 == 0).astype(np.uint16)
    o, g = _build(atoms, box, pots, t["rcut"], precision=precision)
    ao, ag = _forces_both(o, g)
    if precision == "fp64":
        assert _rel(ag["f"], ao["f"]) < FP64_REL
    else:
        _, l2 = H.force_error(g["sys"].forces(), ao["f"])
        assert l2 < MIXED_L2


LJS = (0.9, 0.26, 0.62)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ljs_single(precision):
    atoms, box = _fcc(6, 0.405, 10)
    o, g = _build(atoms, box, ("ljs", LJS), LJS[2], precision=precision)
    ao, ag = _forces_both(o, g)
    assert np.abs(ao["f"]).max() > 1.0
    if precision == "fp64":
        assert _rel(ag["f"], ao["f"]) < FP64_REL
        assert _rel(ag["Ep"], ao["Ep"]) < FP64_REL
        assert _rel(ag["V"], ao["V"]) < FP64_REL
    else:
        _, l2 = H.force_error(g["sys"].forces(), ao["f"])
        assert l2 < MIXED_L2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_multi_all_four_potential_types(precision):
    """EAM, LJs, Pair and (with three kinds) LJsCut in one Multi solver."""
    al = S.al2009()
    t = S.nialpair()
    pots = {(0, 0): ("eam", al), (1, 1): ("ljs", LJS), (0, 1): ("pair", t)}
    atoms, box = _fcc(5, 0.405, 11)
    atoms["kind"] = (np.arange(len(atoms)) % 3 == 1).astype(np.uint16)
    rc = max(al["rcut"], t["rcut"], LJS[2])
    o, g = _build(atoms, box, pots, rc, precision=precision)
    ao, ag = _forces_both(o, g)
    if precision == "fp64":
        assert _rel(ag["f"], ao["f"]) < FP64_REL
        assert _rel(ag["Ep"], ao["Ep"]) < FP64_REL
    else:
        _, l2 = H.force_error(g["sys"].forces(), ao["f"])
        assert l2 < MIXED_L2
    pots = {(0, 0): ("lj", (0.5, 0.26, 0.55)), (1, 1): ("ljs", LJS), (0, 1): ("pair", t)}
    o, g = _build(atoms, box, pots, t["rcut"], precision=precision)
    ao, ag = _forces_both(o, g)
    if precision == "fp64":
        assert _rel(ag["f"], ao["f"]) < FP64_REL
    else:
        _, l2 = H.force_error(g["sys"].forces(), ao["f"])
        assert l2 < MIXED_L2


def test_multi_atoms_of_unknown_kind_contribute_nothing():
    """Atoms whose kind lies outside [0, nkinds) (undefined in the
    reference) see zero tables on the device: finite forces, no fault."""
    pots, rc = _nial_multi()
    atoms, box = _fcc(4, 0.405, 6)
    atoms["kind"] = np.where(np.arange(len(atoms)) % 5 == 0, 3, 0).astype(np.uint16)
    for precision in ("fp64", "mixed"):
        _, g = _build(atoms, box, pots, rc, precision=precision)
        g["nl"].update(-1.0)
        g["solver"].prepare(g["sys"])
        g["solver"].stages(g["sys"])
        assert np.all(np.isfinite(g["sys"].forces()))


LANGEVIN = dict(beta=0.5, temperature=300.0, time_step=0.004, heat_x=1, heat_y=1, heat_z=0, Ux=0.05,
                xmin=-0.6, xmax=0.7, seed=1234)


def test_langevin_fp64_steps_match_oracle():
    """The reference driver's start (prepare, forces, virials) and make_step
    with a Langevin thermostat: same Philox draws on both sides."""
    t = S.nialpair()
    atoms, box = _fcc(5, 0.405, 7)
    o, g = _build(atoms, box, ("pair", t), t["rcut"], thermo=[LANGEVIN])
    _forces_both(o, g)
    ao, ag = o["atoms"], g["sys"].download()
    assert _rel(ag["f"], ao["f"]) < FP64_REL
    stepper = mdg.Verlet(g["solver"])
    for step in range(20):
        o["solver"].make_step(o["atoms"], o["nl"], 0.002)
        stepper.make_step(g["sys"], 0.002)
        if o["nl"].decide():
            o["nl"].update(-1.0)
        if g["nl"].decide():
            g["nl"].update(-1.0)
    ag = g["sys"].download()
    assert o["solver"].thermo_calls() == g["sys"].thermo_calls() == 21
    assert _rel(ag["r"], o["atoms"]["r"]) < FP64_REL
    assert _rel(ag["v"], o["atoms"]["v"]) < 1e-8


def test_langevin_graph_loop_equals_stepwise():
    """mdg_run (one graph per batch of steps) draws the same numbers as
    make_step called step by step."""
    t = S.nialpair()
    atoms, box = _fcc(5, 0.405, 8)
    out = []
    for mode in ("step", "run"):
        _, g = _build(atoms, box, ("pair", t), t["rcut"], thermo=[LANGEVIN, dict(LANGEVIN, seed=7, heat_z=1)])
        g["nl"].update(-1.0)
        st = mdg.Verlet(g["solver"])
        if mode == "step":
            for _ in range(30):
                st.make_step(g["sys"], 0.002)
                if g["nl"].decide():
                    g["nl"].update(-1.0)
        else:
            st.run(g["sys"], 0.002, 30)
        out.append((g["sys"].download(), g["sys"].thermo_calls()))
    assert out[0][1] == out[1][1] == 30
    assert np.array_equal(out[0][0]["r"], out[1][0]["r"])
    assert np.array_equal(out[0][0]["v"], out[1][0]["v"])


def test_langevin_mixed_tracks_fp64_and_changes_with_parameters():
    t = S.nialpair()
    atoms, box = _fcc(5, 0.405, 9)
    res = {}
    for prec in ("fp64", "mixed"):
        _, g = _build(atoms, box, ("pair", t), t["rcut"], precision=prec, thermo=[LANGEVIN])
        g["nl"].update(-1.0)
        mdg.Verlet(g["solver"]).run(g["sys"], 0.002, 10)
        res[prec] = g["sys"].download()
    d = np.abs(res["mixed"]["r"] - res["fp64"]["r"]).max()
    assert d < 1e-6
    # a parameter change reaches the device without rebuilding anything
    lg = mdg.Langevin(**dict(LANGEVIN, temperature=0.0))
    _, g = _build(atoms, box, ("pair", t), t["rcut"])
    g["solver"].set_thermostat(lg)
    g["nl"].update(-1.0)
    st = mdg.Verlet(g["solver"])
    st.run(g["sys"], 0.002, 5)
    r_cold = g["sys"].positions()
    lg.set_temperature(3000.0)
    st.run(g["sys"], 0.002, 5)
    assert lg.temperature() == 3000.0
    assert not np.array_equal(r_cold, g["sys"].positions())


def test_multi_mixed_step_loop_equals_stepwise():
    """A mixed Multi with EAM, LJs and Pair terms: mdg_run's graph (whose force
    pass starts the next step, taking the band pairs' cut decisions of every
    potential type from the density pass) gives the bits of the stepwise API
    (make_step, decide, update), rebuilds included."""
    al = S.al2009()
    t = S.nialpair()
    pots = {(0, 0): ("eam", al), (1, 1): ("ljs", LJS), (0, 1): ("pair", t)}
    atoms, box = _fcc(5, 0.405, 13)
    atoms["kind"] = (np.arange(len(atoms)) % 3 == 1).astype(np.uint16)
    atoms["v"] *= 3.0
    rc = max(al["rcut"], t["rcut"], LJS[2])
    runs = []
    for stepwise in (False, True):
        _, g = _build(atoms, box, pots, rc, precision="mixed")
        g["nl"].update(-1.0)
        g["solver"].prepare(g["sys"])
        g["solver"].stages(g["sys"])
        st = mdg.Verlet(g["solver"])
        rb0 = g["nl"].rebuilds()
        if stepwise:
            for _ in range(30):
                st.make_step(g["sys"], 0.002)
                if g["nl"].decide():
                    g["nl"].update(-1.0)
        else:
            st.run(g["sys"], 0.002, 30)
        runs.append((g["sys"].download(), g["nl"].rebuilds() - rb0))
    (a, ra), (b, rb) = runs
    assert ra == rb and ra >= 1
    assert np.array_equal(a["r"], b["r"])
    assert np.array_equal(a["v"], b["v"])
    assert np.array_equal(a["f"], b["f"])
