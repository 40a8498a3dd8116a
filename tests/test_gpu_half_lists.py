"""Half Verlet lists (mdcraft/neibs/verlet-list.cxx:345) in the FP64 form
against the oracle: pair-type potentials push each pair's force, energy and
virial onto both atoms (LJs-cut.cxx:57-62, pair.cxx:387-420, LJs.cxx:196-256);
EAM uses the atom's half alone, as EAM::force/virial do; the Periodic ghost
pass acts on the atom alone. The GPU sums both sides with atomics, so the
bar is 1e-10 relative, not bit equality. The mixed form refuses half lists."""
import numpy as np
import pytest

import mdcraft_gb300 as mdg
from oracle import mdref as R
from tests import gpu_helpers as H
from tests import mdsupport as S

pytestmark = pytest.mark.gpu

REL = 1e-10


def _atoms(n, a, seed, periodic):
    atoms, box = S.make_fcc_bulk(n, n, n, a, 26.9815, mdg.ATOM_DTYPE)
    rng = np.random.default_rng(seed)
    atoms["r"] += rng.normal(0.0, 0.02 * a, size=(len(atoms), 3))
    atoms["v"] = rng.normal(0.0, 0.3, size=(len(atoms), 3))
    if not periodic:
        lo, hi = box[0::2], box[1::2]
        box = (lo[0] - 0.5, hi[0] + 0.5, lo[1] - 0.5, hi[1] + 0.5, lo[2] - 0.5, hi[2] + 0.5)
    return atoms, box


def _pots(kind):
    t = S.nialpair()
    al = S.al2009()
    if kind == "ljcut":
        return (R.LJsCut(0.5, 0.26, 0.55), mdg.LJsCut(0.5, 0.26, 0.55)), 0.55
    if kind == "ljs":
        return (R.LJs(0.9, 0.26, 0.62), mdg.LJs(0.9, 0.26, 0.62)), 0.62
    if kind == "pair":
        return (R.Pair(t["rcut"], t["Vpar"], t["Nr1"], t["dr"]), mdg.Pair(t["rcut"], t["Vpar"], t["Nr1"], t["dr"])), t["rcut"]
    args = (al["rcut"], al["Femb"], al["Rho"], al["Vpar"], al["Nr1"], al["dr"], al["Nrh1"], al["drh"])
    return (R.EAM(*args), mdg.EAM(*args)), al["rcut"]


def _setup(kind, periodic):
    (po, pg), rc = _pots(kind)
    atoms, box = _atoms(5, 0.405, 3, periodic)
    atoms["rcut"] = rc
    atoms["rns"] = rc + 0.05
    per = (1, 1, 1) if periodic else (0, 0, 0)
    do, dg = H.domains(box, per)
    ao = H.to_oracle_atoms(atoms)
    so = R.Solver(po, periodic=do if periodic else None, threads=1)
    sg = mdg.Single(pg, periodic=periodic, precision="fp64")
    nlo = R.VerletList(ao, do, threads=1, half=True)
    sysg = mdg.System(H.ctx(), dg, atoms)
    nlg = mdg.VerletList(sysg, half=True)
    return dict(atoms=ao, nl=nlo, solver=so, keep=po), dict(sys=sysg, nl=nlg, solver=sg, keep=pg)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("periodic", [False, True], ids=["open", "periodic"])
@pytest.mark.parametrize("kind", ["ljcut", "ljs", "pair", "eam"])
def test_half_list_forces_energies_virials(kind, periodic):
    o, g = _setup(kind, periodic)
    o["nl"].update(-1.0)
    g["nl"].update(-1.0)
    o["solver"].prepare(o["atoms"])
    o["solver"].stages(o["atoms"], o["nl"])
    o["solver"].virials(o["atoms"], o["nl"])
    g["solver"].prepare(g["sys"])
    g["solver"].stages(g["sys"])
    g["solver"].virials(g["sys"])
    ao, ag = o["atoms"], g["sys"].download()
    assert np.abs(ao["f"]).max() > 0.1
    assert _rel(ag["f"], ao["f"]) < REL
    assert _rel(ag["Ep"], ao["Ep"]) < REL
    assert _rel(ag["V"], ao["V"]) < REL
    if kind == "eam":
        assert _rel(ag["Em"], ao["Em"]) < REL


@pytest.mark.parametrize("kind", ["ljcut", "pair"])
def test_half_list_steps(kind):
    o, g = _setup(kind, True)
    o["nl"].update(-1.0)
    g["nl"].update(-1.0)
    o["solver"].prepare(o["atoms"])
    o["solver"].stages(o["atoms"], o["nl"])
    g["solver"].prepare(g["sys"])
    g["solver"].stages(g["sys"])
    mdg.Verlet(g["solver"]).run(g["sys"], 0.002, 30)
    for _ in range(30):
        o["solver"].make_step(o["atoms"], o["nl"], 0.002)
        if o["nl"].decide():
            o["nl"].update(-1.0)
    ag = g["sys"].download()
    assert _rel(ag["r"], o["atoms"]["r"]) < 1e-9
    assert _rel(ag["f"], o["atoms"]["f"]) < 1e-8


def test_mixed_form_refuses_half_lists():
    o, g = _setup("ljcut", True)
    g["nl"].update(-1.0)
    g["solver"].set_precision("mixed")
    with pytest.raises(mdg.MDGError):
        g["solver"].stages(g["sys"])
