"""Per-atom outputs after steps, as the reference leaves them: each step's
prepare (mdcraft/solver/single.cxx:38-53, multi.cxx:51-63) clears Ep and V
(and Em, nc for EAM and for every Multi), and nothing but virials() writes
them again; LJ Single leaves Em alone. Full atom records after steps without
a virial pass must match the oracle's."""
import numpy as np
import pytest

import mdcraft_gb300 as mdg
from mdcraft_gb300 import workloads as W
from oracle import mdref as R
from tests import gpu_helpers as H
from tests import mdsupport as S

pytestmark = pytest.mark.gpu


def _compare_after_steps(o, g, prec_tol):
    o["nl"].update(-1.0)
    g["nl"].update(-1.0)
    o["solver"].prepare(o["atoms"])
    o["solver"].stages(o["atoms"], o["nl"])
    o["solver"].virials(o["atoms"], o["nl"])
    g["solver"].prepare(g["sys"])
    g["solver"].stages(g["sys"])
    g["solver"].virials(g["sys"])
    assert np.abs(g["sys"].download()["Ep"]).max() > 0.0
    st = mdg.Verlet(g["solver"])
    for _ in range(3):
        o["solver"].make_step(o["atoms"], o["nl"], 0.001)
        st.make_step(g["sys"], 0.001)
    ao, ag = o["atoms"], g["sys"].download()
    for f in ("Ep", "Em", "V"):
        assert np.array_equal(ag[f], ao[f]), f
    np.testing.assert_allclose(ag["nc"], ao["nc"], rtol=prec_tol, atol=0.0)
    m = g["sys"].measure()
    assert m["Ep"] == 0.0 and m["virial"] == 0.0


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_eam_outputs_after_steps(prec):
    atoms, box, per, p = W.eam_cu_fcc(ncell=6)
    o, g = H.make_pair(atoms, box, (1, 1, 1), p, precision=prec)
    _compare_after_steps(o, g, 1e-10 if prec == "fp64" else 1e-5)


def test_lj_single_keeps_em():
    atoms, box, per, p = W.lj_argon_fcc(jitter=0.01)
    atoms["Em"] = 7.0
    o, g = H.make_pair(atoms, box, (1, 1, 1), p, precision="fp64")
    _compare_after_steps(o, g, 0.0)
    assert np.all(g["sys"].download()["Em"] == 7.0)


def test_multi_lj_clears_em_and_nc():
    atoms, box, per, p = W.lj_argon_fcc(jitter=0.01)
    atoms["Em"] = 7.0
    atoms["nc"] = 3.0
    atoms["kind"] = (np.arange(len(atoms)) % 2).astype(np.uint16)
    lj = (p["a"], p["s"], p["rcut"])
    do, dg = H.domains(box, (1, 1, 1))
    atoms["rcut"] = p["rcut"]
    ao = H.to_oracle_atoms(atoms)
    so = R.Solver(None, periodic=do, threads=R.hardware_threads(), nkinds=2)
    sg = mdg.Multi(2, periodic=True)
    keep = []
    for (i, j) in ((0, 0), (1, 1), (0, 1)):
        po, pg = R.LJsCut(*lj), mdg.LJsCut(*lj)
        so.add_potential(i, j, po)
        sg.add_potential(i, j, pg)
        keep.append((po, pg))
    sysg = mdg.System(H.ctx(), dg, atoms)
    o = dict(atoms=ao, nl=R.VerletList(ao, do, threads=R.hardware_threads()), solver=so)
    g = dict(sys=sysg, nl=mdg.VerletList(sysg), solver=sg)
    _compare_after_steps(o, g, 0.0)
    d = g["sys"].download()
    assert np.all(d["Em"] == 0.0) and np.all(d["nc"] == 0.0)
