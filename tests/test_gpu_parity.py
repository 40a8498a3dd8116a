"""GPU parity tests through the C-ABI (libmdg via mdcraft_gb300) against the
CPU oracle and the reference's own golden values.

Bars: neighbour sets bit-identical (sorted per atom, self included); FP64
forces/energies within 1e-10 relative; mixed-precision forces within
||dF||_2/||F||_2 <= 1e-5 of the FP64 oracle."""
import numpy as np
import pytest

import mdcraft_gb300 as mdg
from mdcraft_gb300 import workloads as W
from oracle import mdref as R
from tests import gpu_helpers as H
from tests import mdsupport as S

pytestmark = pytest.mark.gpu

FP64_REL = 1e-10
MIXED_L2 = 1e-5


def _small(atoms, keep):
    return atoms[keep].copy()


# ---- reference known answers: test/cxx/neibs/test_verlet_list.cxx ----------
def _mk(rows):
    a = W.new_atoms(len(rows))
    for i, row in enumerate(rows):
        a["r"][i] = row[:3]
        a["rns"][i] = row[3]
        a["rcut"][i] = row[4] if len(row) > 4 else row[3]
        a["m"][i] = 1.0
    return a


def _sys(atoms, box, periodic=(0, 0, 0), half=False):
    dg = mdg.Domain(*box)
    for k in range(3):
        if periodic[k]:
            dg.set_periodic(k, True)
    s = mdg.System(H.ctx(), dg, atoms)
    return s, mdg.VerletList(s, half=half)


def test_known_answers_verlet_list():
    s, nl = _sys(_mk([(0.20, 0, 0, 0.8), (0.85, 0, 0, 0.8), (2.50, 0, 0, 0.8)]), (0.0, 3.0, -1.0, 1.0, -1.0, 1.0))
    nl.update(-1.0)
    L = nl.lists()
    assert [len(x) for x in L] == [2, 2, 1] and list(L[0]) == [0, 1] and list(L[2]) == [2]

    s, nl = _sys(_mk([(-0.48, 0, 0, 0.10), (0.48, 0, 0, 0.10)]), (-0.5, 0.5, -0.5, 0.5, -0.5, 0.5), (1, 0, 0))
    nl.update(-1.0)
    assert [list(x) for x in nl.lists()] == [[0, 1], [0, 1]]

    s, nl = _sys(_mk([(0.15, .1, .1, .4, .4), (0.55, .1, .1, .4, .4), (1.60, .1, .1, .4, .4)]),
                 (0.0, 2.0, 0.0, 1.0, 0.0, 1.0))
    nl.update(-1.0)
    assert list(nl.list_for([0.40, 0.10, 0.10])) == [0, 1]

    atoms = _mk([(0.10, .1, .1, 0.35, 0.20), (0.35, .1, .1, 0.35, 0.60), (1.80, .1, .1, 0.35, 0.10)])
    s, nl = _sys(atoms, (0.0, 2.0, 0.0, 1.0, 0.0, 1.0))
    nl.update(-1.0)
    nl.update(2.0)
    rns = s.download()["rns"]
    assert rns == pytest.approx([1.60, 2.40, 0.40], abs=1e-12)

    s, nl = _sys(_mk([(0.10, .1, .1, 0.35), (0.32, .1, .1, 0.35), (0.95, .1, .1, 0.35)]),
                 (0.0, 2.0, 0.0, 1.0, 0.0, 1.0), half=True)
    nl.update(-1.0)
    assert [list(x) for x in nl.lists()] == [[0, 1], [1], [2]]

    atoms = _mk([(0.10, .1, .1, 0.80, 0.60), (0.50, .1, .1, 0.80, 0.60)])
    atoms["uid"] = [1, 2]
    s, nl = _sys(atoms, (0.0, 2.0, 0.0, 1.0, 0.0, 1.0), half=True)
    nl.update(-1.0)
    r = s.positions()
    r[0, 0] += 0.09
    s.set_positions(r)
    assert not nl.decide()
    r[0, 0] += 0.02
    s.set_positions(r)
    assert nl.decide()


def test_grid_matches_oracle():
    d = (0.0, 4.0, 0.0, 4.0, 0.0, 4.0)
    atoms = _mk([(0.2, 0.2, 0.2, 1.0), (1.8, 1.1, 0.7, 1.0), (2.6, 1.9, 0.8, 1.0)])
    s, nl = _sys(atoms, d)
    nl.update(-1.0)
    g = nl.grid()
    og = R.Grid(R.Domain(*d))
    og.build(H.to_oracle_atoms(atoms))
    f = og.fields
    assert list(g["num_cells"]) == list(f["num_cells"]) and int(np.prod(g["num_cells"])) == 6
    assert list(g["grid_offset"]) == list(f["grid_offset"])
    assert np.array_equal(g["cell_sizes"], f["cell_sizes"])


# ---- test/cxx/solver/test_ljs_cut.cxx ---------------------------------------
EPS, SIG, RC = 1.03120074782442750, 0.33841043857528683, 0.8125


def test_lj_pair_analytic():
    atoms = W.new_atoms(2)
    atoms["r"][1, 0] = 0.40
    atoms["rcut"] = RC
    atoms["rns"] = 0.5
    atoms["m"] = 1.0
    s, nl = _sys(atoms, (-1.0, 1.0, -1.0, 1.0, -1.0, 1.0))
    nl.update(-1.0)
    pot = mdg.LJsCut(EPS, SIG, RC)
    sol = mdg.Single(pot)
    assert sol.num_stages() == 1
    sol.prepare(s)
    sol.stages(s)
    sol.virials(s)
    a = s.download()
    r2inv = 1.0 / 0.16
    r6 = r2inv ** 3
    s6 = SIG ** 6
    fx = -0.5 * (48.0 * EPS * s6) * ((2.0 * s6) * r6 - 1.0) * r6 * r2inv * 0.40
    sr6 = (SIG / 0.40) ** 6
    assert a["f"][0, 0] == pytest.approx(fx, abs=1e-12)
    assert a["f"][1, 0] == pytest.approx(-fx, abs=1e-12)
    assert a["Ep"].sum() == pytest.approx(4.0 * EPS * sr6 * (sr6 - 1.0), abs=1e-12)
    assert (a["V"][:, 0] + a["V"][:, 4] + a["V"][:, 8]).sum() == pytest.approx(fx * 0.40, abs=1e-12)
    assert a["rcut"][0] == RC


# ---- golden: test/cxx/solver/test_argon_ball_md.cxx -------------------------
def _gpu_run_md_steps(sol, s, nl, dt, steps, interval):
    st = mdg.Verlet(sol)

    def state():
        sol.prepare(s)
        sol.stages(s)
        sol.virials(s)
        return s.measure()

    nl.update(-1.0)
    hist = [state()]
    for k in range(1, steps + 1):
        st.make_step(s, dt)
        if interval > 0 and k % interval == 0:
            nl.update(-1.0)
        hist.append(state())
    return hist


def test_argon_ball_golden_fp64():
    atoms, box = S.argon_ball(mdg.ATOM_DTYPE)
    pot = mdg.LJsCut(EPS, SIG, RC)
    S.set_common_atom_properties(atoms, 40.0, pot.rcut(), 10.125 / 8.125)
    atoms["v"] = 0.0
    s, nl = _sys(atoms, box)
    sol = mdg.Single(pot)
    hist = _gpu_run_md_steps(sol, s, nl, 4e-3, 2, 1)
    assert hist[2]["Ep"] == pytest.approx(-1.0244383150033894e06, abs=1e-3)
    assert hist[2]["virial"] == pytest.approx(-1.1164231473675424e05, abs=1e-3)
    assert hist[2]["Etot"] == pytest.approx(hist[0]["Etot"], abs=2.0)
    a = s.download()
    a1 = int(np.nonzero(a["uid"] == 1)[0][0])
    a2 = int(np.nonzero(a["uid"] == 2)[0][0])
    tr = lambda k: a["V"][k, 0] + a["V"][k, 4] + a["V"][k, 8]
    assert a["r"][a1] == pytest.approx([-3.9184367989026225, 2.6440651643797461, 5.2690712254285517], abs=1e-12)
    assert a["v"][a1, 2] == pytest.approx(5.79013209455442e-04, abs=1e-15)
    assert a["f"][a1, 2] == pytest.approx(2.8929546164515996, abs=1e-12)
    assert a["Ep"][a1] == pytest.approx(-4.0629298955784474, abs=1e-12)
    assert tr(a1) == pytest.approx(-3.3178872346261723e-01, abs=1e-12)
    assert a["r"][a2, 2] == pytest.approx(5.7940689066038047, abs=1e-12)
    assert a["v"][a2, 0] == pytest.approx(-1.4268458571713898e-03, abs=1e-15)
    assert a["f"][a2, 0] == pytest.approx(-7.1268568973069453, abs=1e-12)
    assert a["Ep"][a2] == pytest.approx(-4.2002585997144832, abs=1e-12)
    assert tr(a2) == pytest.approx(4.2842826328841377e-01, abs=1e-12)


# ---- golden: test/cxx/solver/test_aluminum_bulk_eam.cxx ---------------------
def _al():
    t = S.al2009()
    pot = mdg.EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
    atoms, box = S.make_fcc_bulk(3, 3, 3, 0.4032, 26.9815384, mdg.ATOM_DTYPE)
    S.set_common_atom_properties(atoms, 26.9815384, pot.rcut(), 1.25)
    S.assign_deterministic_velocities(atoms, 5.0e-3)
    s, nl = _sys(atoms, box, (1, 1, 1))
    return pot, s, nl, mdg.Single(pot, periodic=True)


def test_al_eam_golden_fp64():
    pot, s, nl, sol = _al()
    assert sol.num_stages() == 2
    hist = _gpu_run_md_steps(sol, s, nl, 4e-3, 2, 1)
    h = hist[-1]
    assert h["Etot"] == pytest.approx(-3.4489006959225437e04, abs=1e-6)
    assert h["Ep"] == pytest.approx(-6.7190981865001777e03, abs=1e-6)
    assert h["Em"] == pytest.approx(-2.7770493824864527e04, abs=1e-6)
    assert h["KE"] == pytest.approx(5.8505213926282473e-01, abs=1e-9)
    assert h["virial"] == pytest.approx(7.4272691119381875e01, abs=1e-9)
    a = s.download()
    assert a["r"][0] == pytest.approx([6.0469801558679681e-01, 6.0474258946107018e-01, 6.0477602485847293e-01],
                                      abs=1e-12)
    assert a["v"][0, 0] == pytest.approx(-1.3221213313405629e-02, abs=1e-15)
    assert a["f"][0, 0] == pytest.approx(-1.1358391912725722e01, abs=1e-12)
    assert a["Ep"][0] == pytest.approx(-6.3230321656455359e01, abs=1e-9)
    assert a["Em"][0] == pytest.approx(-2.5721082474679707e02, abs=1e-9)
    assert a["V"][0, 0] + a["V"][0, 4] + a["V"][0, 8] == pytest.approx(1.3557390418206403e01, abs=1e-9)
    assert len(nl.lists()[0]) > 12


def test_al_eam_energy_conservation():
    pot, s, nl, sol = _al()
    hist = _gpu_run_md_steps(sol, s, nl, 4e-3, 5, 1)
    assert hist[-1]["Etot"] == pytest.approx(hist[0]["Etot"], abs=40.0)
    assert np.linalg.norm(hist[-1]["vcom"]) < 1e-12


# ---- neighbour sets vs the oracle on the benchmark geometries --------------
def _cases():
    cases = []
    atoms, box, per, p = W.lj_argon_fcc()
    cases.append(("lj_argon_4000", atoms, box, (1, 1, 1), p))
    atoms, box, per, p = W.eam_cu_fcc(ncell=12)
    cases.append(("eam_cu_6912", atoms, box, (1, 1, 1), p))
    atoms, box, per, p = W.eam_nial_b2(ncell=10)
    cases.append(("nial_b2_2000", atoms, box, (1, 1, 1), p))
    atoms, box, per, p = W.eam_cu_fcc(ncell=4)  # 2 cells per axis: n=2 rules
    cases.append(("eam_cu_small_256", atoms, box, (1, 1, 1), p))
    # 3 cells per periodic axis (the warp build with cell images)
    atoms, box, per, p = W.eam_cu_fcc(ncell=6, T=900.0, jitter=0.03)
    cases.append(("eam_cu_3cells_864", atoms, box, (1, 1, 1), p))
    atoms, box, per, p = W.eam_nial_b2(ncell=8)
    cases.append(("nial_b2_3cells_1024", atoms, box, (1, 1, 1), p))
    rng = np.random.default_rng(7)
    g = W.new_atoms(3000)
    g["r"] = rng.random((3000, 3)) * 6.0
    g["rns"] = 0.35 + 0.15 * rng.random(3000)
    g["rcut"] = 0.3
    g["m"] = 1.0
    g["uid"] = np.arange(1, 3001)
    cases.append(("gas_mixed_rns_open", g, (0.0, 6.0, 0.0, 6.0, 0.0, 6.0), (0, 0, 0), None))
    g2 = g.copy()
    g2["r"][:, 2] = 0.0
    cases.append(("gas_2d_periodic_x", g2, (0.0, 6.0, 0.0, 6.0, 0.0, 0.0), (1, 0, 0), None))
    # one periodic axis of 3 cells with rns equal to a third of it, open axes
    g3 = g.copy()
    g3["r"][:, 0] = rng.random(3000) * 1.5
    g3["rns"] = 0.5
    cases.append(("gas_3cells_periodic_x_rns_third", g3, (0.0, 1.5, 0.0, 6.0, 0.0, 6.0), (1, 0, 0), None))
    # atoms on cell faces: integer sites of a box of 6 unit cells per axis
    # (cs = 1 = rns exactly, so neighbours sit at exactly rns) and the same
    # sites one ulp to either side (below 0 they wrap to just under 6)
    k = np.arange(6.0)
    site = np.stack(np.meshgrid(k, k, k, indexing="ij"), -1).reshape(-1, 3)
    faces = np.concatenate([site, np.nextafter(site, np.inf), np.nextafter(site, -np.inf)])
    g4 = W.new_atoms(len(faces))
    g4["r"] = faces
    g4["rns"] = 1.0
    g4["rcut"] = 0.9
    g4["m"] = 1.0
    g4["uid"] = np.arange(1, len(faces) + 1)
    cases.append(("faces_exact_6cells", g4, (0.0, 6.0, 0.0, 6.0, 0.0, 6.0), (1, 1, 1), None))
    # one cell per periodic axis (L < 2 rns): every pair by its nearest image
    g5 = W.new_atoms(60)
    g5["r"] = rng.random((60, 3)) * 1.5
    g5["rns"] = 1.0
    g5["rcut"] = 0.8
    g5["m"] = 1.0
    g5["uid"] = np.arange(1, 61)
    cases.append(("gas_1cell_periodic", g5, (0.0, 1.5, 0.0, 1.5, 0.0, 1.5), (1, 1, 1), None))
    return cases


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[0])
def test_neighbour_sets_bit_identical(case):
    name, atoms, box, per, _ = case
    _sets_match_oracle(atoms, box, per)


def _sets_match_oracle(atoms, box, per):
    do, dg = H.domains(box, per)
    ao = H.to_oracle_atoms(atoms)
    nlo = R.VerletList(ao, do, threads=R.hardware_threads())
    nlo.update(-1.0)
    s = mdg.System(H.ctx(), dg, atoms)
    nlg = mdg.VerletList(s)
    nlg.update(-1.0)
    assert H.same_sets(nlo.lists(), nlg.lists()) == 0
    # wrapped positions identical too (fit_in_period at the rebuild)
    assert np.array_equal(s.positions(), ao["r"])
    # every listed pair's image within one cell (the mixed pair vectors)
    assert not s.flags() & 16


def test_half_list_matches_oracle():
    atoms, box, per, p = W.eam_cu_fcc(ncell=6)
    do, dg = H.domains(box, (1, 1, 1))
    ao = H.to_oracle_atoms(atoms)
    nlo = R.VerletList(ao, do, threads=1, half=True)
    nlo.update(-1.0)
    s = mdg.System(H.ctx(), dg, atoms)
    nlg = mdg.VerletList(s, half=True)
    nlg.update(-1.0)
    assert H.same_sets(nlo.lists(), nlg.lists()) == 0


# ---- forces / energies ------------------------------------------------------
def _slab(made, keep_below, z_lo, z_hi):
    """A slab of a periodic workload: periodic in x and y, open in z, the
    atoms below keep_below·L kept, the domain's z extent [z_lo, z_hi]·L.
    Atoms above z_hi·L lie outside the domain on the open axis (binned into
    the top cell, their lists walked from the cell above it); atoms below
    z_lo·L extend the grid below the domain (a negative grid offset)."""
    atoms, box, _, p = made
    L = box[1] - box[0]
    a = atoms[atoms["r"][:, 2] < box[4] + keep_below * L].copy()
    return a, (box[0], box[1], box[2], box[3], box[4] + z_lo * L, box[4] + z_hi * L), (1, 1, 0), p


def _cluster(made, radius):
    """A sphere of radius·L cut from a periodic workload, in an open box."""
    atoms, box, _, p = made
    L = box[1] - box[0]
    c = np.array([box[0], box[2], box[4]]) + 0.5 * L
    a = atoms[np.linalg.norm(atoms["r"] - c, axis=1) < radius * L].copy()
    return a, box, (0, 0, 0), p


def _axes(per):
    return (1, 1, 1) if per is True else per


FORCE_CASES = [
    ("lj_argon", lambda: W.lj_argon_fcc(jitter=0.01)),
    ("eam_cu", lambda: W.eam_cu_fcc(ncell=10)),
    ("nial_multi", lambda: W.eam_nial_b2(ncell=8)),
    # 2 cells per periodic axis (the per-atom list build with its minimum
    # image), box edges still above 2 rns
    ("eam_cu_2cells", lambda: W.eam_cu_fcc(ncell=4)),
    ("lj_argon_2cells", lambda: W.lj_argon_fcc(ncell=4, jitter=0.01)),
    # free surfaces on an open axis, with atoms outside the domain on both
    # sides of it (2,400 atoms, 200 above the domain's top)
    ("eam_cu_slab", lambda: _slab(W.eam_cu_fcc(ncell=10), 0.6, 0.05, 0.55)),
    ("lj_argon_slab", lambda: _slab(W.lj_argon_fcc(jitter=0.01), 0.6, 0.0, 0.55)),
    # Multi: 3 periodic cells per axis in x and y, one open cell in z
    ("nial_slab", lambda: _slab(W.eam_nial_b2(ncell=8), 0.6, 0.0, 0.55)),
    # a 1,088-atom Cu nanoparticle in an open box
    ("eam_cu_cluster", lambda: _cluster(W.eam_cu_fcc(ncell=10), 0.4)),
]


@pytest.mark.parametrize("case", [c for c in FORCE_CASES if c[0].endswith(("_slab", "_cluster"))],
                         ids=lambda c: c[0])
def test_neighbour_sets_bit_identical_open_axis(case):
    atoms, box, per, _ = case[1]()
    _sets_match_oracle(atoms, box, per)


@pytest.mark.parametrize("case", FORCE_CASES, ids=lambda c: c[0])
def test_fp64_forces_energies_match_oracle(case):
    atoms, box, per, p = case[1]()
    o, g = H.make_pair(atoms, box, _axes(per), p, precision="fp64")
    o["nl"].update(-1.0)
    g["nl"].update(-1.0)
    for so, ao, nl in [(o["solver"], o["atoms"], o["nl"])]:
        so.prepare(ao)
        so.stages(ao, nl)
        so.virials(ao, nl)
    g["solver"].prepare(g["sys"])
    g["solver"].stages(g["sys"])
    g["solver"].virials(g["sys"])
    a = g["sys"].download()
    fo = o["atoms"]["f"]
    scale = np.sqrt(np.mean(np.sum(fo ** 2, axis=1)))
    # per-atom sums of ~50-80 pair terms in another order: relative to the RMS force
    assert np.max(np.abs(a["f"] - fo)) <= FP64_REL * scale
    for key in ("Ep", "Em", "nc"):
        ref = o["atoms"][key]
        assert np.max(np.abs(a[key] - ref)) <= FP64_REL * max(np.max(np.abs(ref)), 1e-300)
    vs = np.max(np.abs(o["atoms"]["V"]))
    assert np.max(np.abs(a["V"] - o["atoms"]["V"])) <= FP64_REL * vs
    mo = R.measure_state(o["atoms"])
    mg = g["sys"].measure()
    for key in ("Ep", "Em", "KE", "virial"):
        assert mg[key] == pytest.approx(mo[key], rel=FP64_REL, abs=1e-300)


def test_box_below_two_rns_fp64_follows_ghost_pass_mixed_refused():
    """A periodic box shorter than 2 rns (LJ argon, 3 fcc cells per axis:
    1.58 nm against rns 0.88 nm). The FP64 form follows the reference's
    Periodic ghost pass, so its forces match the oracle's; the mixed form,
    whose minimum images equal that pass only for edges of at least 2 rns,
    refuses the box."""
    atoms, box, per, p = W.lj_argon_fcc(ncell=3, jitter=0.01)
    assert box[1] - box[0] < 2.0 * float(atoms["rns"][0])
    o, g = H.make_pair(atoms, box, (1, 1, 1), p, precision="fp64")
    o["nl"].update(-1.0)
    g["nl"].update(-1.0)
    o["solver"].prepare(o["atoms"])
    o["solver"].stages(o["atoms"], o["nl"])
    g["solver"].prepare(g["sys"])
    g["solver"].stages(g["sys"])
    fo = o["atoms"]["f"]
    fg = g["sys"].download()["f"]
    scale = np.sqrt(np.mean(np.sum(fo ** 2, axis=1)))
    assert scale > 0.0
    assert np.max(np.abs(fg - fo)) <= FP64_REL * scale
    _, gm = H.make_pair(atoms, box, (1, 1, 1), p, precision="mixed")
    gm["nl"].update(-1.0)
    with pytest.raises(RuntimeError, match="2 rns"):
        gm["solver"].prepare(gm["sys"])
        gm["solver"].stages(gm["sys"])


@pytest.mark.parametrize("case", FORCE_CASES, ids=lambda c: c[0])
def test_mixed_forces_within_tolerance(case):
    atoms, box, per, p = case[1]()
    o, g = H.make_pair(atoms, box, _axes(per), p, precision="mixed")
    o["nl"].update(-1.0)
    g["nl"].update(-1.0)
    o["solver"].prepare(o["atoms"])
    o["solver"].stages(o["atoms"], o["nl"])
    g["solver"].prepare(g["sys"])
    g["solver"].stages(g["sys"])
    f = g["sys"].forces()
    emax, el2 = H.force_error(f, o["atoms"]["f"])
    print(f"{case[0]}: mixed force error max/RMS {emax:.3e}  L2 {el2:.3e}")
    assert el2 <= MIXED_L2
    assert emax <= 50 * MIXED_L2


def test_run_loop_fp64_matches_oracle():
    atoms, box, per, p = W.lj_argon_fcc()
    o, g = H.make_pair(atoms, box, (1, 1, 1), p, precision="fp64")
    o["nl"].update(-1.0)
    g["nl"].update(-1.0)
    for so, ao, nl in [(o["solver"], o["atoms"], o["nl"])]:
        so.prepare(ao)
        so.stages(ao, nl)
    g["solver"].prepare(g["sys"])
    g["solver"].stages(g["sys"])
    nsteps = 60
    rb_o = o["solver"].run(o["atoms"], o["nl"], o["dom"], p["dt"], nsteps)
    rb0 = g["nl"].rebuilds()
    g["stepper"].run(g["sys"], p["dt"], nsteps)
    rb_g = g["nl"].rebuilds() - rb0
    a = g["sys"].download()
    assert rb_g == rb_o
    assert np.max(np.abs(a["r"] - o["atoms"]["r"])) < 1e-9
    assert np.max(np.abs(a["v"] - o["atoms"]["v"])) < 1e-9
    assert H.same_sets(o["nl"].lists(), g["nl"].lists()) == 0


@pytest.mark.parametrize("make", [lambda: W.eam_cu_fcc(ncell=8), lambda: W.lj_argon_fcc(jitter=0.01)],
                         ids=["eam_cu", "lj_argon"])
def test_mixed_run_tracks_fp64(make):
    """200 mixed steps against 200 FP64 steps from the same state: the
    energy change and the trajectory agree. (The configured EAM density is
    truncated at rc, so energy is not conserved exactly by either form.)"""
    atoms, box, per, p = make()
    out = {}
    for prec in ("fp64", "mixed"):
        _, g = H.make_pair(atoms, box, (1, 1, 1), p, precision=prec)
        g["nl"].update(-1.0)
        g["solver"].prepare(g["sys"])
        g["solver"].stages(g["sys"])
        g["solver"].virials(g["sys"])
        e0 = g["sys"].measure()["Etot"]
        g["stepper"].run(g["sys"], p["dt"], 200)
        g["solver"].prepare(g["sys"])
        g["solver"].virials(g["sys"])
        e1 = g["sys"].measure()["Etot"]
        out[prec] = (e0, e1, g["sys"].positions(), g["sys"].flags())
    e0, e1, r64, fl64 = out["fp64"]
    m0, m1, rmx, flmx = out["mixed"]
    assert m0 == pytest.approx(e0, rel=1e-12)
    assert abs((m1 - m0) - (e1 - e0)) <= 1e-5 * abs(e0)
    assert np.max(np.abs(rmx - r64)) < 1e-5
    assert fl64 == 0 and flmx == 0


def test_empty_and_single_atom_systems():
    s, nl = _sys(W.new_atoms(0), (0, 1, 0, 1, 0, 1))
    nl.update(-1.0)
    assert nl.decide() is False or nl.decide() is True
    one = _mk([(0.5, 0.5, 0.5, 0.3)])
    s, nl = _sys(one, (0, 1, 0, 1, 0, 1), (1, 1, 1))
    nl.update(-1.0)
    assert [list(x) for x in nl.lists()] == [[0]]


def test_out_of_grid_atom_is_flagged():
    a = _mk([(0.1, 0.1, 0.1, 0.3), (0.5, 0.5, 0.5, 0.3), (3.5, 0.5, 0.5, 0.3)])
    s, nl = _sys(a, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    assert nl.update(-1.0) == -4
    assert s.flags() & 1
