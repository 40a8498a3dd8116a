"""Pins the CPU oracle against the reference's own known answers and golden
values: every assertion of test/cxx/{domain,neibs,solver}/*.cxx, with the
reference's tolerances. CPU only."""
import numpy as np
import pytest

from oracle import mdref as R
from tests import mdsupport as S

DT = R.ATOM_DTYPE


# ---- test/cxx/domain/test_domain.cxx:9-34 --------------------------------
def test_domain_fit_shortest_belong():
    d = R.Domain(-1.0, 1.0, -2.0, 2.0, -3.0, 3.0)
    d.set_periodic(0, True)
    d.set_periodic(1, True)
    p = d.fit_in_period([1.25, -2.25, 0.5])
    assert p[0] == pytest.approx(-0.75, abs=1e-12)
    assert p[1] == pytest.approx(1.75, abs=1e-12)
    assert p[2] == pytest.approx(0.5, abs=1e-12)
    assert d.belong(p)
    s = d.shortest([1.8, -3.5, 0.25])
    assert s[0] == pytest.approx(-0.2, abs=1e-12)
    assert s[1] == pytest.approx(0.5, abs=1e-12)
    assert s[2] == pytest.approx(0.25, abs=1e-12)


def test_domain_nearest_distance():
    d = R.Domain(-1.0, 1.0, -1.0, 1.0, 0.0, 0.0)
    d.set_periodic(0, True)
    assert d.nearest_distance([-0.8, 0.0, 0.0], 0) == 0.19999999999999996 or \
        d.nearest_distance([-0.8, 0.0, 0.0], 0) == pytest.approx(0.2, rel=4 * np.finfo(float).eps)
    assert d.nearest_distance([-0.8, 0.0, 0.0], 1) == np.finfo(np.float64).max


# ---- test/cxx/neibs/test_grid.cxx:38-94 ----------------------------------
def _mk(rows):
    a = S.atom_array(len(rows), DT)
    for i, row in enumerate(rows):
        a["r"][i] = row[:3]
        a["rns"][i] = row[3]
        a["rcut"][i] = row[4] if len(row) > 4 else row[3]
        a["m"][i] = 1.0
    return a


def test_grid_local_subgrid_and_indices():
    d = R.Domain(0.0, 4.0, 0.0, 4.0, 0.0, 4.0)
    atoms = _mk([(0.2, 0.2, 0.2, 1.0), (1.8, 1.1, 0.7, 1.0), (2.6, 1.9, 0.8, 1.0)])
    g = R.Grid(d)
    g.build(atoms)
    assert g.cell_size() == pytest.approx(1.0, abs=1e-12)
    assert g.cells_number() == 6
    idx = [g.local_index3D(atoms["r"][k]) for k in range(3)]
    assert list(idx[0]) == [0, 0, 0]
    assert list(idx[1]) == [1, 1, 0]
    assert list(idx[2]) == [2, 1, 0]
    assert [g.cell_index(i) for i in idx] == [0, 4, 5]


def test_grid_adjacent_cells_periodic_wrap():
    d = R.Domain(-2.0, 2.0, -2.0, 2.0, -2.0, 2.0)
    d.set_periodic(0, True)
    atoms = _mk([(-1.8, 0, 0, 1.0), (-0.2, 0, 0, 1.0), (0.2, 0, 0, 1.0), (1.8, 0, 0, 1.0)])
    g = R.Grid(d)
    g.build(atoms)
    cells, edge = g.adjacent_cells(atoms["r"][0])
    compact = sorted(set(int(c) for c in cells if c != -1))
    assert edge[0]
    assert compact == [0, 1, 3]


# ---- test/cxx/neibs/test_verlet_list.cxx:25-196 --------------------------
def test_verlet_without_periodicity():
    atoms = _mk([(0.20, 0, 0, 0.8), (0.85, 0, 0, 0.8), (2.50, 0, 0, 0.8)])
    d = R.Domain(0.0, 3.0, -1.0, 1.0, -1.0, 1.0)
    nl = R.VerletList(atoms, d, threads=1)
    nl.update(-1.0)
    L = nl.lists()
    assert [len(x) for x in L] == [2, 2, 1]
    assert sorted(L[0]) == [0, 1]
    assert list(L[2]) == [2]


def test_verlet_through_periodic_boundary():
    atoms = _mk([(-0.48, 0, 0, 0.10), (0.48, 0, 0, 0.10)])
    d = R.Domain(-0.5, 0.5, -0.5, 0.5, -0.5, 0.5)
    d.set_periodic(0, True)
    nl = R.VerletList(atoms, d, threads=1)
    nl.update(-1.0)
    L = nl.lists()
    assert sorted(L[0]) == [0, 1]
    assert sorted(L[1]) == [0, 1]


def test_verlet_list_for_query_point():
    atoms = _mk([(0.15, 0.10, 0.10, 0.40, 0.40), (0.55, 0.10, 0.10, 0.40, 0.40),
                 (1.60, 0.10, 0.10, 0.40, 0.40)])
    d = R.Domain(0.0, 2.0, 0.0, 1.0, 0.0, 1.0)
    nl = R.VerletList(atoms, d, threads=1)
    nl.update(-1.0)
    assert sorted(nl.list_for([0.40, 0.10, 0.10])) == [0, 1]


def test_verlet_sort_orders_atoms_by_owning_cell():
    # test/cxx/neibs/test_verlet_list.cxx:107-122
    atoms = _mk([(1.60, 0.10, 0.10, 0.40, 0.40), (0.15, 0.10, 0.10, 0.40, 0.40),
                 (0.95, 0.10, 0.10, 0.40, 0.40)])
    d = R.Domain(0.0, 2.0, 0.0, 1.0, 0.0, 1.0)
    nl = R.VerletList(atoms, d, threads=1)
    out = nl.sort(atoms)
    assert len(out) == 3
    assert out["r"][0][0] < out["r"][1][0] < out["r"][2][0]


def test_sort_wraps_and_orders_by_cell_index():
    """put_atoms_in_cells (verlet-list.cxx:176-199) wraps the caller's atoms;
    the copy is ordered by Grid::cell_index (x fastest), ascending index
    inside a cell."""
    rng = np.random.default_rng(8)
    n = 500
    rows = [(*rng.uniform(-0.5, 3.5, 3), 0.45, 0.4) for _ in range(n)]
    atoms = _mk(rows)
    atoms["uid"] = np.arange(n)
    d = R.Domain(0.0, 3.0, 0.0, 3.0, 0.0, 3.0)
    for k in range(3):
        d.set_periodic(k, True)
    out = R.sort_atoms(d, atoms)
    assert np.all((atoms["r"] >= 0.0) & (atoms["r"] < 3.0))
    g = R.Grid(d)
    g.build(atoms)
    cells = np.array([g.cell_index(g.local_index3D(r)) for r in out["r"]])
    assert np.all(np.diff(cells) >= 0)
    same = np.diff(cells) == 0
    assert np.all(np.diff(out["uid"].astype(np.int64))[same] > 0)
    assert np.array_equal(np.sort(out["uid"]), np.arange(n))
    assert np.array_equal(out.view(np.uint8).reshape(n, -1),
                          atoms[out["uid"]].view(np.uint8).reshape(n, -1))


def test_verlet_kbuf_uses_actual_neighbours():
    atoms = _mk([(0.10, 0.10, 0.10, 0.35, 0.20), (0.35, 0.10, 0.10, 0.35, 0.60),
                 (1.80, 0.10, 0.10, 0.35, 0.10)])
    d = R.Domain(0.0, 2.0, 0.0, 1.0, 0.0, 1.0)
    nl = R.VerletList(atoms, d, threads=1)
    nl.update(-1.0)
    nl.update(2.0)
    assert atoms["rns"][0] == pytest.approx(1.60, abs=1e-12)
    assert atoms["rns"][1] == pytest.approx(2.40, abs=1e-12)
    assert atoms["rns"][2] == pytest.approx(0.40, abs=1e-12)


def test_verlet_half_list_each_pair_once():
    atoms = _mk([(0.10, 0.10, 0.10, 0.35), (0.32, 0.10, 0.10, 0.35), (0.95, 0.10, 0.10, 0.35)])
    d = R.Domain(0.0, 2.0, 0.0, 1.0, 0.0, 1.0)
    nl = R.VerletList(atoms, d, threads=1, half=True)
    nl.update(-1.0)
    L = nl.lists()
    assert [len(x) for x in L] == [2, 1, 1]
    assert sorted(L[0]) == [0, 1] and list(L[1]) == [1] and list(L[2]) == [2]


def test_verlet_decide_half_skin():
    atoms = _mk([(0.10, 0.10, 0.10, 0.80, 0.60), (0.50, 0.10, 0.10, 0.80, 0.60)])
    atoms["uid"] = [1, 2]
    d = R.Domain(0.0, 2.0, 0.0, 1.0, 0.0, 1.0)
    nl = R.VerletList(atoms, d, threads=1, half=True)
    nl.update(-1.0)
    atoms["r"][0, 0] += 0.09
    assert not nl.decide()
    atoms["r"][0, 0] += 0.02
    assert nl.decide()


def test_verlet_half_rejects_thread_pool():
    atoms = _mk([(0.10, 0.10, 0.10, 0.30, 0.20)])
    d = R.Domain(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)
    with pytest.raises(RuntimeError):
        R.VerletList(atoms, d, threads=2, half=True)


# ---- test/cxx/solver/test_ljs_cut.cxx:14-118 ------------------------------
EPS, SIG, RC = 1.03120074782442750, 0.33841043857528683, 0.8125


def _lj_prefactor(eps, sig, r):
    s6 = sig ** 6
    r2inv = 1.0 / (r * r)
    r6inv = r2inv * r2inv * r2inv
    return -0.5 * (48.0 * eps * s6) * ((2.0 * s6) * r6inv - 1.0) * r6inv * r2inv


def test_ljs_cut_prepare_resets():
    pot = R.LJsCut(EPS, SIG, RC)
    sol = R.Solver(pot, threads=1)
    atoms = S.atom_array(1, DT)
    atoms["m"] = 40.0
    atoms["f"][0] = [1, 2, 3]
    atoms["Ep"] = 5.0
    atoms["Em"] = 7.0
    atoms["nc"] = 9.0
    atoms["V"][0] = np.eye(3).ravel()
    sol.prepare(atoms)
    assert sol.num_stages() == 1
    assert atoms["rcut"][0] == pot.rcut()
    assert not atoms["f"].any() and not atoms["V"].any() and atoms["Ep"][0] == 0.0


@pytest.mark.parametrize("half", [False, True])
def test_ljs_cut_force_virial_analytic(half):
    pot = R.LJsCut(EPS, SIG, RC)
    sol = R.Solver(pot, threads=1)
    dist = 0.40
    atoms = S.atom_array(2, DT)
    atoms["r"][1, 0] = dist
    atoms["rcut"] = RC
    atoms["rns"] = 0.5
    atoms["m"] = 1.0
    d = R.Domain(-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    nl = R.VerletList(atoms, d, threads=1, half=half)
    nl.update(-1.0)
    sol.prepare(atoms)
    sol.forces(atoms, nl)
    sol.virials(atoms, nl)
    fx = _lj_prefactor(EPS, SIG, dist) * dist
    sr6 = (SIG / dist) ** 6
    e = 2.0 * (0.5 * 4.0 * EPS * sr6 * (sr6 - 1.0))
    assert atoms["f"][0, 0] == pytest.approx(fx, abs=1e-12)
    assert atoms["f"][1, 0] == pytest.approx(-fx, abs=1e-12)
    assert abs(atoms["f"][0, 1]) < 1e-12 and abs(atoms["f"][1, 1]) < 1e-12
    assert atoms["Ep"].sum() == pytest.approx(e, abs=1e-12)
    tr = atoms["V"][:, 0] + atoms["V"][:, 4] + atoms["V"][:, 8]
    assert tr.sum() == pytest.approx(fx * dist, abs=1e-12)


# ---- test/cxx/solver/test_argon_ball_md.cxx:15-83 -------------------------
@pytest.fixture(scope="module")
def argon_history():
    atoms, box = S.argon_ball(DT)
    assert len(atoms) == 130124
    pot = R.LJsCut(EPS, SIG, RC)
    S.set_common_atom_properties(atoms, 40.0, pot.rcut(), 10.125 / 8.125)
    atoms["v"] = 0.0
    d = R.Domain(*box)
    sol = R.Solver(pot, threads=R.hardware_threads())
    nl = R.VerletList(atoms, d, threads=R.hardware_threads())
    hist = R.run_md_steps(sol, atoms, nl, 4e-3, 2, 1)
    return atoms, box, hist


def test_argon_ball_loads(argon_history):
    atoms, box, _ = argon_history
    assert box[1] - box[0] == pytest.approx(31.5, abs=1e-12)
    assert box[3] - box[2] == pytest.approx(31.5, abs=1e-12)
    assert atoms["uid"][0] == 1 and atoms["uid"][-1] == 130124


def test_argon_ball_step_two_energy_virial(argon_history):
    _, _, hist = argon_history
    assert len(hist) == 3
    assert hist[2]["Ep"] == pytest.approx(-1.0244383150033894e06, abs=1e-3)
    assert hist[2]["virial"] == pytest.approx(-1.1164231473675424e05, abs=1e-3)
    assert hist[2]["Etot"] == pytest.approx(hist[0]["Etot"], abs=2.0)


def test_argon_ball_particle_values(argon_history):
    atoms, _, _ = argon_history
    a1 = int(np.nonzero(atoms["uid"] == 1)[0][0])
    a2 = int(np.nonzero(atoms["uid"] == 2)[0][0])
    tr = lambda k: atoms["V"][k, 0] + atoms["V"][k, 4] + atoms["V"][k, 8]
    assert atoms["r"][a1, 0] == pytest.approx(-3.9184367989026225, abs=1e-12)
    assert atoms["r"][a1, 1] == pytest.approx(2.6440651643797461, abs=1e-12)
    assert atoms["r"][a1, 2] == pytest.approx(5.2690712254285517, abs=1e-12)
    assert atoms["v"][a1, 2] == pytest.approx(5.79013209455442e-04, abs=1e-15)
    assert atoms["f"][a1, 2] == pytest.approx(2.8929546164515996, abs=1e-12)
    assert atoms["Ep"][a1] == pytest.approx(-4.0629298955784474, abs=1e-12)
    assert tr(a1) == pytest.approx(-3.3178872346261723e-01, abs=1e-12)
    assert atoms["r"][a2, 2] == pytest.approx(5.7940689066038047, abs=1e-12)
    assert atoms["v"][a2, 0] == pytest.approx(-1.4268458571713898e-03, abs=1e-15)
    assert atoms["f"][a2, 0] == pytest.approx(-7.1268568973069453, abs=1e-12)
    assert atoms["Ep"][a2] == pytest.approx(-4.2002585997144832, abs=1e-12)
    assert tr(a2) == pytest.approx(4.2842826328841377e-01, abs=1e-12)


# ---- test/cxx/solver/test_aluminum_bulk_eam.cxx:16-88 ---------------------
AL_MASS, AL_A, AL_DT, AL_SKIN = 26.9815384, 0.4032, 4e-3, 1.25


def _al_setup(threads=1):
    t = S.al2009()
    pot = R.EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
    atoms, box = S.make_fcc_bulk(3, 3, 3, AL_A, AL_MASS, DT)
    d = R.Domain(*box)
    for k in range(3):
        d.set_periodic(k, True)
    S.set_common_atom_properties(atoms, AL_MASS, pot.rcut(), AL_SKIN)
    S.assign_deterministic_velocities(atoms, 5.0e-3)
    sol = R.Solver(pot, periodic=d, threads=threads)
    nl = R.VerletList(atoms, d, threads=threads)
    return pot, atoms, d, sol, nl


def test_al_eam_two_stages_and_periodic_neighbours():
    pot, atoms, d, sol, nl = _al_setup()
    nl.update(-1.0)
    assert sol.num_stages() == 2
    assert len(atoms) == 108
    assert len(nl.lists()[0]) > 12


def test_al_eam_energy_conservation():
    pot, atoms, d, sol, nl = _al_setup()
    hist = R.run_md_steps(sol, atoms, nl, AL_DT, 5, 1)
    assert len(hist) == 6
    assert hist[-1]["Etot"] == pytest.approx(hist[0]["Etot"], abs=40.0)
    assert np.linalg.norm(hist[-1]["vcom"]) == pytest.approx(0.0, abs=1e-12)
    assert np.isfinite([hist[-1]["Ep"], hist[-1]["Em"], hist[-1]["virial"]]).all()


@pytest.mark.parametrize("threads", [1, 4])
def test_al_eam_golden_values(threads):
    pot, atoms, d, sol, nl = _al_setup(threads)
    hist = R.run_md_steps(sol, atoms, nl, AL_DT, 2, 1)
    h = hist[-1]
    assert h["Etot"] == pytest.approx(-3.4489006959225437e04, abs=1e-6)
    assert h["Ep"] == pytest.approx(-6.7190981865001777e03, abs=1e-6)
    assert h["Em"] == pytest.approx(-2.7770493824864527e04, abs=1e-6)
    assert h["KE"] == pytest.approx(5.8505213926282473e-01, abs=1e-9)
    assert h["virial"] == pytest.approx(7.4272691119381875e01, abs=1e-9)
    assert atoms["r"][0, 0] == pytest.approx(6.0469801558679681e-01, abs=1e-12)
    assert atoms["r"][0, 1] == pytest.approx(6.0474258946107018e-01, abs=1e-12)
    assert atoms["r"][0, 2] == pytest.approx(6.0477602485847293e-01, abs=1e-12)
    assert atoms["v"][0, 0] == pytest.approx(-1.3221213313405629e-02, abs=1e-15)
    assert atoms["f"][0, 0] == pytest.approx(-1.1358391912725722e01, abs=1e-12)
    assert atoms["Ep"][0] == pytest.approx(-6.3230321656455359e01, abs=1e-9)
    assert atoms["Em"][0] == pytest.approx(-2.5721082474679707e02, abs=1e-9)
    assert atoms["V"][0, 0] + atoms["V"][0, 4] + atoms["V"][0, 8] == pytest.approx(
        1.3557390418206403e01, abs=1e-9)
