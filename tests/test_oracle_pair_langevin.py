"""CPU checks of the oracle's tabulated Pair and LJs potentials and the
Langevin thermostat, and of the product's Pair file reader (host code, no
GPU).

The reference's tests hold no golden values for these two, so the oracle is
pinned by identities with pinned parts:
- Pair::force/virial (mdcraft/solver/potential/pair.cxx:228-462) is the pair
  term of EAM::force/virial (EAM.cxx:306-497) with zero density tables, and
  the EAM arithmetic is pinned by the Al EAM golden test;
- LJs (mdcraft/solver/potential/LJs.cxx) forces are minus the gradient of
  its energies, and both vanish at the cutoff, which is what its cubic in
  X = (r/rVr)^2 - 2^(1/3) is built for;
- Philox4x32-10 reproduces the published known-answer vectors of Salmon et
  al. (SC'11, Random123 kat_vectors);
- Langevin::apply_one (mdcraft/solver/thermostat/langevin.cxx:29-42) at zero
  temperature is the friction term exactly, and its random part has the
  normal law N(0, m sigma^2) per heated axis.
"""
import numpy as np
import pytest

from oracle import mdref as R
from tests import mdsupport as S


def test_philox_known_answers():
    kat = [
        (([0, 0, 0, 0], [0, 0]), [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
        (([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2), [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
        (([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]),
         [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
    ]
    for (ctr, key), want in kat:
        assert list(R.philox4x32_10(ctr, key)) == want


def _fcc_jitter(n, a, seed, jitter=0.02):
    atoms, box = S.make_fcc_bulk(n, n, n, a, 26.9815, R.ATOM_DTYPE)
    rng = np.random.default_rng(seed)
    atoms["r"] += rng.normal(0.0, jitter * a, size=(len(atoms), 3))
    return atoms, box


def _periodic(box):
    d = R.Domain(*box)
    for k in range(3):
        d.set_periodic(k, True)
    return d


def _run_forces(solver, atoms, box, rc, skin=0.05):
    atoms["rcut"] = rc
    atoms["rns"] = rc + skin
    nl = R.VerletList(atoms, _periodic(box), threads=2)
    nl.update(-1.0)
    solver.prepare(atoms)
    solver.stages(atoms, nl)
    solver.virials(atoms, nl)
    return atoms


def test_pair_equals_eam_pair_term():
    t = S.nialpair()
    a1, box = _fcc_jitter(4, 0.405, 1)
    a2 = a1.copy()
    d = _periodic(box)
    pair = R.Pair(t["rcut"], t["Vpar"], t["Nr1"], t["dr"])
    zeros_r = np.zeros(t["Nr1"])
    eam = R.EAM(t["rcut"], np.zeros(64), zeros_r, t["Vpar"], t["Nr1"], t["dr"], 64, 1.0)
    sp = R.Solver(pair, periodic=d, threads=2)
    se = R.Solver(eam, periodic=d, threads=2)
    assert sp.num_stages() == 1 and se.num_stages() == 2
    _run_forces(sp, a1, box, t["rcut"])
    _run_forces(se, a2, box, t["rcut"])
    assert np.abs(a1["f"]).max() > 1.0
    assert np.array_equal(a1["f"], a2["f"])
    assert np.array_equal(a1["Ep"], a2["Ep"])
    assert np.array_equal(a1["V"], a2["V"])
    assert np.all(a2["Em"] == 0.0)
    # Newton's third law over the periodic box
    assert np.abs(a1["f"].sum(axis=0)).max() < 1e-9 * np.abs(a1["f"]).max() * len(a1)


def test_pair_half_list_matches_full_list():
    t = S.nialpair()
    a_full, box = _fcc_jitter(3, 0.405, 2)
    a_half = a_full.copy()
    pair = R.Pair(t["rcut"], t["Vpar"], t["Nr1"], t["dr"])
    res = []
    for atoms, half in ((a_full, False), (a_half, True)):
        atoms["rcut"] = t["rcut"]
        atoms["rns"] = t["rcut"] + 0.05
        nl = R.VerletList(atoms, R.Domain(*box), threads=1, half=half)
        nl.update(-1.0)
        s = R.Solver(pair, periodic=None, threads=1)
        s.prepare(atoms)
        s.forces(atoms, nl)
        s.virials(atoms, nl)
        res.append(atoms)
    np.testing.assert_allclose(res[1]["f"], res[0]["f"], rtol=0, atol=1e-9 * np.abs(res[0]["f"]).max())
    np.testing.assert_allclose(res[1]["Ep"].sum(), res[0]["Ep"].sum(), rtol=1e-12)


def test_multi_with_pair_cross_term():
    al = S.al2009()
    t = S.nialpair()
    atoms, box = _fcc_jitter(4, 0.405, 3)
    atoms["kind"] = (np.arange(len(atoms)) % 3 == 0).astype(np.uint16)
    d = _periodic(box)
    s = R.Solver(None, periodic=d, threads=2, nkinds=2)
    eam = R.EAM(al["rcut"], al["Femb"], al["Rho"], al["Vpar"], al["Nr1"], al["dr"], al["Nrh1"], al["drh"])
    pair = R.Pair(t["rcut"], t["Vpar"], t["Nr1"], t["dr"])
    s.add_potential(0, 0, eam)
    s.add_potential(1, 1, eam)
    s.add_potential(0, 1, pair)
    assert s.num_stages() == 2
    rc = max(al["rcut"], t["rcut"])
    atoms["rns"] = rc + 0.05
    atoms["rcut"] = rc
    nl = R.VerletList(atoms, d, threads=2)
    nl.update(-1.0)
    s.prepare(atoms)
    s.stages(atoms, nl)
    f = atoms["f"].copy()
    assert np.abs(f.sum(axis=0)).max() < 1e-8 * np.abs(f).max() * len(atoms)
    # the cross term is a pure pair term: dropping it changes forces
    s2 = R.Solver(None, periodic=d, threads=2, nkinds=2)
    s2.add_potential(0, 0, eam)
    s2.add_potential(1, 1, eam)
    zero = R.Pair(t["rcut"], np.zeros(t["Nr1"]), t["Nr1"], t["dr"])
    s2.add_potential(0, 1, zero)
    s2.prepare(atoms)
    s2.stages(atoms, nl)
    assert np.abs(atoms["f"] - f).max() > 1e-3 * np.abs(f).max()


def _isolated_atoms(n, box_len, seed):
    rng = np.random.default_rng(seed)
    atoms = R.new_atoms(n)
    atoms["r"] = rng.uniform(-0.5 * box_len, 0.5 * box_len, size=(n, 3))
    atoms["v"] = rng.normal(0.0, 0.3, size=(n, 3))
    atoms["m"] = rng.uniform(20.0, 60.0, size=n)
    atoms["rcut"] = 0.3
    atoms["rns"] = 0.35
    atoms["uid"] = np.arange(1, n + 1)
    return atoms, (-0.5 * box_len, 0.5 * box_len) * 3


def _langevin_forces(atoms, box, terms, calls=0):
    box = (box[0], box[1], box[0], box[1], box[0], box[1])
    pot = R.LJsCut(0.0, 0.3, 0.3)  # zero well depth: the thermostat alone acts
    s = R.Solver(pot, periodic=None, threads=2)
    th = R.Thermostat(*terms)
    s.set_thermostat(th, calls)
    nl = R.VerletList(atoms, R.Domain(*box), threads=2)
    nl.update(-1.0)
    s.prepare(atoms)
    s.forces(atoms, nl)
    return s


def test_langevin_friction_at_zero_temperature():
    atoms, box = _isolated_atoms(500, 50.0, 4)
    U = (0.1, -0.2, 0.05)
    s = _langevin_forces(atoms, box, [dict(beta=0.7, temperature=0.0, time_step=0.004, heat_y=0,
                                           Ux=U[0], Uy=U[1], Uz=U[2], seed=9)])
    want = -(atoms["v"] - np.array(U)) * 0.7 * atoms["m"][:, None]
    want[:, 1] = 0.0
    np.testing.assert_array_equal(atoms["f"][:, [0, 2]], want[:, [0, 2]])
    assert np.all(atoms["f"][:, 1] == 0.0)
    assert s.thermo_calls() == 1


def test_langevin_x_window_and_reproducibility():
    atoms, box = _isolated_atoms(400, 50.0, 5)
    a2 = atoms.copy()
    a3 = atoms.copy()
    term = dict(beta=0.5, temperature=300.0, time_step=0.004, xmin=-5.0, xmax=5.0, seed=11)
    _langevin_forces(atoms, box, [term])
    _langevin_forces(a2, box, [term])
    _langevin_forces(a3, box, [dict(term, seed=12)])
    inside = (atoms["r"][:, 0] >= -5.0) & (atoms["r"][:, 0] <= 5.0)
    assert inside.any() and (~inside).any()
    assert np.all(atoms["f"][~inside] == 0.0)
    assert np.all(atoms["f"][inside] != 0.0)
    assert np.array_equal(atoms["f"], a2["f"])
    assert not np.array_equal(atoms["f"][inside], a3["f"][inside])


def test_langevin_random_force_law():
    n = 40000
    atoms, box = _isolated_atoms(n, 60.0, 6)
    atoms["v"] = 0.0
    beta, T, dt = 0.5, 300.0, 0.004
    _langevin_forces(atoms, box, [dict(beta=beta, temperature=T, time_step=dt, seed=3)], calls=17)
    sigma = np.sqrt(2.0 * beta * 0.008314462175 * T / dt)
    z = atoms["f"] / (np.sqrt(atoms["m"])[:, None] * sigma)
    assert abs(z.mean()) < 4.0 / np.sqrt(3 * n)
    assert abs(z.var() - 1.0) < 0.03
    # the three components are independent draws
    c = np.corrcoef(z.T)
    assert np.abs(c - np.eye(3)).max() < 0.03
    # one draw of the oracle's stream, by hand
    i = 123
    zi = R.langevin_normals(3, i, 17, 0)
    np.testing.assert_allclose(atoms["f"][i], zi * sigma * np.sqrt(atoms["m"][i]), rtol=1e-15)


def test_compound_applies_terms_in_order():
    atoms, box = _isolated_atoms(300, 50.0, 7)
    a1 = atoms.copy()
    t1 = dict(beta=0.5, temperature=100.0, time_step=0.004, seed=1)
    t2 = dict(beta=0.2, temperature=0.0, time_step=0.004, seed=2, heat_x=0)
    _langevin_forces(atoms, box, [t1, t2])
    _langevin_forces(a1, box, [t1])
    fric = -(a1["v"]) * 0.2 * a1["m"][:, None]
    fric[:, 0] = 0.0
    np.testing.assert_allclose(atoms["f"], a1["f"] + fric, rtol=1e-14, atol=1e-12)


def test_product_pair_reader(tmp_path):
    """mdg_pot_pair_create_from_file (host code) reads the NiAl pair table
    like pair.cxx:36-56; no GPU is touched."""
    import mdcraft_gb300 as mdg
    from mdcraft_gb300 import build
    build.build()
    path = tmp_path / "NiAlpair.eam.alloy"
    path.write_text(S.nialpair_text())
    p = mdg.Pair.from_file(str(path))
    t = S.nialpair()
    assert p.rcut() == t["rcut"] == pytest.approx(0.6724884, rel=1e-7)
    assert t["Nr1"] == 10000 and t["dr"] == pytest.approx(6.724884e-5, rel=1e-6)
    with pytest.raises(mdg.MDGError):
        mdg.Pair.from_file(str(tmp_path / "missing"))
    short = tmp_path / "short"
    short.write_text("\n".join(S.nialpair_text().splitlines()[:100]))
    with pytest.raises(mdg.MDGError):
        mdg.Pair.from_file(str(short))


def _two_atoms(r, pot, rc):
    atoms = R.new_atoms(2)
    atoms["r"][1, 0] = r
    atoms["m"] = 1.0
    atoms["rcut"] = rc
    atoms["rns"] = rc + 0.05
    nl = R.VerletList(atoms, R.Domain(-2.0, 2.0, -2.0, 2.0, -2.0, 2.0), threads=1)
    nl.update(-1.0)
    s = R.Solver(pot, periodic=None, threads=1)
    s.prepare(atoms)
    s.forces(atoms, nl)
    s.virials(atoms, nl)
    return atoms


def test_ljs_force_is_energy_gradient_and_vanishes_at_cutoff():
    aVr, rVr, rc = 1.0, 0.34, 0.85
    pot = R.LJs(aVr, rVr, rc)
    for r in (0.33, 0.38, 0.5, 0.7):
        h = 1e-6
        up = _two_atoms(r + h, pot, rc)["Ep"].sum()
        dn = _two_atoms(r - h, pot, rc)["Ep"].sum()
        a = _two_atoms(r, pot, rc)
        # atom 1 sits at +r on x: its force is -dU/dr
        assert a["f"][1, 0] == pytest.approx(-(up - dn) / (2 * h), rel=1e-6)
        assert a["f"][0, 0] == -a["f"][1, 0]
        # the short-range limit is Lennard-Jones 4 aVr [(rVr/r)^12 - (rVr/r)^6] plus the smooth tail
    near = _two_atoms(rc * (1 - 1e-7), pot, rc)
    assert abs(near["Ep"].sum()) < 1e-9 and abs(near["f"][0, 0]) < 1e-5
    assert _two_atoms(rc * (1 + 1e-7), pot, rc)["Ep"].sum() == 0.0
    # V = 1/2 sum f_i (r_j - r_i): both sides give f_1 . (r_0 - r_1) / 2
    a = _two_atoms(0.4, pot, rc)
    assert (a["V"][:, 0]).sum() == pytest.approx(a["f"][1, 0] * -0.4, rel=1e-12)
