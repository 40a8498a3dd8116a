"""CPU checks of the oracle's force arithmetic by identities that hold for
any correct implementation (no GPU).

On open-box clusters and on slabs periodic in x and y (the Periodic ghost
pass, mdcraft/solver/boundary/periodic.cxx:9-102) cut from the benchmark
lattices (LJ argon, EAM Cu, NiAl B2 through Multi's per-kind-pair tables):
- the forces of LJsCut::force (mdcraft/solver/potential/LJs-cut.cxx:22),
  EAM::force (mdcraft/solver/potential/EAM.cxx:453) and Multi::force_one
  (mdcraft/solver/multi.cxx:97) are minus the gradient of the total energy
  sum(Ep) + sum(Em) (Em is set by EAM::virial, EAM.cxx:306), checked by
  central differences;
- in the open clusters, without periodic images, the virial traces of
  LJsCut::virial (LJs-cut.cxx:70), EAM::virial (EAM.cxx:306) and
  Multi::virial_one (multi.cxx:125), V_i = 1/2 sum_j f_ij (r_j - r_i), sum
  to -sum_i r_i . F_i.

These tie the oracle's forces to its energies, which the reference's golden
values (Ar ball, Al EAM) pin; the device forces match the oracle's to 1e-10.
"""
import numpy as np
import pytest

from mdcraft_gb300 import workloads as W
from oracle import mdref as R


def _solver(p, periodic):
    def eam(t):
        return R.EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])

    if p["kind"] == "lj":
        return R.Solver(R.LJsCut(p["a"], p["s"], p["rcut"]), periodic=periodic, threads=1)
    if p["kind"] == "eam":
        return R.Solver(eam(p["tables"]), periodic=periodic, threads=1)
    s = R.Solver(None, periodic=periodic, threads=1, nkinds=p.get("nkinds", 2))
    for (i, j), t in p["tables"].items():
        s.add_potential(i, j, eam(t))
    return s


def _evaluate(atoms, box, p, per=(0, 0, 0)):
    a = atoms.copy()
    d = R.Domain(*box)
    for k in range(3):
        if per[k]:
            d.set_periodic(k, True)
    nl = R.VerletList(a, d, threads=1)
    nl.update(-1.0)
    s = _solver(p, d if any(per) else None)
    s.prepare(a)
    s.stages(a, nl)
    s.virials(a, nl)
    return a


def _oracle_atoms(keep):
    a = np.zeros(len(keep), dtype=R.ATOM_DTYPE)
    a.view(np.uint8)[:] = np.ascontiguousarray(keep).view(np.uint8)
    return a


def _cluster(made, radius=0.45):
    """Atoms within radius·L of the box centre, in an open box."""
    atoms, box, _, p = made
    L = box[1] - box[0]
    c = np.array([box[0], box[2], box[4]]) + 0.5 * L
    return _oracle_atoms(atoms[np.linalg.norm(atoms["r"] - c, axis=1) < radius * L]), box, p, (0, 0, 0)


def _slab(made, keep_below=0.5):
    """The lower half of a periodic lattice, periodic in x and y, open in z."""
    atoms, box, _, p = made
    L = box[1] - box[0]
    return _oracle_atoms(atoms[atoms["r"][:, 2] < box[4] + keep_below * L]), box, p, (1, 1, 0)


CASES = [
    ("lj_argon", lambda: _cluster(W.lj_argon_fcc(ncell=4, jitter=0.02))),
    ("eam_cu", lambda: _cluster(W.eam_cu_fcc(ncell=5, jitter=0.02))),
    ("nial_multi", lambda: _cluster(W.eam_nial_b2(ncell=6))),
]
SLABS = [
    ("lj_argon_slab", lambda: _slab(W.lj_argon_fcc(ncell=5, jitter=0.02))),
    ("eam_cu_slab", lambda: _slab(W.eam_cu_fcc(ncell=6, jitter=0.02))),
    ("nial_multi_slab", lambda: _slab(W.eam_nial_b2(ncell=6))),
]


@pytest.mark.parametrize("case", CASES + SLABS, ids=lambda c: c[0])
def test_forces_are_minus_energy_gradient(case):
    atoms, box, p, per = case[1]()
    a = _evaluate(atoms, box, p, per)
    scale = np.sqrt(np.mean(np.sum(a["f"] ** 2, axis=1)))
    assert scale > 0.0
    h = 1e-6
    rng = np.random.default_rng(0)

    def energy(b):
        e = _evaluate(b, box, p, per)
        return e["Ep"].sum() + e["Em"].sum()

    for i in rng.choice(len(atoms), 6, replace=False):
        for ax in range(3):
            up = atoms.copy()
            up["r"][i, ax] += h
            dn = atoms.copy()
            dn["r"][i, ax] -= h
            g = -(energy(up) - energy(dn)) / (2.0 * h)
            # measured 1e-9 to 4e-8 of the RMS force (table interpolation, h^2 terms)
            assert abs(g - a["f"][i, ax]) <= 1e-6 * scale


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_virial_trace_is_minus_r_dot_f(case):
    atoms, box, p, _ = case[1]()
    a = _evaluate(atoms, box, p)
    tr = (a["V"][:, 0] + a["V"][:, 4] + a["V"][:, 8]).sum()
    rf = (a["r"] * a["f"]).sum()
    assert tr == pytest.approx(-rf, rel=1e-12)
    # Newton's third law: the forces sum to zero
    assert np.max(np.abs(a["f"].sum(axis=0))) <= 1e-12 * len(atoms) * np.max(np.abs(a["f"]))
