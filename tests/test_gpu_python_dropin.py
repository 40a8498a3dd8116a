"""The Python drop-in (`mdcraft` package under mdcraft_gb300/dropin): the call
sequence of the reference's EAM driver (test/python/solver/test-EAM.py:18-200:
mesh of fcc Al, EAM from a setfl file, Periodic, Single, Verlet, VerletList
with kbuf 1.25, initial prepare/forces/virials, then make_step with virials
every 10 steps and update() every 10 steps) through the drop-in on the GPU,
against the same sequence through the CPU oracle."""
from __future__ import annotations

import lzma
import os
import sys

import numpy as np
import pytest

from tests import gpu_helpers as H
from tests import mdsupport as S

pytestmark = pytest.mark.gpu

_DROPIN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "mdcraft_gb300", "dropin")


def _mesh(Atoms, D, n):
    """fcc positions in the layout of the driver's mesh helper (4 atoms per
    cell, box centred at the origin), kind 1."""
    L = n * D
    lo = -0.5 * L
    g = np.linspace(lo + 0.25 * D, lo + L - 0.75 * D, n)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    atoms = Atoms(0)
    atoms.resize(4 * X.size)
    d = atoms.data
    for k, (ox, oy, oz) in enumerate(((0, 0, 0), (0.5, 0.5, 0), (0.5, 0, 0.5), (0, 0.5, 0.5))):
        d["r"]["x"][k::4] = X.ravel() + ox * D
        d["r"]["y"][k::4] = Y.ravel() + oy * D
        d["r"]["z"][k::4] = Z.ravel() + oz * D
    d["kind"] = 1
    return atoms, (lo, lo + L, lo, lo + L, lo, lo + L)


def test_reference_driver_sequence(tmp_path):
    H.ctx()  # builds libmdg
    sys.path.insert(0, _DROPIN)
    try:
        from mdcraft.data import Atoms
        from mdcraft.lattice import Domain
        from mdcraft.neibs import VerletList
        from mdcraft.solver import Single as Solver
        from mdcraft.solver.boundary import Periodic
        from mdcraft.solver.potential import EAM
        from mdcraft.solver.stepper import Verlet as Stepper
        from mdcraft.solver.thermostat import Langevin
        from mdcraft.tools import Threads
    finally:
        sys.path.remove(_DROPIN)
    setfl = tmp_path / "Al2009.eam.alloy"
    with lzma.open(os.path.join(S.GOLDEN, "al2009_eam_alloy.xz"), "rt") as f:
        setfl.write_text(f.read())

    threads = Threads(4)
    potential = EAM(str(setfl))
    atoms, box = _mesh(Atoms, 0.4032, 5)
    atoms.data["rcut"] = potential.rcut
    atoms.data["m"] = 26.9815384
    rng = np.random.default_rng(17)
    sigma = (1.2 * 0.008314462175 * 300.0 / 26.9815384) ** 0.5
    for c in "xyz":
        v = rng.normal(0.0, sigma, atoms.data.size)
        atoms.data["v"][c] = v - v.mean()
    domain = Domain(*box)
    for k in range(3):
        domain.set_periodic(k, True)
    periodic = Periodic(domain)
    Langevin(beta=0.5, temperature=300.0, time_step=4e-3, heat_x=1, heat_y=1, heat_z=1, Ux=0, Uy=0, Uz=0)
    solver = Solver(potential=potential, boundary=periodic, threads=threads)
    solver_cold = Solver(potential=potential, boundary=periodic, threads=threads)
    stepper = Stepper(solver=solver, threads=threads)
    atoms.data["rns"] = 1.25 * atoms.data["rcut"]
    start = atoms.data.copy()
    nlist = VerletList(atoms=atoms, neighbors=atoms, threads=threads, domain=domain)
    nlist.update()
    solver_cold.prepare(atoms, atoms, nlist.get())
    solver_cold.forces(atoms, atoms, nlist.get())
    solver_cold.virials(atoms, atoms, nlist.get())
    energies = []
    for step in range(1, 41):
        stepper.make_step(atoms, nlist.get(), 4e-3)
        if step % 10 == 0:
            solver.virials(atoms, atoms, nlist.get())
            energies.append(float(np.sum(atoms.data["Ep"]) + np.sum(atoms.data["Em"])))
            nlist.update()
    gpu = atoms.data

    # the oracle, same calls
    from oracle import mdref as R
    ao = np.zeros(len(start), dtype=R.ATOM_DTYPE)
    ao.view(np.uint8)[:] = start.view(np.uint8)
    do = R.Domain(*box)
    for k in range(3):
        do.set_periodic(k, True)
    t = S.al2009()
    po = R.EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
    so = R.Solver(po, periodic=do, threads=4)
    nlo = R.VerletList(ao, do, threads=4)
    nlo.update(-1.0)
    so.prepare(ao)
    so.forces(ao, nlo)
    so.virials(ao, nlo)
    e_o = []
    for step in range(1, 41):
        so.make_step(ao, nlo, 4e-3)
        if step % 10 == 0:
            so.virials(ao, nlo)
            e_o.append(float(np.sum(ao["Ep"]) + np.sum(ao["Em"])))
            nlo.update(-1.0)
    g = gpu.view(np.uint8).reshape(len(gpu), 208)
    o = ao.view(np.uint8).reshape(len(ao), 208)
    rg = g[:, :24].copy().view(np.float64)
    ro = o[:, :24].copy().view(np.float64)
    assert np.max(np.abs(rg - ro)) < 1e-9
    assert np.allclose(energies, e_o, rtol=1e-9, atol=0.0)


def _import_dropin():
    sys.path.insert(0, _DROPIN)
    try:
        import mdcraft
        from mdcraft import data, lattice, neibs, solver, tools
        from mdcraft.solver import boundary, potential, stepper, thermostat
        return mdcraft
    finally:
        sys.path.remove(_DROPIN)


def test_nial_driver_sequence_with_pair_and_langevin(tmp_path):
    """The call sequence of problems/NiAl/test-NiAl.py:37-240 (two EAM kinds,
    the tabulated Ni-Al Pair as cross term read from its file, Multi with
    Periodic and a Langevin thermostat, Verlet, VerletList with kbuf 1.25,
    update() every 10 steps) through the drop-in, against the oracle with
    the same Philox seed. The driver loads Al.eam.alloy for both kinds; the
    Al2009 setfl fixture stands in for it."""
    H.ctx()
    _import_dropin()
    from mdcraft.data import Atoms
    from mdcraft.lattice import Domain
    from mdcraft.neibs import VerletList
    from mdcraft.solver import Multi as Solver
    from mdcraft.solver.boundary import Periodic
    from mdcraft.solver.potential import EAM, Pair
    from mdcraft.solver.stepper import Verlet as Stepper
    from mdcraft.solver.thermostat import Langevin
    from mdcraft.tools import Threads

    setfl = tmp_path / "Al.eam.alloy"
    setfl.write_text(S.al2009_text())
    pairfile = tmp_path / "NiAlpair.eam.alloy"
    pairfile.write_text(S.nialpair_text())
    threads = Threads(4)
    Al_potential = EAM(str(setfl))
    Ni_potential = EAM(str(setfl))
    NiAl_potential = Pair(str(pairfile))
    atoms, box = _mesh(Atoms, 0.405, 6)
    rng = np.random.default_rng(23)
    kinds = rng.choice([0, 1], atoms.data.size, p=[0.8, 0.2])
    iAl, iNi = np.where(kinds == 0), np.where(kinds == 1)
    atoms.data["kind"] = kinds
    atoms.data["m"][iAl] = 26.9815384
    atoms.data["m"][iNi] = 58.6934
    atoms.data["rcut"][iAl] = Al_potential.rcut
    atoms.data["rcut"][iNi] = Ni_potential.rcut
    for idx, mass in ((iAl, 26.9815384), (iNi, 58.6934)):
        sigma = (1.2 * 0.008314462175 * 300.0 / mass) ** 0.5
        for c in "xyz":
            atoms.data["v"][c][idx] = rng.normal(0.0, sigma, idx[0].size)
    m = atoms.data["m"]
    for c in "xyz":
        atoms.data["v"][c] -= np.sum(m * atoms.data["v"][c]) / np.sum(m)
    domain = Domain(*box)
    for k in range(3):
        domain.set_periodic(k, True)
    periodic = Periodic(domain)
    thermostat = Langevin(beta=0.5, temperature=300.0, time_step=4e-3, heat_x=1, heat_y=1, heat_z=1,
                          Ux=0, Uy=0, Uz=0, seed=99)
    assert thermostat.temperature == 300.0 and thermostat.friction == 0.5
    solver = Solver(boundary=periodic, thermostat=thermostat, nkinds=2, threads=threads)
    solver.add_potential(0, 0, Al_potential)
    solver.add_potential(1, 1, Ni_potential)
    solver.add_potential(0, 1, NiAl_potential)
    solver_cold = Solver(boundary=periodic, nkinds=2, threads=threads)
    solver_cold.add_potential(0, 0, Al_potential)
    solver_cold.add_potential(1, 1, Ni_potential)
    solver_cold.add_potential(0, 1, NiAl_potential)
    stepper = Stepper(solver=solver, threads=threads)
    atoms.data["rns"] = 1.25 * atoms.data["rcut"]
    start = atoms.data.copy()
    nlist = VerletList(atoms=atoms, neighbors=atoms, threads=threads, domain=domain)
    nlist.update()
    solver_cold.prepare(atoms, atoms, nlist.get())
    solver_cold.forces(atoms, atoms, nlist.get())
    solver_cold.virials(atoms, atoms, nlist.get())
    e_g = []
    for step in range(1, 31):
        stepper.make_step(atoms, nlist.get(), 4e-3)
        if step % 10 == 0:
            solver.virials(atoms, atoms, nlist.get())
            e_g.append(float(np.sum(atoms.data["Ep"]) + np.sum(atoms.data["Em"])))
            nlist.update()
    gpu = atoms.data

    from oracle import mdref as R
    ao = np.zeros(len(start), dtype=R.ATOM_DTYPE)
    ao.view(np.uint8)[:] = start.view(np.uint8)
    do = R.Domain(*box)
    for k in range(3):
        do.set_periodic(k, True)
    al = S.al2009()
    pt = S.nialpair()
    p_al = R.EAM(al["rcut"], al["Femb"], al["Rho"], al["Vpar"], al["Nr1"], al["dr"], al["Nrh1"], al["drh"])
    p_x = R.Pair(pt["rcut"], pt["Vpar"], pt["Nr1"], pt["dr"])
    so = R.Solver(None, periodic=do, threads=4, nkinds=2)
    cold = R.Solver(None, periodic=do, threads=4, nkinds=2)
    for s_ in (so, cold):
        s_.add_potential(0, 0, p_al)
        s_.add_potential(1, 1, p_al)
        s_.add_potential(0, 1, p_x)
    so.set_thermostat(R.Thermostat(dict(beta=0.5, temperature=300.0, time_step=4e-3, seed=99)))
    nlo = R.VerletList(ao, do, threads=4)
    nlo.update(-1.0)
    cold.prepare(ao)
    cold.forces(ao, nlo)
    cold.virials(ao, nlo)
    e_o = []
    for step in range(1, 31):
        so.make_step(ao, nlo, 4e-3)
        if step % 10 == 0:
            so.virials(ao, nlo)
            e_o.append(float(np.sum(ao["Ep"]) + np.sum(ao["Em"])))
            nlo.update(-1.0)
    g = gpu.view(np.uint8).reshape(len(gpu), 208)
    o = ao.view(np.uint8).reshape(len(ao), 208)
    rg = g[:, :24].copy().view(np.float64)
    ro = o[:, :24].copy().view(np.float64)
    assert np.max(np.abs(rg - ro)) < 1e-9
    assert np.allclose(e_g, e_o, rtol=1e-9, atol=0.0)
