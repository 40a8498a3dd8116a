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
    so.stages(ao, nlo)
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
