"""mdcraft.solver (python/mdcraft/solver/_solver.cxx:56-102): Single and Multi
over the GPU engine. Calls take (atoms, neibs, nlist) as the reference's do."""
from __future__ import annotations

import mdcraft_gb300 as _mdg

from .._engine import device_of


class Pair:
    """Common calls of the pair solvers (Pair::prepare/charge/forces/virials)."""

    def _run(self, atoms, neibs, nlist, what):
        if neibs is not atoms:
            raise NotImplementedError("one domain: neibs must be the atoms themselves")
        dev = device_of(atoms)
        dev.push()
        getattr(self._s, what)(dev.sys)
        dev.pull()

    def prepare(self, atoms, neibs, nlist):
        self._run(atoms, neibs, nlist, "prepare")

    def charge(self, atoms, neibs, nlist):
        self._run(atoms, neibs, nlist, "charge")

    def forces(self, atoms, neibs, nlist):
        self._run(atoms, neibs, nlist, "forces")

    def virials(self, atoms, neibs, nlist):
        self._run(atoms, neibs, nlist, "virials")

    def stages(self, atoms, neibs, nlist):
        self._run(atoms, neibs, nlist, "stages")


def _attach(solver, thermostat):
    """The thermostat argument of Single / Multi: applied after each atom's
    forces in the force stage (pair.cxx:72-86)."""
    solver._thermostat = thermostat
    if thermostat is not None and thermostat._t is not None:
        solver._s.set_thermostat(thermostat._t)


class Single(Pair):
    def __init__(self, potential, boundary=None, thermostat=None, threads=None, precision="fp64"):
        self.potential = potential
        self._s = _mdg.Single(potential._p, periodic=boundary is not None, precision=precision)
        _attach(self, thermostat)


class Multi(Pair):
    def __init__(self, boundary=None, thermostat=None, nkinds: int = 1, threads=None, precision="fp64"):
        self._keep = []
        self._s = _mdg.Multi(nkinds, periodic=boundary is not None, precision=precision)
        _attach(self, thermostat)

    def add_potential(self, i: int, j: int, potential):
        self._keep.append(potential)
        self._s.add_potential(i, j, potential._p)
