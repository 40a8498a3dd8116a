"""mdcraft.solver.stepper.Verlet (python/mdcraft/solver/stepper/_stepper.cxx:28-72)."""
from __future__ import annotations

import mdcraft_gb300 as _mdg

from .._engine import device_of


class Verlet:
    def __init__(self, solver, threads=None):
        self.solver = solver
        self._st = _mdg.Verlet(solver._s)

    def make_step(self, atoms, nlist, dt: float):
        dev = device_of(atoms)
        dev.push()
        self._st.make_step(dev.sys, dt)
        dev.pull()
