"""mdcraft.neibs.VerletList (python/mdcraft/neibs/_neibs.cxx:23-196) on the GPU."""
from __future__ import annotations

import numpy as np

import mdcraft_gb300 as _mdg

from ._engine import DeviceAtoms, engine_view


class VerletList:
    def __init__(self, atoms, neighbors, domain, threads=None, half: bool = False):
        if neighbors is not atoms:
            raise NotImplementedError("one domain: the neighbours must be the atoms themselves")
        if half and threads is not None and threads.count > 1:  # verlet-list.cxx:28-31
            raise RuntimeError("Half Verlet lists are currently incompatible with multithreaded pair-force "
                               "evaluation. Disable threads or use a full neighbor list.")
        atoms._device = DeviceAtoms(atoms, domain)
        self._dev = atoms._device
        self._nl = _mdg.VerletList(self._dev.sys, half=half)
        self._dev.nl = self._nl

    def update(self, kbuf: float = -1.0):
        self._dev.push()
        self._nl.update(kbuf)
        self._dev.pull()  # positions fitted into the period, as the reference does

    @property
    def half(self) -> bool:
        return self._nl.half

    def decide(self) -> bool:
        self._dev.push()
        return self._nl.decide()

    def get(self):
        return self

    def __getitem__(self, i):
        return self._nl.lists()[i]

    def list_for(self, x, y=0.0, z=0.0):
        return np.asarray(self._nl.list_for((x, y, z)))

    def sort(self, elems):
        """Atoms ordered by owning cell (_neibs.cxx:80-97, verlet-list.cxx:237-249);
        `elems` are wrapped into the period in place, as the reference does."""
        from .data import Atoms
        data = np.ascontiguousarray(elems.data)
        flat = engine_view(data)
        out = Atoms(0)
        out._data = np.empty_like(data)
        engine_view(out._data)[:] = self._nl.sort(flat)
        elems._data = data
        return out
