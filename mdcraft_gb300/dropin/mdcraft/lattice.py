"""mdcraft.lattice.Domain (python/mdcraft/lattice/_lattice.cxx)."""
from __future__ import annotations

import mdcraft_gb300 as _mdg


class Domain:
    def __init__(self, xmin=0.0, xmax=0.0, ymin=0.0, ymax=0.0, zmin=0.0, zmax=0.0):
        self._d = _mdg.Domain(xmin, xmax, ymin, ymax, zmin, zmax)

    def set_periodic(self, axis: int, periodic: bool = True):
        self._d.set_periodic(axis, periodic)

    def periodic(self, axis: int) -> bool:
        return bool(self._d.c.periodic[axis])

    def _b(self, k, hi):
        return (self._d.c.bmax if hi else self._d.c.bmin)[k]

    xmin = property(lambda s: s._b(0, 0))
    xmax = property(lambda s: s._b(0, 1))
    ymin = property(lambda s: s._b(1, 0))
    ymax = property(lambda s: s._b(1, 1))
    zmin = property(lambda s: s._b(2, 0))
    zmax = property(lambda s: s._b(2, 1))
    xsize = property(lambda s: s.xmax - s.xmin)
    ysize = property(lambda s: s.ymax - s.ymin)
    zsize = property(lambda s: s.zmax - s.zmin)
