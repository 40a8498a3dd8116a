"""mdcraft.lattice.Domain (python/mdcraft/lattice/_lattice.cxx).

The geometry helpers (belong, fit_in_period, nearest_distance, reshape) are
host-side utilities in the reference too (per-atom loops in the binding over
Domain's methods, mdcraft/lattice/domain.cxx:23-66); here they are the same
expressions over the records' numpy view."""
from __future__ import annotations

import sys as _sys

import numpy as np

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
    xperiodic = property(lambda s: s.periodic(0))
    yperiodic = property(lambda s: s.periodic(1))
    zperiodic = property(lambda s: s.periodic(2))

    def _arrays(self):
        lo = np.array([self._b(k, 0) for k in range(3)])
        hi = np.array([self._b(k, 1) for k in range(3)])
        return lo, hi, hi - lo

    def reshape(self, xmin=0.0, xmax=0.0, ymin=0.0, ymax=0.0, zmin=0.0, zmax=0.0):
        """Domain::reshape (domain.cxx:23-32): new bounds, periodic flags kept."""
        self._d.c.bmin[:] = [xmin, ymin, zmin]
        self._d.c.bmax[:] = [xmax, ymax, zmax]

    def belong(self, *args):
        """Domain::belong (domain.cxx:34-40): a point (x, y, z) -> bool, or
        Atoms -> int array, 1 where bmin <= r <= bmax on every axis."""
        lo, hi, _ = self._arrays()
        if len(args) == 3:
            v = np.array(args, dtype=np.float64)
            return bool(np.all((lo <= v) & (v <= hi)))
        r = _xyz(args[0])
        return np.all((lo <= r) & (r <= hi), axis=1).astype(np.int32)

    def fit_in_period(self, atoms):
        """Domain::fit_in_period on every atom (domain.cxx:42-48): one period
        added below bmin or taken off above bmax, on periodic axes."""
        lo, hi, size = self._arrays()
        d = atoms.data
        for k, c in enumerate("xyz"):
            if not self.periodic(k):
                continue
            x = d["r"][c]
            d["r"][c] = np.where(x < lo[k], x + size[k], np.where(x > hi[k], x - size[k], x))

    def nearest_distance(self, atoms, axis: int):
        """Domain::nearest_distance per atom (domain.cxx:50-57): distance to
        the nearer face of a periodic axis, the largest double otherwise."""
        lo, hi, _ = self._arrays()
        r = _xyz(atoms)[:, axis]
        if not self.periodic(axis):
            return np.full(len(r), _sys.float_info.max)
        return np.minimum(np.abs(r - lo[axis]), np.abs(r - hi[axis]))


def _xyz(atoms):
    d = atoms.data
    return np.stack([d["r"]["x"], d["r"]["y"], d["r"]["z"]], axis=1)
