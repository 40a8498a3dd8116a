"""mdcraft.solver.potential (python/mdcraft/solver/potential/_potential.cxx):
EAM (arrays or a setfl file), Pair (arrays or a file), LJs and LJsCut on the
GPU engine."""
from __future__ import annotations

import numpy as np

import mdcraft_gb300 as _mdg

from .._engine import context as _context


def _value_at(pot, r):
    """value(r) of a scalar distance: the pair energy term at r^2 = r*r (the
    bindings build the vector (r, 0, 0), _potential.cxx:155-159, 197-201)."""
    return float(pot.values(_context(), np.array([float(r) * float(r)]))[0])


class EAM:
    def __init__(self, *args, **kw):
        if (len(args) == 1 and isinstance(args[0], str)) or "filename" in kw:
            self._p = _mdg.EAM.from_file(args[0] if args else kw["filename"])
            return
        names = ["Rcutoff", "pairPotential", "chargeDensity", "embeddingEnergy", "NrPot", "drPot", "NrEmb", "drEmb"]
        a = dict(zip(names, args))
        a.update(kw)
        self._p = _mdg.EAM(a["Rcutoff"], np.asarray(a["embeddingEnergy"], dtype=np.float64),
                           np.asarray(a["chargeDensity"], dtype=np.float64),
                           np.asarray(a["pairPotential"], dtype=np.float64), int(a["NrPot"]), float(a["drPot"]),
                           int(a["NrEmb"]), float(a["drEmb"]))

    @property
    def rcut(self) -> float:
        return self._p.rcut()

    def value(self, r: float) -> float:
        """Pair energy term at distance r (_potential.cxx:155-159)."""
        return _value_at(self._p, r)

    def embeddingEnergy(self, r):
        """F(rho) of each density (_potential.cxx:160-168)."""
        F, _ = self._p.embedding(_context(), r)
        return F


class LJsCut:
    def __init__(self, a: float, s: float, rcut: float):
        self._p = _mdg.LJsCut(a, s, rcut)

    @property
    def rcut(self) -> float:
        return self._p.rcut()


class LJs:
    """LJs(aVr, rVr, Rcutoff) (_potential.cxx:82-100)."""

    def __init__(self, aVr: float, rVr: float, Rcutoff: float):
        self._p = _mdg.LJs(aVr, rVr, Rcutoff)

    @property
    def rcut(self) -> float:
        return self._p.rcut()

    def value(self, r2):
        """value(array of r^2) -> array, or value(r) -> float for a scalar
        distance (_potential.cxx:88-100)."""
        if np.ndim(r2) == 0:
            return _value_at(self._p, r2)
        return self._p.values(_context(), np.asarray(r2, dtype=np.float64))


class Pair:
    """Pair(Rcutoff, pairPotential, NrPot, drPot) or Pair(filename)
    (_potential.cxx:170-201): tabulated r*phi(r)."""

    def __init__(self, *args, **kw):
        if (len(args) == 1 and isinstance(args[0], str)) or "filename" in kw:
            self._p = _mdg.Pair.from_file(args[0] if args else kw["filename"])
            return
        names = ["Rcutoff", "pairPotential", "NrPot", "drPot"]
        a = dict(zip(names, args))
        a.update(kw)
        self._p = _mdg.Pair(a["Rcutoff"], np.asarray(a["pairPotential"], dtype=np.float64), int(a["NrPot"]),
                            float(a["drPot"]))

    @property
    def rcut(self) -> float:
        return self._p.rcut()


    def value(self, r: float) -> float:
        """Pair energy term at distance r (_potential.cxx:197-201)."""
        return _value_at(self._p, r)


# the reference's module also exports LJsCut under this name (_potential.cxx:110)
LJsTEST = LJsCut
