"""CPU check of the oracle's boundary semantics (no GPU).

In the reference, periodic forces come only from the Periodic boundary's
ghost pass (mdcraft/solver/boundary/periodic.cxx:36-102). The Verlet list of
a periodic domain still holds the pairs that cross a periodic face, found by
are_neibs' minimum image (mdcraft/neibs/verlet-list.cxx:392-397). A solver
without the Periodic boundary evaluates them at their raw separation, which
lies beyond the cutoff (mdcraft/solver/potential/LJs-cut.cxx:45; the EAM
density and force loops cut the same way). So those pairs add nothing, and
a periodic domain with no boundary gives exactly the forces, energies and
virials of the same atoms in an open box. With the boundary the crossing
pairs count and the forces differ.
"""
import numpy as np
import pytest

from mdcraft_gb300 import workloads as W
from oracle import mdref as R
from tests.test_oracle_gradients import _oracle_atoms, _solver

CASES = [
    ("lj_argon", lambda: W.lj_argon_fcc(ncell=6, jitter=0.02)),
    ("eam_cu", lambda: W.eam_cu_fcc(ncell=6)),
    ("nial_multi", lambda: W.eam_nial_b2(ncell=8)),
]


def _run(atoms, box, p, periodic_domain, boundary):
    a = atoms.copy()
    d = R.Domain(*box)
    if periodic_domain:
        for k in range(3):
            d.set_periodic(k, True)
    nl = R.VerletList(a, d, threads=1)
    nl.update(-1.0)
    s = _solver(p, d if boundary else None)
    s.prepare(a)
    s.stages(a, nl)
    s.virials(a, nl)
    return a, nl


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_periodic_domain_without_boundary_equals_open_box(case):
    atoms, box, _, p = case[1]()
    atoms = _oracle_atoms(atoms)
    no_bc, nl_p = _run(atoms, box, p, True, False)
    open_, nl_o = _run(atoms, box, p, False, False)
    # the periodic list holds the face-crossing pairs the open one lacks
    assert sum(map(len, nl_p.lists())) > sum(map(len, nl_o.lists()))
    for key in ("f", "Ep", "Em", "V", "nc"):
        assert np.array_equal(no_bc[key], open_[key]), key
    with_bc, _ = _run(atoms, box, p, True, True)
    assert np.max(np.abs(with_bc["f"] - no_bc["f"])) > 1.0
