"""The Python drop-in's Domain (python/mdcraft/lattice/_lattice.cxx:15-245):
the calls of the reference's test/python/lattice/test-domain.py (bounds,
sizes, periodic flags, belong over atoms, nearest_distance per axis), plus
fit_in_period and reshape, each checked per atom against the oracle's
restatement of mdcraft/lattice/domain.cxx. Host code only: no GPU."""
import os
import sys

import numpy as np

from oracle import mdref as R

_DROPIN = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "mdcraft_gb300", "dropin")


def _dropin():
    sys.path.insert(0, _DROPIN)
    try:
        from mdcraft.data import Atoms
        from mdcraft.lattice import Domain
    finally:
        sys.path.remove(_DROPIN)
    return Atoms, Domain


def _grid_atoms(Atoms):
    X, Y, Z = np.meshgrid(np.linspace(-20, 20, 41), np.linspace(-6, 6, 13), np.linspace(-6, 6, 13))
    atoms = Atoms(X.size)
    atoms.data["r"]["x"] = X.ravel()
    atoms.data["r"]["y"] = Y.ravel()
    atoms.data["r"]["z"] = Z.ravel()
    return atoms


def test_domain_calls_of_the_reference_script():
    Atoms, Domain = _dropin()
    domain = Domain(xmin=-10, xmax=10, ymin=-5, ymax=5, zmin=-5, zmax=5)
    domain.set_periodic(0, True)
    domain.set_periodic(1, True)
    assert (domain.xmin, domain.ymin, domain.zmin) == (-10, -5, -5)
    assert (domain.xmax, domain.ymax, domain.zmax) == (10, 5, 5)
    assert (domain.xsize, domain.ysize, domain.zsize) == (20, 10, 10)
    assert (domain.xperiodic, domain.yperiodic, domain.zperiodic) == (True, True, False)
    atoms = _grid_atoms(Atoms)
    do = R.Domain(-10, 10, -5, 5, -5, 5)
    do.set_periodic(0, True)
    do.set_periodic(1, True)
    r = np.stack([atoms.data["r"][c] for c in "xyz"], axis=1)
    inside = domain.belong(atoms)
    assert inside.dtype == np.int32
    assert np.array_equal(inside, [int(do.belong(v)) for v in r])
    assert domain.belong(0.0, 0.0, 0.0) and not domain.belong(11.0, 0.0, 0.0)
    for axis in range(3):
        got = domain.nearest_distance(atoms, axis)
        want = [do.nearest_distance(v, axis) for v in r]
        assert np.array_equal(got, want), axis


def test_fit_in_period_and_reshape():
    Atoms, Domain = _dropin()
    domain = Domain(0.0, 2.0, -1.0, 1.0, 0.0, 3.0)
    domain.set_periodic(0, True)
    domain.set_periodic(2, True)
    do = R.Domain(0.0, 2.0, -1.0, 1.0, 0.0, 3.0)
    do.set_periodic(0, True)
    do.set_periodic(2, True)
    rng = np.random.default_rng(3)
    atoms = Atoms(500)
    for c, (lo, hi) in zip("xyz", ((-1.5, 3.5), (-2.0, 2.0), (-2.0, 5.0))):
        atoms.data["r"][c] = rng.uniform(lo, hi, 500)
    r = np.stack([atoms.data["r"][c] for c in "xyz"], axis=1)
    domain.fit_in_period(atoms)
    got = np.stack([atoms.data["r"][c] for c in "xyz"], axis=1)
    want = np.array([do.fit_in_period(v.copy()) for v in r])
    assert np.array_equal(got, want)
    domain.reshape(xmin=1.0, xmax=4.0, ymin=0.0, ymax=2.0, zmin=0.0, zmax=0.0)
    assert (domain.xmin, domain.xmax, domain.ysize, domain.zsize) == (1.0, 4.0, 2.0, 0.0)
    assert domain.xperiodic and domain.zperiodic and not domain.yperiodic


def test_threads_counts_and_half_list_refusal():
    """tools::Threads (mdcraft/tools/threads.cxx:10-12,58-74): the count is
    capped at the hardware threads; a half VerletList with an active pool is
    refused before anything reaches the GPU (verlet-list.cxx:28-31)."""
    import pytest

    sys.path.insert(0, _DROPIN)
    try:
        from mdcraft.data import Atoms
        from mdcraft.lattice import Domain
        from mdcraft.neibs import VerletList
        from mdcraft.tools import Threads
    finally:
        sys.path.remove(_DROPIN)
    hw = max(1, os.cpu_count() or 1)
    t = Threads(4)
    assert t.count == min(4, hw)
    t.off()
    assert t.count == 1
    t.on(0)
    assert t.count == hw
    assert Threads().count == hw
    if hw < 2:
        pytest.skip("one hardware thread: no active pool")
    atoms = Atoms(2)
    with pytest.raises(RuntimeError, match="Half Verlet lists"):
        VerletList(atoms=atoms, neighbors=atoms, domain=Domain(0, 1, 0, 1, 0, 1), threads=Threads(2), half=True)
