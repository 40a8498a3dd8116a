"""VerletList::sort (mdcraft/neibs/verlet-list.cxx:237-249) through the C-ABI
(mdg_nlist_sort) against the oracle's restatement: the caller's atoms are
wrapped in place and the copy lists them by Grid::cell_index, x fastest,
ascending index inside a cell. Records are compared byte for byte."""
import os
import sys

import numpy as np
import pytest

import mdcraft_gb300 as mdg
from mdcraft_gb300 import workloads as W
from oracle import mdref as R
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu


def _random_atoms(n, lo, hi, rns, seed):
    rng = np.random.default_rng(seed)
    a = np.zeros(n, dtype=mdg.ATOM_DTYPE)
    a["r"] = rng.uniform(lo, hi, (n, 3))
    a["v"] = rng.normal(size=(n, 3))
    a["rns"] = rns
    a["rcut"] = 0.9 * rns
    a["m"] = 1.0
    a["uid"] = np.arange(1, n + 1)
    a["kind"] = rng.integers(0, 3, n)
    a["tag"] = 0xFFFF  # moved by the stepper (tag 0 atoms stay put)
    return a


def _both(atoms, box, periodic):
    do, dg = H.domains(box, periodic)
    sysg = mdg.System(H.ctx(), dg, atoms)
    nlg = mdg.VerletList(sysg)
    ag, ao = atoms.copy(), H.to_oracle_atoms(atoms)
    sg = nlg.sort(ag)
    so = R.sort_atoms(do, ao)
    b = lambda x: np.ascontiguousarray(x).view(np.uint8)
    assert np.array_equal(b(ag), b(ao)), "wrapped atoms differ"
    assert np.array_equal(b(sg), b(so)), "sorted copies differ"
    return sg, nlg


@pytest.mark.parametrize("periodic", [(1, 1, 1), (0, 0, 0), (1, 0, 1)])
def test_sort_random_boxes(periodic):
    box = (0.0, 3.1, -1.0, 1.4, 0.5, 2.9)
    atoms = _random_atoms(3000, (-0.3, -1.2, 0.3), (3.4, 1.6, 3.1), 0.37, seed=sum(periodic) + 3)
    for a in range(3):
        if not periodic[a]:  # inside the box on axes without a period
            lo, hi = box[2 * a], box[2 * a + 1]
            atoms["r"][:, a] = np.clip(atoms["r"][:, a], lo, hi - 1e-9)
    _both(atoms, box, periodic)


def test_sort_small_periodic_box_and_ragged_cells():
    # 2 and 3 cells on periodic axes (the reference's n = 2 rule), most cells
    # empty or nearly so
    box = (0.0, 1.0, 0.0, 1.5, 0.0, 8.0)
    atoms = _random_atoms(40, (0.0, 0.0, 0.0), (1.0, 1.5, 8.0), 0.49, seed=11)
    _both(atoms, box, (1, 1, 1))


def test_sort_eam_lattice_and_list_untouched():
    atoms, box, per, p = W.eam_cu_fcc(ncell=12)
    per = (1, 1, 1)
    do, dg = H.domains(box, per)
    sysg = mdg.System(H.ctx(), dg, atoms)
    nlg = mdg.VerletList(sysg)
    nlg.update(-1.0)
    before = nlg.csr()
    _both(atoms, box, per)
    ag = atoms.copy()
    sg = nlg.sort(ag)
    after = nlg.csr()
    assert all(np.array_equal(x, y) for x, y in zip(before, after))
    # sorted by cell: the cell index never decreases
    g = R.Grid(do)
    g.build(H.to_oracle_atoms(ag))
    cells = np.array([g.cell_index(g.local_index3D(r)) for r in sg["r"]])
    assert np.all(np.diff(cells) >= 0)


def test_sort_known_answer_and_empty():
    # test/cxx/neibs/test_verlet_list.cxx:107-122
    a = np.zeros(3, dtype=mdg.ATOM_DTYPE)
    a["r"] = [(1.60, 0.10, 0.10), (0.15, 0.10, 0.10), (0.95, 0.10, 0.10)]
    a["rcut"] = a["rns"] = 0.40
    a["m"] = 1.0
    sg, nlg = _both(a, (0.0, 2.0, 0.0, 1.0, 0.0, 1.0), (0, 0, 0))
    assert sg["r"][0][0] < sg["r"][1][0] < sg["r"][2][0]
    empty = np.zeros(0, dtype=mdg.ATOM_DTYPE)
    assert len(nlg.sort(empty)) == 0


def test_sort_python_dropin():
    H.ctx()
    here = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "mdcraft_gb300", "dropin")
    sys.path.insert(0, here)
    try:
        from mdcraft.data import Atoms
        from mdcraft.lattice import Domain
        from mdcraft.neibs import VerletList
    finally:
        sys.path.remove(here)
    atoms = Atoms(3)
    atoms.data["r"]["x"] = [1.60, 0.15, 0.95]
    atoms.data["r"]["y"] = 0.10
    atoms.data["r"]["z"] = 0.10
    atoms.data["rcut"] = atoms.data["rns"] = 0.40
    atoms.data["m"] = 1.0
    nl = VerletList(atoms=atoms, neighbors=atoms, domain=Domain(0.0, 2.0, 0.0, 1.0, 0.0, 1.0))
    out = nl.sort(atoms)
    assert list(out.data["r"]["x"]) == [0.15, 0.95, 1.60]


@pytest.mark.parametrize("periodic", [(1, 1, 1), (1, 0, 1)])
def test_list_for_matches_oracle(periodic):
    """VerletList::list_for (verlet-list.cxx:251-276) on a random system:
    query points in every kind of cell (faces, edges, interior), on the first
    list and again after steps (rebuilds inside the device loop) and a
    rebuild, against the oracle's list_for on the same atoms."""
    box = (0.0, 2.6, -1.0, 1.3, 0.5, 2.8)
    atoms = _random_atoms(1500, (0.0, -1.0, 0.5), (2.6, 1.3, 2.8), 0.33, seed=5 + periodic[1])
    do, dg = H.domains(box, periodic)
    sysg = mdg.System(H.ctx(), dg, atoms)
    nlg = mdg.VerletList(sysg)
    nlg.update(-1.0)
    rng = np.random.default_rng(21)
    lo = np.array([box[0], box[2], box[4]])
    hi = np.array([box[1], box[3], box[5]])
    queries = np.concatenate([rng.uniform(lo, hi, (40, 3)), [lo + 0.01], [hi - 0.01],
                              np.array([[lo[0] + 0.001, 0.0, hi[2] - 0.001], [hi[0] - 0.02, lo[1] + 0.02, 1.6]])])

    def compare():
        ao = H.to_oracle_atoms(sysg.download())
        nlo = R.VerletList(ao, do, threads=1)
        nlo.update(-1.0)  # wrapped already: the same grid as the device's last rebuild
        for x in queries:
            assert list(nlg.list_for(x)) == sorted(nlo.list_for(x)), x
        # the exported list (CSR in caller order, each atom's entries ascending)
        off, idx = nlg.csr()
        lists_o = nlo.lists()
        for i in range(len(ao)):
            assert np.array_equal(idx[off[i]:off[i + 1]], np.sort(np.asarray(lists_o[i], dtype=np.uint64))), i

    compare()
    # free flight (a zero-strength LJsCut) along the periodic axes, with
    # rebuilds inside the device loop, then a rebuild on the final positions
    v = rng.normal(0.0, 2.0, (len(atoms), 3))
    for a in range(3):
        if not periodic[a]:
            v[:, a] = 0.0
    sysg.set_velocities(v)
    pot = mdg.LJsCut(0.0, 0.1, 0.3)
    solver = mdg.Single(pot, periodic=True)
    solver.prepare(sysg)
    solver.stages(sysg)
    mdg.Verlet(solver).run(sysg, 0.002, 60)
    assert nlg.rebuilds() >= 3
    nlg.update(-1.0)
    compare()
