"""CPU check of the oracle's Verlet lists against a brute-force pair search
(no GPU).

The reference's list (VerletList::build_linked_cells and are_neibs,
mdcraft/neibs/verlet-list.cxx:306-400, over Grid::adjacent_cells,
mdcraft/neibs/grid.cxx:138-207) walks the 27 neighbour cells, or fewer on
periodic axes of one or two cells, and takes the minimum image only for edge
cells. When every atom lies inside the grid and every periodic edge is at
least 2 max(rns), that walk must find exactly the pairs whose nearest-image
distance satisfies d^2 <= max(rns_i, rns_j)^2, self included. A half list
keeps the j >= i of them (verlet-list.cxx:345). The brute-force search
below states that set directly over all pairs.
"""
import numpy as np
import pytest

from mdcraft_gb300 import workloads as W
from oracle import mdref as R


def _oracle_atoms(k):
    a = np.zeros(len(k), dtype=R.ATOM_DTYPE)
    a.view(np.uint8)[:] = np.ascontiguousarray(k).view(np.uint8)
    return a


def _brute(a, box, per):
    r, rns = a["r"], a["rns"]
    L = np.array([box[1] - box[0], box[3] - box[2], box[5] - box[4]])
    out = []
    for i in range(len(a)):
        d = r - r[i]
        for k in range(3):
            if per[k]:
                d[:, k] -= L[k] * np.round(d[:, k] / L[k])
        d2 = (d * d).sum(axis=1)
        out.append(set(np.nonzero(d2 <= np.maximum(rns, rns[i]) ** 2)[0].tolist()))
    return out


def _gas(n=1500, edge=5.0, seed=11):
    rng = np.random.default_rng(seed)
    g = R.new_atoms(n)
    g["r"] = rng.random((n, 3)) * edge
    g["rns"] = 0.3 + 0.2 * rng.random(n)
    g["rcut"] = 0.25
    g["m"] = 1.0
    return g, (0.0, edge, 0.0, edge, 0.0, edge)


def _lattice(made):
    atoms, box, _, _ = made
    return _oracle_atoms(atoms), box


CASES = [
    ("lj_argon_3cells", lambda: _lattice(W.lj_argon_fcc(ncell=6, jitter=0.02)), (1, 1, 1)),
    ("eam_cu_3cells", lambda: _lattice(W.eam_cu_fcc(ncell=6)), (1, 1, 1)),
    ("eam_cu_2cells", lambda: _lattice(W.eam_cu_fcc(ncell=4)), (1, 1, 1)),
    ("nial_b2_3cells", lambda: _lattice(W.eam_nial_b2(ncell=8)), (1, 1, 1)),
    ("gas_mixed_rns_open", _gas, (0, 0, 0)),
    ("gas_mixed_rns_periodic", _gas, (1, 1, 1)),
    ("gas_mixed_rns_slab", _gas, (1, 1, 0)),
]


@pytest.mark.parametrize("half", [False, True], ids=["full", "half"])
@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_lists_equal_brute_force_pairs(case, half):
    name, make, per = case
    atoms, box = make()
    d = R.Domain(*box)
    for k in range(3):
        if per[k]:
            d.set_periodic(k, True)
    nl = R.VerletList(atoms, d, threads=1, half=half)
    nl.update(-1.0)
    got = [set(map(int, x)) for x in nl.lists()]
    want = _brute(atoms, box, per)
    if half:
        want = [{j for j in s if j >= i} for i, s in enumerate(want)]
    assert got == want


@pytest.mark.parametrize("half", [False, True], ids=["full", "half"])
def test_lists_equal_brute_force_pairs_random_boxes(half):
    """60 seeded random systems: 2 to 400 atoms, rns in [0.2, 0.5], box edges
    in [1, 4] (at least 2 max(rns), so 2 to 8 cells per axis), and each
    axis periodic or open at random."""
    rng = np.random.default_rng(123)
    for _ in range(60):
        n = int(rng.integers(2, 400))
        per = tuple(int(x) for x in rng.integers(0, 2, 3))
        edges = rng.uniform(1.0, 4.0, 3)
        box = (0.0, edges[0], 0.0, edges[1], 0.0, edges[2])
        a = R.new_atoms(n)
        a["r"] = rng.random((n, 3)) * edges
        a["rns"] = rng.uniform(0.2, 0.5, n)
        a["rns"][0] = 0.5
        a["rcut"] = 0.1
        a["m"] = 1.0
        d = R.Domain(*box)
        for k in range(3):
            if per[k]:
                d.set_periodic(k, True)
        nl = R.VerletList(a, d, threads=1, half=half)
        nl.update(-1.0)
        want = _brute(a, box, per)
        if half:
            want = [{j for j in s if j >= i} for i, s in enumerate(want)]
        assert [set(map(int, x)) for x in nl.lists()] == want, (n, per, edges)


def test_decide_is_the_half_skin_rule():
    """VerletList::decide (mdcraft/neibs/verlet-list.cxx:110-158): a rebuild
    is due when some atom moved, by the nearest periodic image, more than
    half its skin (rns - rcut) since the last update, or changed its uid,
    rcut or rns. Random displacements near the threshold, some of them
    wrapped back across a periodic face (which is no motion), on 200 trials."""
    rng = np.random.default_rng(5)
    L = np.array([3.0, 3.0, 3.0])
    box = (0.0, 3.0, 0.0, 3.0, 0.0, 3.0)
    for trial in range(200):
        n = 50
        a = R.new_atoms(n)
        a["r"] = rng.random((n, 3)) * L
        a["rns"] = rng.uniform(0.3, 0.5, n)
        a["rcut"] = a["rns"] - rng.uniform(0.05, 0.2, n)
        a["m"] = 1.0
        a["uid"] = np.arange(1, n + 1)
        d = R.Domain(*box)
        per = (1, 1, trial % 2)
        for k in range(3):
            if per[k]:
                d.set_periodic(k, True)
        nl = R.VerletList(a, d, threads=1)
        nl.update(-1.0)
        r0 = a["r"].copy()
        half = 0.5 * (a["rns"] - a["rcut"])
        # each atom moves by a fraction of its half skin in a random direction
        u = rng.normal(size=(n, 3))
        u /= np.linalg.norm(u, axis=1)[:, None]
        frac = rng.uniform(0.0, 0.999, n)
        if trial % 4 == 1:
            frac[rng.integers(n)] = rng.uniform(1.001, 1.5)
        a["r"] = r0 + u * (frac * half)[:, None]
        # wrap some coordinates back into the box on periodic axes: no motion
        for k in range(3):
            if per[k]:
                a["r"][:, k] = np.where(rng.random(n) < 0.5, np.mod(a["r"][:, k], L[k]), a["r"][:, k])
        dr = a["r"] - r0
        for k in range(3):
            if per[k]:
                dr[:, k] -= L[k] * np.round(dr[:, k] / L[k])
        want = bool(np.any((dr * dr).sum(axis=1) > half * half))
        assert nl.decide() == want, trial
        if trial % 10 == 0 and not want:
            a["rns"][3] += 1e-12
            assert nl.decide()


def test_list_for_equals_brute_force_in_cubic_grids():
    """VerletList::list_for (mdcraft/neibs/verlet-list.cxx:251-276) keeps the
    atoms of the point's adjacent cells within max(cell_size, rns_j) of it,
    cell_size being the largest cell edge (mdcraft/neibs/grid.h:116). In a
    cube with equal cells every atom within that radius (nearest image on
    periodic axes) lies in those cells, so the result is the brute-force
    set: 40 random gases, periodic or open, 10 query points each."""
    rng = np.random.default_rng(9)
    for trial in range(40):
        n = int(rng.integers(20, 500))
        edge = rng.uniform(1.0, 4.0)
        periodic = trial % 2 == 0
        box = (0.0, edge, 0.0, edge, 0.0, edge)
        a = R.new_atoms(n)
        a["r"] = rng.random((n, 3)) * edge
        a["rns"] = rng.uniform(0.2, 0.5, n)
        a["rns"][0] = 0.5
        a["rcut"] = 0.1
        a["m"] = 1.0
        d = R.Domain(*box)
        if periodic:
            for k in range(3):
                d.set_periodic(k, True)
        nl = R.VerletList(a, d, threads=1)
        nl.update(-1.0)
        radius = np.maximum(nl.grid().fields["cell_sizes"].max(), a["rns"])
        lo, hi = a["r"].min(axis=0), a["r"].max(axis=0)
        for _ in range(10):
            x = lo + rng.random(3) * (hi - lo)
            dd = a["r"] - x
            if periodic:
                dd -= edge * np.round(dd / edge)
            want = set(np.nonzero((dd * dd).sum(axis=1) <= radius * radius)[0].tolist())
            assert set(map(int, nl.list_for(x))) == want, (trial, x)
