"""Grid::build on the device without a list (mdg_grid_build, the C++
drop-in's neibs::Grid) against the oracle's Grid (mdcraft/neibs/grid.cxx:
43-95, 209-243): domain cells, local subgrid offset and size, cell sizes,
for open, periodic and mixed boxes with atoms filling part of the box, and
the empty system (Grid::initialize_empty, grid.cxx:26-34)."""
import numpy as np
import pytest

import mdcraft_gb300 as mdg
from oracle import mdref as R
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu


def _atoms(n, lo, hi, rns, seed):
    rng = np.random.default_rng(seed)
    a = mdg.new_atoms(n)
    a["r"] = rng.uniform(lo, hi, (n, 3))
    a["rns"] = rns
    a["rcut"] = rns
    a["m"] = 1.0
    return a


CASES = [
    ("open_corner", (0.0, 4.0, 0.0, 4.0, 0.0, 4.0), (0, 0, 0), (0.1, 0.1, 0.1), (2.7, 1.9, 0.9), 1.0),
    ("periodic_full", (-2.0, 2.0, -2.0, 2.0, -2.0, 2.0), (1, 1, 1), (-1.9, -1.9, -1.9), (1.9, 1.9, 1.9), 0.7),
    ("mixed_slab", (0.0, 6.0, 0.0, 3.0, 0.0, 9.0), (1, 0, 1), (0.2, 0.5, 3.0), (5.8, 2.5, 6.1), 0.45),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_grid_build_matches_oracle_and_rebuild(case):
    _, box, per, lo, hi, rns = case
    atoms = _atoms(500, lo, hi, rns, seed=4)
    do, dg = H.domains(box, per)
    sys = mdg.System(H.ctx(), dg, atoms)
    g = sys.grid_build()
    og = R.Grid(do)
    og.build(H.to_oracle_atoms(atoms))
    f = og.fields
    for k in ("domain_num_cells", "grid_offset", "num_cells"):
        assert list(g[k]) == list(f[k]), k
    assert np.array_equal(g["cell_sizes"], f["cell_sizes"])
    # the list rebuild's grid on the same atoms is the same
    nl = mdg.VerletList(sys)
    nl.update(-1.0)
    gl = nl.grid()
    for k in ("domain_num_cells", "grid_offset", "num_cells", "cell_sizes"):
        assert np.array_equal(gl[k], g[k]), k


def test_grid_build_empty_system():
    box = (0.0, 3.0, 0.0, 2.0, 0.0, 5.0)
    _, dg = H.domains(box, (0, 0, 0))
    sys = mdg.System(H.ctx(), dg, 0)
    g = sys.grid_build()
    assert list(g["domain_num_cells"]) == [1, 1, 1]
    assert list(g["grid_offset"]) == [1, 1, 1]
    assert list(g["num_cells"]) == [0, 0, 0]
    assert np.array_equal(g["cell_sizes"], [3.0, 2.0, 5.0])
