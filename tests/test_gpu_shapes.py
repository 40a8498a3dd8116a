"""Launch shapes of a system's step kernels (list cells per block, register
budgets of the mixed force and density passes). A shape changes how the work
is laid out on the SMs, never the arithmetic: the neighbour lists and every
force and position must be bit for bit those of the default shapes, and the
tuner must pick among the candidates it measured."""
import numpy as np
import pytest

import mdcraft_gb300 as mdg
from mdcraft_gb300 import tune
from mdcraft_gb300 import workloads as W
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu


def _system(kind, precision="mixed"):
    if kind == "eam":
        atoms, box, per, p = W.eam_cu_fcc(ncell=10)
    else:
        atoms, box, per, p = W.eam_nial_b2(ncell=10)
    o, g = H.make_pair(atoms, box, (1, 1, 1), p, precision=precision)
    return atoms, g


def _state(g, steps=15, dt=0.001):
    g["sys"].upload(g["atoms0"])
    g["nl"].update(-1.0)
    off, idx = g["nl"].csr()
    g["solver"].prepare(g["sys"])
    g["solver"].stages(g["sys"])
    f0 = g["sys"].forces().copy()
    g["stepper"].run(g["sys"], dt, steps)
    d = g["sys"].download()
    return off, idx, f0, d["r"].copy(), d["v"].copy()


@pytest.mark.parametrize("kind", ["eam", "multi"])
def test_shapes_do_not_change_results(kind):
    atoms, g = _system(kind)
    g["atoms0"] = atoms
    s = g["sys"]
    ref = _state(g)
    for name, cands in tune.SHAPE_CANDIDATES.items():
        for v in cands:
            s.set_shape(name, v)
            assert s.get_shape(name) == v
            got = _state(g)
            for a, b in zip(ref, got):
                assert np.array_equal(a, b), (name, v)
        s.set_shape(name, 0)


def test_shape_values_checked():
    atoms, g = _system("eam")
    s = g["sys"]
    for name, bad in (("list_cells_per_block", 3), ("force_blocks_per_sm", 5), ("density_blocks_per_sm", 2)):
        with pytest.raises(RuntimeError):
            s.set_shape(name, bad)
        assert s.get_shape(name) == 0


def test_tuner_picks_a_candidate():
    atoms, g = _system("eam")
    g["atoms0"] = atoms
    s = g["sys"]
    g["nl"].update(-1.0)
    g["solver"].prepare(s)
    g["solver"].stages(s)
    best, sec = tune.tune_shapes(s, g["nl"], g["stepper"], 0.001, signature="test_eam_cu_4000", eam=True,
                                 steps=4, rebuilds=2, use_cache=False)
    assert set(best) == set(tune.SHAPE_CANDIDATES)
    for name, v in best.items():
        assert v in tune.SHAPE_CANDIDATES[name]
        assert s.get_shape(name) == v
        assert set(sec[name]) == set(tune.SHAPE_CANDIDATES[name])
        assert all(t > 0.0 for t in sec[name].values())
