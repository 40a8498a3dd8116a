"""Host logic of the launch-shape autotuner (mdcraft_gb300.tune.tune_shapes)
on CPU with stand-ins for the system, list and stepper: it times every
candidate of each shape, keeps the fastest, leaves it set on the system,
skips the density budget for pair-only systems, and a second call with the
same GPU and workload signature takes the cached choice without measuring.
The force and density budgets are compared by per-launch device times,
which the list rebuilds inside the timed steps do not enter."""
import time

import pytest

from mdcraft_gb300 import tune


class _Ctx:
    """Stand-in for a Context's timing mode: per-stage (ms, launches)."""

    def __init__(self):
        self.timing = False
        self.acc = {}

    def synchronize(self):
        pass

    def set_timing(self, on=True):
        self.timing = bool(on)
        self.acc = {}

    def stage_time(self, stage):
        return self.acc.get(stage, (0.0, 0))

    def record(self, stage, seconds):
        if self.timing:
            ms, n = self.acc.get(stage, (0.0, 0))
            self.acc[stage] = (ms + seconds * 1e3, n + 1)


class _System:
    def __init__(self, eam=True):
        self.ctx = _Ctx()
        self.shape = {}
        self.calls = []
        self.eam = eam

    def set_shape(self, name, v):
        self.shape[name] = v
        self.calls.append((name, v))


# seconds per unit of work for each candidate: the fastest is unambiguous
_COST = {"list_cells_per_block": {2: 1.5e-3, 4: 5e-4, 8: 1e-3},
         "force_blocks_per_sm": {3: 1e-3, 4: 2.5e-4, 8: 6e-4},
         "density_blocks_per_sm": {3: 1e-3, 4: 1e-3, 5: 2.5e-4}}


class _List:
    def __init__(self, system):
        self.system = system

    def update(self, kbuf):
        time.sleep(_COST["list_cells_per_block"][self.system.shape["list_cells_per_block"]])


class _Stepper:
    """Each step: a force launch (and a density launch for EAM) whose device
    time is the candidate's cost, plus a rebuild every third step that the
    per-launch times must not see."""

    def run(self, system, dt, steps):
        for k in range(steps):
            system.ctx.record("forces", _COST["force_blocks_per_sm"][system.shape["force_blocks_per_sm"]])
            if system.eam:
                d = system.shape.get("density_blocks_per_sm", 4)
                system.ctx.record("density", _COST["density_blocks_per_sm"][d])
            if k % 3 == 2:
                system.ctx.record("rebuild", 1e-2)


@pytest.fixture
def cache(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setattr(tune, "CACHE", str(path))
    return path


def test_picks_fastest_and_caches(cache):
    s = _System()
    best, sec = tune.tune_shapes(s, _List(s), _Stepper(), 1e-3, signature="fake", steps=4, rebuilds=2)
    assert best == {"list_cells_per_block": 4, "force_blocks_per_sm": 4, "density_blocks_per_sm": 5}
    assert all(s.shape[k] == v for k, v in best.items())
    for name, cands in tune.SHAPE_CANDIDATES.items():
        assert sorted(sec[name]) == sorted(cands)
    assert cache.exists()
    # the same workload again: the cached choice, no measurement
    s2 = _System()
    best2, sec2 = tune.tune_shapes(s2, None, None, 1e-3, signature="fake")
    assert best2 == best and s2.shape == best
    assert sorted(sec2["force_blocks_per_sm"]) == [3, 4, 8]  # integer keys, as when measured
    assert sec["force_blocks_per_sm"][4] == pytest.approx(2.5e-4)  # per launch, rebuilds excluded
    assert len(s2.calls) == len(best)


def test_pair_only_system_skips_density(cache):
    s = _System(eam=False)
    best, sec = tune.tune_shapes(s, _List(s), _Stepper(), 1e-3, signature="pair", eam=False, steps=4,
                                 rebuilds=2, use_cache=False)
    assert set(best) == {"list_cells_per_block", "force_blocks_per_sm"}
    assert "density_blocks_per_sm" not in s.shape
    assert not cache.exists()
