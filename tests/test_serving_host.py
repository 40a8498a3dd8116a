"""Host-side pieces of the serving loop: the request stream generator and
the admission footprint (no GPU)."""
from __future__ import annotations

import math

import numpy as np

from mdcraft_gb300 import workloads as W


def test_stream_shape():
    s = W.serving_stream()
    assert len(s) == 4096
    n = np.array([x["n"] for x in s])
    assert n.min() >= 256 and n.max() <= 4 * 21 ** 3
    assert abs(np.mean([x["kind"] == "lj" for x in s]) - 0.6) < 0.03
    t = np.array([x["t_arrival"] for x in s])
    assert np.all(np.diff(t) > 0)
    assert abs(len(s) / t[-1] - 2000.0) < 100.0
    # log-uniform sizes: the median sits near the geometric mean of the range
    assert 0.7 < np.median(n) / math.sqrt(256 * 32768) < 1.4
    for x in s:
        p = W.SERVE_LJ if x["kind"] == "lj" else W.SERVE_EAM
        # every box edge holds two list radii (the periodic grid needs 2 cells)
        assert min(x["dims"]) * p["a"] >= 2 * (p["rcut"] + p["skin"])


def test_request_atoms_are_seeded():
    spec = W.serving_stream(count=3)[1]
    a1, box1 = W.serving_atoms(spec)
    a2, box2 = W.serving_atoms(spec)
    assert box1 == box2 and len(a1) == spec["n"]
    assert np.array_equal(a1["r"], a2["r"]) and np.array_equal(a1["v"], a2["v"])
    L = np.array([box1[1], box1[3], box1[5]])
    assert np.all(a1["r"] >= 0) and np.all(a1["r"] < L)
    p = (a1["m"][:, None] * a1["v"]).sum(axis=0)
    assert np.all(np.abs(p) < 1e-9)


def test_footprint_monotone():
    import mdcraft_gb300 as mdg
    f = mdg.Server.footprint
    assert f(256, 60) < f(4096, 60) < f(32768, 60)
    assert f(4096, 60) < f(4096, 120)
    # per-atom cost of a dense request: a few hundred bytes of state plus the list
    assert 500 < f(32768, 80) / 32768 < 3000
