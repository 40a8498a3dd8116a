"""The driver loop's host-facing forms: mdg_run_host (uploads, the graph
loop and downloads in stream order) equals upload + mdg_run + download, and
the graph loop's device-side prologue (rebuild test after an upload) equals
the host-side one of the stepwise loop."""
from __future__ import annotations

import numpy as np
import pytest

import mdcraft_gb300 as mdg
from mdcraft_gb300 import workloads as W
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu


def _pair(make, prec):
    atoms, box, per, p = make()
    _, g = H.make_pair(atoms, box, (1, 1, 1), p, precision=prec)
    g["nl"].update(-1.0)
    g["solver"].prepare(g["sys"])
    g["solver"].stages(g["sys"])
    return atoms, p, g


CASES = [(lambda: W.eam_cu_fcc(ncell=8), "mixed"), (lambda: W.lj_argon_fcc(jitter=0.01), "fp64"),
         (lambda: W.lj_argon_fcc(jitter=0.01), "mixed")]


def _host(x, pinned):
    """A copy of x in page-locked memory (torch's pinned allocator) or in
    ordinary memory."""
    if not pinned:
        return np.ascontiguousarray(np.array(x, dtype=np.float64))
    import torch
    t = torch.empty(np.shape(x), dtype=torch.float64, pin_memory=True)
    a = t.numpy()
    a[...] = x
    return a, t


@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "pinned"])
@pytest.mark.parametrize("make,prec", CASES, ids=["eam_mixed", "lj_fp64", "lj_mixed"])
def test_run_host_equals_run_and_download(make, prec, pinned):
    atoms, p, a = _pair(make, prec)
    a["stepper"].run(a["sys"], p["dt"], 50)
    ref = a["sys"].download()
    _, _, b = _pair(make, prec)
    keep = []
    if pinned:
        (pos, t1), (vel, t2), (frc, t3) = (_host(atoms["r"], True), _host(atoms["v"], True),
                                            _host(np.zeros_like(atoms["r"]), True))
        keep = [t1, t2, t3]
    else:
        pos, vel, frc = _host(atoms["r"], False), _host(atoms["v"], False), np.zeros((len(atoms), 3))
    b["stepper"].run_host(b["sys"], p["dt"], 50, pos, vel, frc)
    assert np.array_equal(pos, ref["r"])
    assert np.array_equal(vel, ref["v"])
    assert np.array_equal(frc, ref["f"])
    assert a["nl"].rebuilds() == b["nl"].rebuilds()
    del keep


@pytest.mark.parametrize("pinned", [False, True], ids=["pageable", "pinned"])
@pytest.mark.parametrize("make,prec", CASES, ids=["eam_mixed", "lj_fp64", "lj_mixed"])
def test_one_step_host_calls_equal_run(make, prec, pinned):
    """A host loop of one-step mdg_run_host calls (pinned buffers: result
    downloads overlapped with the step; pageable: the graph path) gives the
    bits of mdg_run over the same steps, rebuilds included."""
    atoms, p, a = _pair(make, prec)
    a["stepper"].run(a["sys"], p["dt"], 60)
    ref = a["sys"].download()
    _, _, b = _pair(make, prec)
    keep = []
    if pinned:
        (pos, t1), (vel, t2), (frc, t3) = (_host(atoms["r"], True), _host(atoms["v"], True),
                                            _host(np.zeros_like(atoms["r"]), True))
        keep = [t1, t2, t3]
    else:
        pos, vel, frc = _host(atoms["r"], False), _host(atoms["v"], False), np.zeros((len(atoms), 3))
    for step in range(60):
        b["stepper"].run_host(b["sys"], p["dt"], 1, pos, vel, frc if step % 2 == 0 else None)
    assert np.array_equal(pos, ref["r"])
    assert np.array_equal(vel, ref["v"])
    assert np.array_equal(b["sys"].forces(), ref["f"])
    assert a["nl"].rebuilds() == b["nl"].rebuilds()
    del keep


def test_one_step_host_calls_through_rebuilds():
    """Hot atoms: the one-step overlapped path rebuilds often (positions are
    sent again after each rebuild's wrap) and still matches mdg_run."""
    make = lambda: W.eam_cu_fcc(ncell=8, T=3000.0)
    atoms, p, a = _pair(make, "mixed")
    a["stepper"].run(a["sys"], p["dt"], 40)
    ref = a["sys"].download()
    _, _, b = _pair(make, "mixed")
    (pos, t1), (vel, t2), (frc, t3) = (_host(atoms["r"], True), _host(atoms["v"], True),
                                        _host(np.zeros_like(atoms["r"]), True))
    for _ in range(40):
        b["stepper"].run_host(b["sys"], p["dt"], 1, pos, vel, frc)
    assert b["nl"].rebuilds() == a["nl"].rebuilds() >= 3
    assert np.array_equal(pos, ref["r"])
    assert np.array_equal(vel, ref["v"])
    assert np.array_equal(frc, ref["f"])
    del t1, t2, t3


@pytest.mark.parametrize("make", [lambda: W.eam_cu_fcc(ncell=8), lambda: W.lj_argon_fcc(jitter=0.01)],
                         ids=["eam", "lj"])
def test_graph_prologue_rebuilds_after_upload(make):
    """Positions moved past the half skin by an upload: the graph loop's
    prologue rebuilds on the device, as the stepwise loop's host prologue
    does; the two runs give the same bits."""
    out = []
    for timing in (False, True):
        atoms, p, g = _pair(make, "mixed")
        g["stepper"].run(g["sys"], p["dt"], 5)
        r = g["sys"].positions()
        rng = np.random.default_rng(9)
        r = r + rng.uniform(-1, 1, r.shape) * 0.6 * p["skin"]
        g["sys"].set_positions(np.ascontiguousarray(r))
        rb0 = g["nl"].rebuilds()
        ctx = g["sys"].ctx
        ctx.set_timing(timing)
        g["stepper"].run(g["sys"], p["dt"], 20)
        ctx.set_timing(False)
        out.append((g["sys"].download(), g["nl"].rebuilds() - rb0))
    (a, ra), (b, rb) = out
    assert ra == rb and ra >= 1
    for k in ("r", "v", "f"):
        assert np.array_equal(a[k], b[k]), k


def _tagged(make):
    def f():
        atoms, box, per, p = make()
        atoms["tag"][::17] = 0  # held in place: no kick, no drift (verlet.cxx:36-85)
        return atoms, box, per, p
    return f


@pytest.mark.parametrize("make", [_tagged(lambda: W.eam_cu_fcc(ncell=8, T=3000.0)),
                                  _tagged(lambda: W.lj_argon_fcc(ncell=6, T=600.0, jitter=0.01)),
                                  lambda: W.eam_nial_b2(ncell=8, T=3000.0)],
                         ids=["eam_hot_tagged", "lj_hot_tagged", "nial_multi_hot"])
def test_step_loop_equals_stepwise_api(make):
    """mdg_run's mixed step loop starts each next step inside the force pass
    (its epilogue runs the next half-kick, drift, offsets refresh and rebuild
    test); the stepwise API (make_step, decide, update) runs those as passes
    of their own. Same bits, rebuilds included."""
    atoms, p, a = _pair(make, "mixed")
    a["stepper"].run(a["sys"], p["dt"], 40)
    ref = a["sys"].download()
    _, _, b = _pair(make, "mixed")
    for _ in range(40):
        b["stepper"].make_step(b["sys"], p["dt"])
        if b["nl"].decide():
            b["nl"].update(-1.0)
    got = b["sys"].download()
    assert b["nl"].rebuilds() == a["nl"].rebuilds() >= 2
    assert np.array_equal(got["r"], ref["r"])
    assert np.array_equal(got["v"], ref["v"])
    assert np.array_equal(got["f"], ref["f"])
    frozen = np.asarray(atoms["tag"]) == 0
    if frozen.any():
        assert np.array_equal(ref["v"][frozen], np.asarray(atoms["v"])[frozen])
