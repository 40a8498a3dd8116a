"""Serving loop (mdg_server_*): results do not depend on the mix, match the
plain driver loop bit for bit and the oracle in the FP64 form; admission
respects the device-memory budget."""
from __future__ import annotations

import numpy as np
import pytest

import mdcraft_gb300 as mdg
from mdcraft_gb300 import serving as SV
from mdcraft_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _ensure_built():
    from tests import gpu_helpers as H
    H.ctx()


def _direct(spec, solv):
    """The plain driver loop through the single-system API: update(-1),
    prepare, stages, then the steps."""
    from tests import gpu_helpers as H
    atoms, box = W.serving_atoms(spec)
    dom = SV.periodic_domain(box)
    s = mdg.System(H.ctx(), dom, atoms)
    nl = mdg.VerletList(s)
    nl.update(-1.0)
    sol = solv[spec["kind"]]
    sol.prepare(s)
    sol.stages(s)
    mdg.Verlet(sol).run(s, spec["dt"], spec["steps"])
    out = s.download()
    s.close()
    return out


def _same(a, b):
    return all(np.array_equal(a[k], b[k]) for k in ("r", "v", "f"))


def _specs(count, steps, seed=11, n_max=4000):
    return W.serving_stream(count=count, rate=1e9, seed=seed, steps=steps, n_min=256, n_max=n_max)


def test_result_same_alone_and_in_mix():
    _ensure_built()
    solv = SV.solvers("mixed")
    specs = _specs(10, 60)
    reqs = SV.prepare(specs)
    probe = 3
    # alone: a one-slot server with nothing else queued
    alone = mdg.Server(slots=1, max_atoms=8192)
    s, atoms, dom = reqs[probe]
    rid = alone.submit(solv[s["kind"]], dom, atoms, s["dt"], s["steps"])
    alone.wait(rid, 120.0)
    a_alone, info = alone.result(rid)
    assert info["status"] == 0 and info["done"] == 1
    alone.close()
    # in the mix: all ten at once on four slots, overlapping on the device
    mix = mdg.Server(slots=4, max_atoms=8192)
    ids = [mix.submit(solv[s["kind"]], dom, atoms, s["dt"], s["steps"]) for s, atoms, dom in reqs]
    outs = {}
    for k, rid in enumerate(ids):
        mix.wait(rid, 300.0)
        outs[k], info = mix.result(rid)
        assert info["status"] == 0
    st = mix.stats()
    assert st["admitted"] == 10 and st["finished"] == 10 and st["used"] == 0
    mix.close()
    assert _same(outs[probe], a_alone)
    # and every request equals the plain single-system driver loop
    for k in (0, probe, 7):
        assert _same(outs[k], _direct(specs[k], solv)), f"request {k}"


@pytest.mark.parametrize("dims", [(4, 4, 4), (6, 6, 8)], ids=["2_cells", "3_cells"])
def test_small_boxes_two_cells_per_dimension(dims):
    """The smallest requests (4^3 fcc cells, 2 grid cells per dimension: the
    reference's n = 2 rule; 6x6x8 cells, 3 grid cells on two axes): mixed
    forces within the bar of the FP64 ones on the same positions, and mixed
    vs FP64 runs through the server."""
    _ensure_built()
    from tests import gpu_helpers as H
    n = 4 * dims[0] * dims[1] * dims[2]
    specs = [dict(index=0, kind=k, dims=dims, n=n, t_arrival=0.0, steps=40, dt=p["dt"], seed=77 + j)
             for j, (k, p) in enumerate((("lj", W.SERVE_LJ), ("eam", W.SERVE_EAM)))]
    s64, smx = SV.solvers("fp64"), SV.solvers("mixed")
    for spec in specs:
        atoms, box = W.serving_atoms(spec)
        s = mdg.System(H.ctx(), SV.periodic_domain(box), atoms)
        nl = mdg.VerletList(s)
        nl.update(-1.0)
        f = {}
        for name, solv in (("fp64", s64), ("mixed", smx)):
            solv[spec["kind"]].prepare(s)
            solv[spec["kind"]].stages(s)
            f[name] = s.forces()
        emax, el2 = H.force_error(f["mixed"], f["fp64"])
        assert el2 <= 1e-5 and emax <= 5e-4, (spec["kind"], emax, el2)
        s.close()
    out = {}
    for prec, solv in (("fp64", s64), ("mixed", smx)):
        srv = mdg.Server(slots=2, max_atoms=max(1024, n))
        reqs = SV.prepare(specs)
        ids = [srv.submit(solv[s["kind"]], d, a, s["dt"], s["steps"]) for s, a, d in reqs]
        for k, rid in enumerate(ids):
            srv.wait(rid, 120.0)
            out[(prec, k)], info = srv.result(rid)
            assert info["status"] == 0
        srv.close()
    for k in range(2):
        assert np.max(np.abs(out[("mixed", k)]["r"] - out[("fp64", k)]["r"])) < 1e-5


def test_served_fp64_matches_oracle():
    """A request in the FP64 form against the oracle's driver loop."""
    _ensure_built()
    from oracle import mdref as R
    from tests import gpu_helpers as H
    spec = _specs(1, 30, seed=21, n_max=2000)[0]
    spec["kind"] = "lj"
    spec["dt"] = W.SERVE_LJ["dt"]
    atoms, box = W.serving_atoms(spec)
    lj = W.SERVE_LJ
    params = dict(kind="lj", a=lj["eps"], s=lj["sigma"], rcut=lj["rcut"])
    o, _ = H.make_pair(atoms, box, (1, 1, 1), params, precision="fp64")
    o["nl"].update(-1.0)
    o["solver"].prepare(o["atoms"])
    o["solver"].stages(o["atoms"], o["nl"])
    o["solver"].run(o["atoms"], o["nl"], o["dom"], spec["dt"], spec["steps"])
    solv = SV.solvers("fp64")
    srv = mdg.Server(slots=2, max_atoms=4096)
    rid = srv.submit(solv["lj"], SV.periodic_domain(box), atoms, spec["dt"], spec["steps"])
    srv.wait(rid, 120.0)
    a, info = srv.result(rid)
    srv.close()
    assert info["status"] == 0
    assert np.max(np.abs(a["r"] - o["atoms"]["r"])) < 1e-9
    assert np.max(np.abs(a["v"] - o["atoms"]["v"])) < 1e-9
    del R


def test_admission_by_footprint():
    """A budget that holds one request at a time serialises them; a request
    larger than the whole budget is refused at submission."""
    _ensure_built()
    solv = SV.solvers("mixed")
    # equal sizes: any two together exceed the budget, one always fits
    specs = [dict(index=j, kind=("lj", "eam")[j % 2], dims=(6, 6, 6), n=864, t_arrival=0.0, steps=20,
                  dt=(W.SERVE_LJ, W.SERVE_EAM)[j % 2]["dt"], seed=31 + j) for j in range(4)]
    reqs = SV.prepare(specs)
    budget = int(1.5 * mdg.Server.footprint(864, 90))
    srv = mdg.Server(slots=4, hbm_budget=budget, max_atoms=8192)
    ids = [srv.submit(solv[s["kind"]], d, a, s["dt"], s["steps"]) for s, a, d in reqs]
    running_max = 0
    while srv.stats()["finished"] < len(ids):
        running_max = max(running_max, srv.progress())
        st = srv.stats()
        assert st["used"] <= budget or st["running"] == 1
    st = srv.stats()
    assert st["peak"] <= budget
    assert running_max == 1
    for rid in ids:
        _, info = srv.result(rid, atoms=False)
        assert info["status"] == 0
    big = W.serving_atoms(dict(kind="eam", dims=(12, 12, 12), seed=1))
    with pytest.raises(mdg.MDGError) as e:
        srv.submit(solv["eam"], SV.periodic_domain(big[1]), big[0], 0.001, 10)
    assert e.value.code == -2
    srv.close()


def test_first_list_overflow_takes_checked_path():
    """Two dense fcc slabs at the ends of a long periodic box: the grid spans
    the box, so the host-side capacity estimate from the mean density is too
    small, the first list overflows, and the request is repeated on the
    checked path. Its result equals the plain driver loop's."""
    _ensure_built()
    from tests import gpu_helpers as H
    p = W.SERVE_LJ
    a = p["a"]
    base = W.fcc_positions(16, 4, 4, a) + 0.25 * a
    cell_x = np.floor(base[:, 0] / a).astype(int)
    keep = (cell_x < 4) | (cell_x >= 12)
    r = base[keep]
    atoms = mdg.new_atoms(len(r))
    atoms["r"] = r
    atoms["m"] = p["mass"]
    atoms["rcut"] = p["rcut"]
    atoms["rns"] = p["rcut"] + p["skin"]
    atoms["uid"] = np.arange(1, len(r) + 1)
    rng = np.random.default_rng(5)
    atoms["v"] = W.maxwell_boltzmann(rng, atoms["m"].copy(), 300.0)
    box = (0.0, 16 * a, 0.0, 4 * a, 0.0, 4 * a)
    solv = SV.solvers("mixed")
    srv = mdg.Server(slots=2, max_atoms=4096)
    rid = srv.submit(solv["lj"], SV.periodic_domain(box), atoms, p["dt"], 30)
    srv.wait(rid, 120.0)
    out, info = srv.result(rid)
    st = srv.stats()
    srv.close()
    assert info["status"] == 0
    assert st["rechecked"] == 1
    s = mdg.System(H.ctx(), SV.periodic_domain(box), atoms)
    nl = mdg.VerletList(s)
    nl.update(-1.0)
    solv["lj"].prepare(s)
    solv["lj"].stages(s)
    mdg.Verlet(solv["lj"]).run(s, p["dt"], 30)
    assert _same(out, s.download())
    s.close()


@pytest.mark.parametrize("threads", [256, 512, 640, 768, 896, 1024])
def test_fused_block_loop_matches_graph_loop(threads):
    """The fused one-block loop (every pass of every step, rebuilds included,
    in one block per system) gives the same bits as the graph loop, for LJ
    and EAM, from the smallest box (n = 2 cell rule) up."""
    _ensure_built()
    solv = SV.solvers("mixed")
    specs = [dict(index=0, kind=k, dims=d, n=4 * d[0] * d[1] * d[2], t_arrival=0.0, steps=120,
                  dt=(W.SERVE_LJ if k == "lj" else W.SERVE_EAM)["dt"], seed=900 + j)
             for j, (k, d) in enumerate((("lj", (4, 4, 4)), ("eam", (4, 4, 4)), ("lj", (9, 8, 10)),
                                         ("eam", (12, 12, 11))))]
    reqs = SV.prepare(specs)
    out = {}
    for bt in (-1, threads):
        srv = mdg.Server(slots=4, max_atoms=8192, block_threads=bt)
        ids = [srv.submit(solv[s["kind"]], d, a, s["dt"], s["steps"]) for s, a, d in reqs]
        for k, rid in enumerate(ids):
            srv.wait(rid, 120.0)
            out[(bt, k)], info = srv.result(rid)
            assert info["status"] == 0
            assert info["rebuilds"] >= 2, (k, info)
        srv.close()
    for k in range(len(specs)):
        assert _same(out[(-1, k)], out[(threads, k)]), f"request {k}"


def test_autotuner_picks_a_measured_candidate():
    _ensure_built()
    from mdcraft_gb300 import tune
    solv = SV.solvers("mixed")
    specs = _specs(12, 50, seed=41, n_max=3000)
    best, rates = tune.tune_serving(specs, solv, candidates=(256, 1024), sample=12, steps=50, slots=16,
                                    use_cache=False)
    assert best in (256, 1024)
    assert set(rates) == {256, 1024} and all(r > 0 for r in rates.values())
    assert rates[best] == max(rates.values())


@pytest.mark.parametrize("block_threads", [0, -1], ids=["fused_block", "graph_loop"])
def test_largest_first_order_and_service_time(block_threads):
    """Admission by most atom-steps first: requests queued together start
    largest first and each result is still the single-system driver loop's,
    bit for bit; every record carries a service time that excludes the
    request's queueing."""
    _ensure_built()
    solv = SV.solvers("mixed")
    specs = _specs(8, 40, seed=23)
    reqs = SV.prepare(specs)
    srv = mdg.Server(slots=1, max_atoms=8192, block_threads=block_threads, order="largest")
    ids = [srv.submit(solv[s["kind"]], dom, atoms, s["dt"], s["steps"]) for s, atoms, dom in reqs]
    infos = {}
    for k, rid in enumerate(ids):
        srv.wait(rid, 300.0)
        out, infos[k] = srv.result(rid)
        assert infos[k]["status"] == 0
        if k in (0, 5):
            assert _same(out, _direct(specs[k], solv)), f"request {k}"
    srv.close()
    # one slot: the admissions are sequential, so their order is visible
    order = sorted(range(len(specs)), key=lambda k: infos[k]["t_admit"])
    work = [specs[k]["n"] * specs[k]["steps"] for k in order]
    # the first admission may go to the first request before the rest are
    # queued; every later one takes the largest waiting request
    assert work[1:] == sorted(work[1:], reverse=True)
    for k in range(len(specs)):
        svc = infos[k]["service_s"]
        assert 0.0 < svc <= infos[k]["t_done"] - infos[k]["t_submit"] + 1e-3


def _balanced_order(works, first, per):
    """The admission rule of MDG_ORDER_BALANCED restated: after the first
    admissions, the largest waiting request (the earliest of equals) goes
    first when its work times `per` (the workers) is at least the waiting
    work, else the earliest waiting request."""
    queue = [k for k in range(len(works)) if k not in first]
    out = list(first)
    while queue:
        largest = max(queue, key=lambda k: works[k])
        pick = largest if works[largest] * per >= sum(works[k] for k in queue) else queue[0]
        queue.remove(pick)
        out.append(pick)
    return out


def test_balanced_order_promotes_the_largest_on_the_tail():
    """MDG_ORDER_BALANCED on two graph-loop slots (no fused kernel, so the
    workers are the slots): arrival order until the largest waiting request
    holds at least half the waiting atom-steps, then that one; results stay
    the single-system driver loop's."""
    _ensure_built()
    solv = SV.solvers("mixed")
    specs = W.serving_stream(count=10, rate=1e9, seed=20, steps=100, n_min=256, n_max=4000)
    reqs = SV.prepare(specs)
    srv = mdg.Server(slots=2, max_atoms=8192, block_threads=-1, order="balanced")
    ids = [srv.submit(solv[s["kind"]], dom, atoms, s["dt"], s["steps"]) for s, atoms, dom in reqs]
    infos = {}
    for k, rid in enumerate(ids):
        srv.wait(rid, 300.0)
        out, infos[k] = srv.result(rid)
        assert infos[k]["status"] == 0
        if k in (1, 7):
            assert _same(out, _direct(specs[k], solv)), f"request {k}"
    srv.close()
    order = sorted(range(len(specs)), key=lambda k: infos[k]["t_admit"])
    # every request was queued before the third admission
    assert max(i["t_submit"] for i in infos.values()) < infos[order[2]]["t_admit"]
    works = [s["n"] * s["steps"] for s in specs]
    assert order == _balanced_order(works, order[:2], 2)
    # on this stream the rule is neither arrival order nor largest-first
    assert order[2:] != sorted(order[2:])
    assert [works[k] for k in order[2:]] != sorted((works[k] for k in order[2:]), reverse=True)


def test_mixed_request_in_a_box_below_two_rns_is_refused():
    """A periodic box shorter than 2 rns: a mixed-precision request is
    refused at submission (the mixed form's minimum images are the Periodic
    boundary's only for edges of at least 2 rns); an FP64 one runs."""
    _ensure_built()
    atoms, box, _, p = W.lj_argon_fcc(ncell=3, jitter=0.01)
    dom = SV.periodic_domain(box)
    srv = mdg.Server(slots=1, max_atoms=4096)
    with pytest.raises(RuntimeError, match="2 rns"):
        srv.submit(SV.solvers("mixed")["lj"], dom, atoms, p["dt"], 10)
    s64 = SV.solvers("fp64")
    rid = srv.submit(s64["lj"], dom, atoms, p["dt"], 10)
    srv.wait(rid, 120.0)
    _, info = srv.result(rid, atoms=False)
    assert info["status"] == 0
    srv.close()
