"""Project autotuner: launch shapes chosen by measuring them on the workload.

Serving: the threads of the fused per-request block (512, 640, 768, 896 or
1024; the block count follows from occupancy) are timed on a sample of the
request stream itself, each candidate on the same sample through its own
server, and the one with the highest saturated throughput is kept.

A system's step kernels (`tune_shapes`): the cells per block of the list
build (2, 4 or 8 warps, a cell each) are timed on the system's own rebuilds
(median of single rebuilds), then the register budgets of the mixed force
and density passes (blocks of 256 threads per SM; for the force pass also
eight blocks of 128 threads, whose last partial wave is shorter) by the CUDA events the
step loop puts around each of its force and density launches, one
dimension at a time. Whole-step times are not used: a list rebuild (about
three steps' worth of work) lands in some windows and not others.

Results are cached per (GPU, workload signature) in `_build/tune.json`
beside the library, so a later run on the same GPU and workload reuses the
choice without measuring.
"""
from __future__ import annotations

import hashlib
import json
import os
import time

from . import Server
from . import serving as SV

_HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(_HERE, "_build", "tune.json")


def _gpu_name(device: int) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:  # no torch CUDA: the library still runs; key by index
        return f"device{device}"


def _signature(specs) -> str:
    h = hashlib.sha1()
    for s in specs:
        h.update(f"{s['kind']}:{s['n']}:{s['steps']};".encode())
    return h.hexdigest()[:16]


def _load():
    try:
        return json.load(open(CACHE))
    except (OSError, ValueError):
        return {}


def _store(table):
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def tune_serving(specs, solvers, device=0, candidates=(512, 640, 768, 896, 1024), sample=192, steps=200, slots=320,
                 use_cache=True):
    """Fastest block size for a stream like `specs` (request specs of
    workloads.serving_stream): returns (threads, {threads: atom-steps/s}).
    The sample is the first `sample` requests with `steps` steps each, all
    submitted at once. A candidate's rate is the throughput of a saturated
    GPU, the regime of a backlog: its resident blocks (the most seen alive
    while the sample runs) times the sample's atom-steps per block-second
    (atom-steps over the sum of the requests' service times). The time to
    finish the sample would instead be set by its few longest requests
    running on after the rest."""
    sub = [dict(s, steps=steps, t_arrival=0.0) for s in specs[:sample]]
    key = f"serving-saturated|{_gpu_name(device)}|{_signature(sub)}|{','.join(map(str, candidates))}"
    table = _load() if use_cache else {}
    if key in table:
        got = table[key]
        return got["best"], {int(k): v for k, v in got["rates"].items()}
    reqs = SV.prepare(sub)
    rates = {}
    for nt in candidates:
        srv = Server(device=device, slots=slots, max_atoms=max(s["n"] for s in sub), block_threads=nt)
        # one short request first: pool pages and the kernel's first launch
        s0, a0, d0 = reqs[0]
        rid = srv.submit(solvers[s0["kind"]], d0, a0, s0["dt"], 5)
        srv.wait(rid, 120.0)
        srv.result(rid, atoms=False)
        ids = {srv.submit(solvers[s["kind"]], d, a, s["dt"], s["steps"]): k for k, (s, a, d) in enumerate(reqs)}
        busy = 0.0
        blocks = 0
        left = len(ids)
        t_end = time.perf_counter() + 600.0
        while left:
            blocks = max(blocks, srv.stats()["live_blocks"])
            got = srv.poll()
            for rid in got:
                _, info = srv.result(rid, atoms=False)
                if info["status"] != 0:
                    srv.close()
                    raise RuntimeError(f"tuning request failed with status {info['status']}")
                busy += info["service_s"]
                left -= 1
            if not got:
                if time.perf_counter() > t_end:
                    srv.close()
                    raise TimeoutError("tuning sample did not finish in 600 s")
                time.sleep(1e-3)
        srv.close()
        rates[nt] = max(blocks, 1) * sum(s["n"] * s["steps"] for s in sub) / busy
    best = max(rates, key=rates.get)
    if use_cache:
        table = _load()
        table[key] = {"best": best, "rates": {str(k): v for k, v in rates.items()}, "sample": len(sub),
                      "steps": steps}
        _store(table)
    return best, rates


SHAPE_CANDIDATES = {"list_cells_per_block": (2, 4, 8), "force_blocks_per_sm": (3, 4, 8),
                    "density_blocks_per_sm": (3, 4, 5)}


def _median_call(ctx, fn, reps):
    """Median wall time of `reps` single calls (each synchronised)."""
    ts = []
    for _ in range(reps):
        ctx.synchronize()
        t0 = time.perf_counter()
        fn()
        ctx.synchronize()
        ts.append(time.perf_counter() - t0)
    ts.sort()
    return ts[len(ts) // 2]


def _stage_seconds(ctx, run, stage):
    """Mean device time of one launch of `stage` ("forces", "density") over
    the launches `run()` makes, from the events of the context's timing
    mode."""
    ctx.set_timing(True)
    try:
        run()
        ms, count = ctx.stage_time(stage)
    finally:
        ctx.set_timing(False)
    if count == 0:
        raise RuntimeError(f"no {stage} launches to time")
    return ms / count / 1e3


def tune_shapes(system, nlist, stepper, dt, signature, device=0, eam=True, steps=30, rebuilds=7, use_cache=True):
    """Launch shapes for one system (a Context's System with its VerletList
    and Verlet stepper). The system's state advances while it is measured.
    Returns ({shape: value}, {shape: {value: seconds}}) and leaves the
    chosen shapes set on the system."""
    key = f"shapes-v2|{_gpu_name(device)}|{signature}"
    table = _load() if use_cache else {}
    if key in table:
        got = table[key]
        for name, v in got["best"].items():
            system.set_shape(name, v)
        return got["best"], {k: {int(a): b for a, b in v.items()} for k, v in got["seconds"].items()}
    ctx = system.ctx
    best, seconds = {}, {}
    # the list build, on its own rebuilds
    sec = {}
    for v in SHAPE_CANDIDATES["list_cells_per_block"]:
        system.set_shape("list_cells_per_block", v)
        nlist.update(-1.0)
        sec[v] = _median_call(ctx, lambda: nlist.update(-1.0), rebuilds)
    best["list_cells_per_block"] = min(sec, key=sec.get)
    seconds["list_cells_per_block"] = sec
    system.set_shape("list_cells_per_block", best["list_cells_per_block"])
    # the force and density passes, per launch (a short run first loads the
    # candidate's kernels)
    for name, stage in (("force_blocks_per_sm", "forces"), ("density_blocks_per_sm", "density")):
        if name == "density_blocks_per_sm" and not eam:
            continue
        sec = {}
        for v in SHAPE_CANDIDATES[name]:
            system.set_shape(name, v)
            stepper.run(system, dt, 2)
            sec[v] = _stage_seconds(ctx, lambda: stepper.run(system, dt, steps), stage)
        best[name] = min(sec, key=sec.get)
        seconds[name] = sec
        system.set_shape(name, best[name])
    if use_cache:
        table = _load()
        table[key] = {"best": best, "seconds": {k: {str(a): b for a, b in v.items()} for k, v in seconds.items()}}
        _store(table)
    return best, seconds
