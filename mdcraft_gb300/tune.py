"""Project autotuner: launch shapes chosen by measuring them on the workload.

Serving: the threads of the fused per-request block (256, 512 or 1024; the
block count follows from occupancy) are timed on a sample of the request
stream itself, each candidate on the same sample through its own server, and
the fastest is kept. Results are cached per (GPU, workload signature) in
`_build/tune.json` beside the library, so a later run on the same GPU and
workload reuses the choice without measuring.

The per-stage kernels' shapes (threads per block, register budgets, lanes
per cell of the list build) were chosen by the same kind of measurement and
are fixed in the sources; the list build picks its lanes per cell from the
cell occupancy of each grid at run time.
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


def tune_serving(specs, solvers, device=0, candidates=(256, 512, 1024), sample=192, steps=200, slots=320,
                 use_cache=True):
    """Fastest block size for a stream like `specs` (request specs of
    workloads.serving_stream): returns (threads, {threads: atom-steps/s}).
    The sample is the first `sample` requests with `steps` steps each, all
    submitted at once (the throughput regime of a backlog)."""
    sub = [dict(s, steps=steps, t_arrival=0.0) for s in specs[:sample]]
    key = f"serving|{_gpu_name(device)}|{_signature(sub)}|{','.join(map(str, candidates))}"
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
        t0 = time.perf_counter()
        ids = [srv.submit(solvers[s["kind"]], d, a, s["dt"], s["steps"]) for s, a, d in reqs]
        for rid in ids:
            srv.wait(rid, 600.0)
        sec = time.perf_counter() - t0
        for rid in ids:
            srv.result(rid, atoms=False)
        srv.close()
        rates[nt] = sum(s["n"] * s["steps"] for s in sub) / sec
    best = max(rates, key=rates.get)
    if use_cache:
        table = _load()
        table[key] = {"best": best, "rates": {str(k): v for k, v in rates.items()}, "sample": len(sub),
                      "steps": steps}
        _store(table)
    return best, rates
