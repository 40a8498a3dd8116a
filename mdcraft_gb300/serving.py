"""Serving client: replays a stream of timed requests against a Server.

A request is one independent system (LJ argon or EAM Cu, 256-32768 atoms)
run for its step count through the server's continuous batching. The client
submits each request when its arrival time has passed, polls for finished
ones and records the latency from arrival to result (atoms copied back to
the host) and the service time (the request's run alone, without
queueing). Atoms are made before the clock starts, so the measured time is
the server's alone.
"""
from __future__ import annotations

import time

import numpy as np

from . import Domain, EAM, LJsCut, Server, Single
from . import workloads as W


def solvers(precision="mixed"):
    """The serving stream's two solvers (periodic boundary), keyed by kind."""
    lj = W.SERVE_LJ
    pl = LJsCut(lj["eps"], lj["sigma"], lj["rcut"])
    t = W.serve_eam_tables()
    pe = EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
    return {"lj": Single(pl, periodic=True, precision=precision),
            "eam": Single(pe, periodic=True, precision=precision), "_pots": (pl, pe)}


def periodic_domain(box):
    d = Domain(*box)
    for k in range(3):
        d.set_periodic(k, True)
    return d


def prepare(specs):
    """(spec, atoms, domain) per request, made ahead of the run."""
    out = []
    for s in specs:
        atoms, box = W.serving_atoms(s)
        out.append((s, atoms, periodic_domain(box)))
    return out


def replay(server: Server, reqs, solv, keep_results=False, release_inputs=False, idle_sleep=1e-4,
           sample_every=0.05):
    """Runs the prepared requests at their arrival times. Returns a summary
    (latency percentiles, aggregate atom-steps/s) and, when asked, the result
    atoms by request index. With release_inputs the client drops its copy of
    each request's atoms once submitted (the server keeps its own). Every
    `sample_every` seconds it records the server's occupancy (host queue,
    published and allocating requests, live and busy blocks of the fused
    loop); the summary gives their means."""
    n = len(reqs)
    arrival = np.array([s["t_arrival"] for s, _, _ in reqs])
    lat = np.full(n, np.nan)
    status = np.zeros(n, dtype=np.int64)
    queue_s = np.zeros(n)
    service_s = np.zeros(n)
    results = {}
    id2i = {}
    i = 0
    done = 0
    t0 = time.perf_counter()
    t_last = 0.0
    samples = []  # (t, host queue, published, allocating, live blocks, busy blocks)
    t_sample = 0.0
    while done < n:
        now = time.perf_counter() - t0
        if sample_every and now >= t_sample:
            st = server.stats()
            samples.append((now, st["queued"], st["block_slots"], st["alloc_slots"], st["live_blocks"],
                            st["busy_blocks"]))
            t_sample = now + sample_every
        busy = False
        while i < n and arrival[i] <= now:
            s, atoms, dom = reqs[i]
            rid = server.submit(solv[s["kind"]], dom, atoms, s["dt"], s["steps"])
            id2i[rid] = i
            if release_inputs:
                reqs[i] = (s, None, dom)
            i += 1
            busy = True
        for rid in server.poll():
            t = time.perf_counter() - t0
            k = id2i.pop(rid)
            atoms_out, info = server.result(rid, atoms=keep_results)
            lat[k] = t - arrival[k]
            status[k] = info["status"]
            queue_s[k] = info["t_admit"] - info["t_submit"]
            service_s[k] = info["service_s"]
            if keep_results:
                results[k] = atoms_out
            done += 1
            t_last = t
            busy = True
        if not busy:
            wait = idle_sleep
            if i < n:
                wait = min(wait, max(0.0, arrival[i] - (time.perf_counter() - t0)))
            if wait > 0:
                time.sleep(wait)
    atom_steps = float(sum(s["n"] * s["steps"] for s, _, _ in reqs))
    span = t_last - float(arrival[0])
    # requests running over time (each from its result time minus its
    # service time): the mean over the span and over its last fifth
    done_t = arrival + lat
    okm = np.isfinite(done_t)
    grid = np.linspace(float(arrival[0]), t_last, 400)
    running = np.zeros(len(grid))
    for a, b in zip(done_t[okm] - service_s[okm], done_t[okm]):
        running += (grid >= a) & (grid < b)
    ok = status == 0
    summary = {
        "requests": n, "failed": int((~ok).sum()),
        "p50_ms": float(np.percentile(lat[ok], 50) * 1e3) if ok.any() else None,
        "p99_ms": float(np.percentile(lat[ok], 99) * 1e3) if ok.any() else None,
        "mean_ms": float(np.mean(lat[ok]) * 1e3) if ok.any() else None,
        "max_ms": float(np.max(lat[ok]) * 1e3) if ok.any() else None,
        "queue_p50_ms": float(np.percentile(queue_s, 50) * 1e3),
        # time each request ran (its block's start to its result on the GPU
        # clock; graph loops: admission to completion), without queueing
        "service_p50_ms": float(np.percentile(service_s[ok], 50) * 1e3) if ok.any() else None,
        "service_p99_ms": float(np.percentile(service_s[ok], 99) * 1e3) if ok.any() else None,
        "atom_steps_per_s": atom_steps / span if span > 0 else None,
        "span_s": span, "atom_steps": atom_steps,
        "arrival_span_s": float(arrival[-1] - arrival[0]),
        "running_mean": float(running.mean()),
        "running_mean_last_fifth": float(running[int(0.8 * len(grid)):].mean()),
    }
    if samples:
        a = np.array(samples, dtype=np.float64)
        summary["occupancy"] = {  # means over the samples
            "samples": len(a), "host_queue": float(a[:, 1].mean()), "published": float(a[:, 2].mean()),
            "allocating": float(a[:, 3].mean()), "live_blocks": float(a[:, 4].mean()),
            "busy_blocks": float(a[:, 5].mean()),
        }
    return summary, results
