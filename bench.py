#!/usr/bin/env python
"""Benchmark of the MD hot path: velocity-Verlet steps of EAM Cu, fcc 63^3 =
1,000,188 atoms (periodic, rc 5.0 A, skin 0.5 A, 300 K, dt 1 fs), in the
mixed-precision form, on one GB300 per rank.

One "step" = one MD step (drift + rebuild test, EAM density, EAM force with
the second half-kick, and the neighbour-list rebuild whenever the half-skin
test fires), the loop
of the reference's drivers. Prints one JSON line (rank 0).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU oracle (the restated reference path) on this
machine's host cores on the same workload. N>1 runs N independent replicas
(one per GPU, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# the serving loop runs one stream per slot: give each its own hardware
# queue (read when the CUDA context is created)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

WORKLOAD = ("EAM Cu fcc 63^3 = 1,000,188 atoms, periodic cube 22.77 nm, Finnis-Sinclair-type analytic tables "
            "(5000-point splines), rc 5.0 A, skin 0.5 A, 1% jitter, 300 K, dt 1 fs")
METRIC = "atom-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="mdg", choices=["mdg", "reference"])
    ap.add_argument("--ncell", type=int, default=63)
    ap.add_argument("--e2e-steps", type=int, default=60)  # spans about two list rebuilds
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--cpu-steps", type=int, default=6)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=4096)
    ap.add_argument("--serve-slots", type=int, default=320)
    ap.add_argument("--serve-steps", type=int, default=1000)
    ap.add_argument("--serve-block-threads", type=int, default=0,
                    help="threads of the fused per-system block (256, 512, 640, 768, 896, 1024; 0: chosen by the autotuner "
                         "on a sample of the stream; -1: a graph loop per request)")
    ap.add_argument("--serve-order", default="balanced", choices=["fifo", "largest", "balanced"],
                    help="admission order of waiting requests in the serving stream")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-only", action="store_true", help="only the serving stream (prints its summary)")
    ap.add_argument("--config", default="", choices=["", "lj_argon", "nial", "lj_liquid", "nve_drift"],
                    help="one of the other benchmark configurations (prints its own JSON line)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def Dist(world, local):
    from mdcraft_gb300.replicas import Replicas
    return Replicas(world, local, "nccl")


class Clocks:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.device = device
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and "Active" in r[5 + k] and "Not" not in r[5 + k]:
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(ncell):
    from mdcraft_gb300 import workloads as W
    return W.eam_cu_fcc(ncell=ncell)


def cpu_baseline(ncell, steps, threads=None, warmup=1):
    """The CPU oracle (C restatement of the reference path, all host threads)
    on the same workload: one list build, `warmup` untimed driver steps,
    then `steps` timed driver steps."""
    from oracle import mdref as R
    atoms, box, _, p = make_workload(ncell)
    threads = threads or R.hardware_threads()
    ao = np.zeros(len(atoms), dtype=R.ATOM_DTYPE)
    ao.view(np.uint8)[:] = atoms.view(np.uint8)
    d = R.Domain(*box)
    for k in range(3):
        d.set_periodic(k, True)
    t = p["tables"]
    pot = R.EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
    sol = R.Solver(pot, periodic=d, threads=threads)
    nl = R.VerletList(ao, d, threads=threads)
    nl.update(-1.0)
    sol.prepare(ao)
    sol.stages(ao, nl)
    if warmup > 0:
        sol.run(ao, nl, d, p["dt"], warmup)
    t0 = time.perf_counter()
    rebuilds = sol.run(ao, nl, d, p["dt"], steps)
    dt = time.perf_counter() - t0
    return {"value": len(ao) * steps / dt, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{len(ao)}-atom EAM Cu, {steps} timed Verlet steps after one list build and "
                      f"{warmup} warm-up steps ({rebuilds} rebuilds in the timed steps), {threads} threads",
            "seconds": dt, "rebuilds": rebuilds}


def run_reference(args, rank, world):
    if rank != 0:
        return
    from oracle import mdref as R
    threads = R.hardware_threads()
    # size the timed sample from one measured step (its own run, no warm-up):
    # the whole arm stays within a few minutes
    probe = cpu_baseline(args.ncell, 1, threads, warmup=0)
    per_step = probe["seconds"]
    warmup = max(0, min(args.warmup, int(30.0 / max(per_step, 1e-3))))
    steps = max(1, min(args.steps, int(90.0 / max(per_step, 1e-3))))
    cb = cpu_baseline(args.ncell, steps, threads, warmup=warmup)
    line = {"metric": METRIC, "value": cb["value"], "unit": METRIC, "n_gpus": args.gpus, "steps": steps,
            "warmup": warmup, "ms_per_step": 1e3 * cb["seconds"] / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "atoms": 4 * args.ncell ** 3, "threads": threads},
            "impl": "reference", "rebuilds": cb["rebuilds"],
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


# ncu summary of the dominant kernel (committed under profiles/): its DRAM
# bytes of one launch and the atoms that launch processed give the traffic
# per atom; its L1 figure names what limits the kernel
FORCE_PROFILE = os.path.join(ROOT, "profiles", "k_force_step_eam_cu_442k.md")


def profile_figures(path):
    """dram__bytes_read.sum + dram__bytes_write.sum (bytes), the atoms of the
    captured launch and l1tex__throughput (%) from an ncu summary."""
    import re
    try:
        text = open(path).read()
    except OSError:
        return None

    def metric(name):
        m = re.search(r"`" + re.escape(name) + r"`\s*\|\s*([0-9.]+)\s*(MB|GB|KB|%|us)?", text)
        if not m:
            return None
        v = float(m.group(1))
        return v * {"GB": 1e9, "MB": 1e6, "KB": 1e3}.get(m.group(2) or "", 1.0)

    atoms = re.search(r"Case:\s*([0-9,]+) atoms", text)
    rd, wr = metric("dram__bytes_read.sum"), metric("dram__bytes_write.sum")
    if atoms is None or rd is None or wr is None:
        return None
    return {"bytes": rd + wr, "atoms": int(atoms.group(1).replace(",", "")),
            "l1tex_pct": metric("l1tex__throughput.avg.pct_of_peak_sustained_active"),
            "dram_pct": metric("gpu__dram_throughput.avg.pct_of_peak_sustained_elapsed"),
            "file": os.path.relpath(path, ROOT)}


def energies(sol, sysg):
    """Ep + Em and Etot after prepare, stages and virials (the reference's
    recompute_state, test/cxx/support/md_test_utils.h:241-253)."""
    sol.prepare(sysg)
    sol.stages(sysg)
    sol.virials(sysg)
    m = sysg.measure()
    return m["Ep"] + m["Em"], m["Etot"]


SERVE_WORKLOAD = ("serving stream: Poisson arrivals at 2000/s, 60% LJ argon (rc 2.5 sigma, skin 0.3 A, dt 2 fs) / "
                  "40% EAM Cu (rc 5 A, skin 0.5 A, dt 1 fs), fcc boxes of 256-32768 atoms (log-uniform), "
                  "1% jitter, 300 K, mixed precision, periodic")


def run_serving(args, device):
    """The serving stream through mdg_server: latency from arrival to the
    result on the host, and aggregate atom-steps/s over the whole stream."""
    import mdcraft_gb300 as mdg
    from mdcraft_gb300 import serving as SV
    from mdcraft_gb300 import workloads as W
    specs = W.serving_stream(count=args.serve_requests, steps=args.serve_steps)
    solv = SV.solvers("mixed")
    threads, tuning = args.serve_block_threads, None
    if threads == 0:
        from mdcraft_gb300 import tune
        threads, tuning = tune.tune_serving(specs, solv, device=device, slots=args.serve_slots)
    reqs = SV.prepare(specs)
    srv = mdg.Server(device=device, slots=args.serve_slots, max_atoms=32768, block_threads=threads,
                     order=args.serve_order)
    # warm-up: one request of each kind (pool pages, potential tables)
    for kind in ("lj", "eam"):
        s = next(x for x in specs if x["kind"] == kind)
        atoms, box = W.serving_atoms(s)
        rid = srv.submit(solv[kind], SV.periodic_domain(box), atoms, s["dt"], 10)
        srv.wait(rid, 120.0)
        srv.result(rid, atoms=False)
    st0 = srv.stats()
    clocks = Clocks(device)
    clocks.start()
    summary, _ = SV.replay(srv, reqs, solv, release_inputs=True)
    ck = clocks.stop()
    st = srv.stats()
    srv.close()
    summary.update({"workload": SERVE_WORKLOAD, "slots": args.serve_slots, "steps_per_request": args.serve_steps,
                    "order": args.serve_order,
                    "block_threads": threads,
                    "tuning": ({str(k): v for k, v in tuning.items()} if tuning else "given"),
                    "arrival_rate_per_s": 2000.0, "budget_bytes": st["budget"], "peak_bytes": st["peak"],
                    # the persistent kernel launched for the warm-up may still be the one that
                    # serves the stream: count every launch of the server
                    "gpu_launches": st["launches"], "gpu_launches_in_stream": st["launches"] - st0["launches"],
                    "clocks": ck,
                    "host_s": {"admit": st["host_admit_s"], "graph": st["host_graph_s"],
                               "retire": st["host_retire_s"],
                               "retire_detail": dict(zip(("bookkeeping", "gather", "graph_release", "memory_release"),
                                                         st["host_detail_s"]))},
                    "latency": "arrival to result atoms on the host"})
    return summary


def run_mdg(args, rank, world, local):
    import torch

    import mdcraft_gb300 as mdg
    from mdcraft_gb300 import build as B

    B.build()
    dist = Dist(world, local)
    if args.config:
        if rank == 0:
            import bench_configs as BM
            clocks = Clocks(local)
            clocks.start()
            res = BM.CONFIGS[args.config](device=local)
            res["clocks"] = clocks.stop()
            print(json.dumps({"bench_config": args.config, **res}), flush=True)
        dist.close()
        return
    if args.serve_only:
        if rank == 0:
            print(json.dumps({"serving": run_serving(args, local)}), flush=True)
        dist.close()
        return
    atoms, box, _, p = make_workload(args.ncell)
    t = p["tables"]
    n = len(atoms)
    ctx = mdg.Context(local)
    dom = mdg.Domain(*box)
    for k in range(3):
        dom.set_periodic(k, True)
    sysg = mdg.System(ctx, dom, atoms)
    nl = mdg.VerletList(sysg)
    nl.update(-1.0)
    pot = mdg.EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])

    # accuracy gate on the initial configuration: mixed vs FP64 forces
    s64 = mdg.Single(pot, periodic=True, precision="fp64")
    s64.prepare(sysg)
    s64.stages(sysg)
    f64 = sysg.forces()
    smx = mdg.Single(pot, periodic=True, precision="mixed")
    smx.prepare(sysg)
    smx.stages(sysg)
    fmx = sysg.forces()
    dF = np.linalg.norm(fmx - f64, axis=1)
    rms = np.sqrt(np.mean(np.sum(f64 ** 2, axis=1)))
    err_l2 = float(np.linalg.norm(fmx - f64) / np.linalg.norm(f64))
    err_max = float(dF.max() / rms)
    L = float((nl.total() - n) / n)  # listed neighbours per atom, self excluded

    # energies of both forms at the start (both evaluate energies in FP64)
    pot64_0, _ = energies(s64, sysg)
    potmx_0, _ = energies(smx, sysg)

    # FP64 form throughput (same loop, FP64 stages)
    s64.prepare(sysg)
    s64.stages(sysg)
    st64 = mdg.Verlet(s64)
    st64.run(sysg, p["dt"], 1)
    ctx.synchronize()
    t0 = time.perf_counter()
    st64.run(sysg, p["dt"], args.fp64_steps)
    ctx.synchronize()
    fp64_rate = n * args.fp64_steps / (time.perf_counter() - t0)
    pot64_1, tot64_1 = energies(s64, sysg)
    # the mixed form over the same 1 + fp64_steps steps from the same start:
    # energy error of its trajectory against the FP64 form's
    sysg.upload(atoms)
    nl.update(-1.0)
    smx.prepare(sysg)
    smx.stages(sysg)
    mdg.Verlet(smx).run(sysg, p["dt"], 1 + args.fp64_steps)
    potmx_1, totmx_1 = energies(smx, sysg)
    energy_error = {"at_start_potential_rel": abs(potmx_0 - pot64_0) / abs(pot64_0),
                    "after_steps": 1 + args.fp64_steps,
                    "potential_rel": abs(potmx_1 - pot64_1) / abs(pot64_1),
                    "total_rel": abs(totmx_1 - tot64_1) / abs(tot64_1),
                    "note": "mixed vs FP64 form from the same start; energies are evaluated in FP64 in both forms"}

    # launch shapes of the mixed step kernels, measured on this system
    # (project autotuner; cached per GPU and workload)
    from mdcraft_gb300 import tune
    smx.prepare(sysg)
    smx.stages(sysg)
    shapes, shape_sec = tune.tune_shapes(sysg, nl, mdg.Verlet(smx), p["dt"], signature=f"eam_cu_{n}",
                                         device=local, eam=True)

    # mixed form: warm-up, then K timed steps bracketed by events on the
    # engine's stream
    sysg.upload(atoms)
    nl.update(-1.0)
    smx.prepare(sysg)
    smx.stages(sysg)
    stepper = mdg.Verlet(smx)
    stepper.run(sysg, p["dt"], args.warmup)
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=torch.device("cuda", local))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    ctx.synchronize()
    rb0 = nl.rebuilds()
    l0 = ctx.launches()
    clocks = Clocks(local)
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0.record(stream)
    stepper.run(sysg, p["dt"], args.steps)  # one captured graph: steps + device-side rebuilds
    e1.record(stream)
    ctx.synchronize()
    torch.cuda.synchronize()
    ck = clocks.stop()
    dist.barrier()
    ms = e0.elapsed_time(e1)
    launches = ctx.launches() - l0
    rebuilds = nl.rebuilds() - rb0

    # per-kernel durations: the same loop step by step with CUDA events around
    # each stage on the engine's stream (events cannot sit inside the graph)
    ctx.set_timing(True)
    stepper.run(sysg, p["dt"], min(args.steps, 40))
    fms, fn = ctx.stage_time("forces")
    dms, dn = ctx.stage_time("density")
    drms, drn = ctx.stage_time("drift")
    rms_, rn = ctx.stage_time("rebuild")
    ctx.set_timing(False)
    ms_max = dist.max(ms)
    total_atom_steps = dist.sum(float(n) * args.steps)
    value = total_atom_steps / (ms_max / 1e3)

    # end to end through the public API with pinned host buffers: each step
    # uploads positions + velocities and downloads positions, velocities, forces
    pos = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    vel = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    frc = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    pos[:] = sysg.positions()
    vel[:] = sysg.velocities()
    stepper.run_host(sysg, p["dt"], 1, pos, vel, frc)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        stepper.run_host(sysg, p["dt"], 1, pos, vel, frc)
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e = dist.sum(float(n) * args.e2e_steps) / e2e_s

    # roofline of the dominant kernel (k_force_step: the EAM force pass, mixed,
    # with the step's second half-kick and, on every step that needs no
    # rebuild and is not the last, the next step's first half-kick and drift):
    # compulsory bytes per atom = own offsets+F' (16) + list count (4) + list
    # entries (4 L) + FP32 force (12) + kick: mass (8), velocity read and
    # write (48); + on the steps it starts the next one: position read and
    # write (48), cell centre (24), rebuild-time offsets (16) and threshold
    # (8), new offsets (16) = 112. Its launches in the timed stepwise run:
    # fn, of which all but the rebuild steps and the last started the next.
    started = max(fn - rn - 1, 0) / max(fn, 1)
    bytes_atom = 32.0 + 4.0 * L + 56.0 + 112.0 * started
    force_launch_ms = fms / max(fn, 1)
    achieved = bytes_atom * n / (force_launch_ms / 1e3) / 1e9
    pk = peaks()
    peak = pk.get("hbm_gbs", 6800.0)
    prof = profile_figures(FORCE_PROFILE)
    roof = {"bound": "hbm",
            "kernel": "k_force_step (EAM force, mixed, with the second half-kick and the next step's start)",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": (prof["bytes"] / prof["atoms"] * n) if prof else None,
            "peak_source": "measured" if "hbm_gbs" in pk else "fallback",
            "bytes_per_atom": bytes_atom, "launch_ms": force_launch_ms,
            "launches_starting_next_step": started}
    if prof:
        roof["traffic_source"] = (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on "
                                  f"{prof['atoms']:,} atoms ({prof['file']}), scaled to {n:,} atoms")
        roof["limiter"] = {"l1tex_throughput_pct": prof["l1tex_pct"], "dram_throughput_pct": prof["dram_pct"],
                           "source": prof["file"]}

    serving = None
    if not args.no_serve:
        serving = run_serving(args, local)

    if rank == 0:
        cb = None
        if not args.no_cpu and world == 1:
            cb = cpu_baseline(args.ncell, args.cpu_steps)
            cb = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "mixed: f32 pair math, f64 state",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "atoms": n, "precision": "mixed",
                       "l2": f"inputs larger than L2 (~{n * 500 / 1e6:.0f} MB resident per replica)",
                       "parallelism": f"replicas x{world}", "neighbours_per_atom": L},
            "fp64_form": {"value": fp64_rate, "unit": METRIC, "mixed_speedup": value / world / fp64_rate},
            "force_error": {"l2_rel": err_l2, "max_over_rms": err_max, "bar": 1e-5},
            "energy_error": energy_error,
            "rebuilds": rebuilds,
            "stage_ms_per_launch": {"drift": drms / max(drn, 1), "density": dms / max(dn, 1),
                                    "forces_and_kick": force_launch_ms, "rebuild": rms_ / max(rn, 1)},
            "e2e": {"value": e2e, "unit": METRIC, "h2d_bytes_per_step": n * 48, "d2h_bytes_per_step": n * 72},
            "gpu_launches": launches,
            "shape_tuning": {"chosen": shapes, "seconds": shape_sec},
            "roofline": roof,
            "cpu_baseline": cb,
            "clocks": ck,
            "serving": serving,
        }
        print(json.dumps(line), flush=True)
    dist.close()


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_mdg(args, rank, world, local)


if __name__ == "__main__":
    main()
