"""Measurements of the benchmark configurations other than the headline one
(bench.py --config NAME). A measurement harness beside bench.py, not part of
the library: its CPU leg and checks call the oracle.

Each function runs one configuration on the GPU through the public API and
returns a dict (one JSON line of bench.py --config NAME):

- lj_argon   : LJ argon fcc 10^3 (4000 atoms), FP64 and mixed, 1000 steps,
               the FP64 trajectory checked against the CPU oracle's.
- nial       : two-species EAM NiAl B2 80^3 (~1.02M atoms), Multi solver,
               mixed precision, 500 steps; force error against FP64.
- lj_liquid  : LJ liquid 16,777,216 atoms, mixed, 200 steps (rebuilds
               re-sort the atoms every time, as every rebuild here does).
- nve_drift  : LJ liquid subset of 262,144 atoms, 10^4 NVE steps in the
               FP64 and the mixed form; relative total-energy drift.

The CPU numbers come from the oracle (C restatement of the reference's
path, all host threads) on the same inputs, on a bounded number of steps
stated in the result.
"""
from __future__ import annotations

import time

import numpy as np

from mdcraft_gb300 import EAM, Context, Domain, LJsCut, Multi, Single, System, Verlet, VerletList
from mdcraft_gb300 import tune
from mdcraft_gb300 import workloads as W


def _domain(box):
    d = Domain(*box)
    for k in range(3):
        d.set_periodic(k, True)
    return d


def _solver(params, precision):
    kind = params["kind"]
    if kind == "lj":
        pot = LJsCut(params["a"], params["s"], params["rcut"])
        return Single(pot, periodic=True, precision=precision), [pot]
    if kind == "eam":
        t = params["tables"]
        pot = EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
        return Single(pot, periodic=True, precision=precision), [pot]
    sol = Multi(params.get("nkinds", 2), periodic=True, precision=precision)
    pots = []
    for (i, j), t in params["tables"].items():
        pot = EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
        sol.add_potential(i, j, pot)
        pots.append(pot)
    return sol, pots


def _force_error(f_test, f_ref):
    d = np.linalg.norm(f_test - f_ref, axis=1)
    rms = np.sqrt(np.mean(np.sum(f_ref ** 2, axis=1)))
    return {"l2_rel": float(np.linalg.norm(f_test - f_ref) / np.linalg.norm(f_ref)), "max_over_rms": float(d.max() / rms)}


def _timed_run(ctx, sysg, stepper, dt, steps):
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=torch.device("cuda", ctx.device))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    ctx.synchronize()
    e0.record(stream)
    stepper.run(sysg, dt, steps)
    e1.record(stream)
    ctx.synchronize()
    return e0.elapsed_time(e1) / 1e3


def _energy(sol, sysg):
    sol.prepare(sysg)
    sol.virials(sysg)
    return sysg.measure()


def _state_energy(sol, sysg):
    """(Ep + Em, Etot) after prepare, stages and virials (recompute_state,
    test/cxx/support/md_test_utils.h:241-253)."""
    sol.prepare(sysg)
    sol.stages(sysg)
    sol.virials(sysg)
    m = sysg.measure()
    return m["Ep"] + m["Em"], m["Etot"]


def _energy_error(sysg, nl, atoms, s64, smx, dt, steps):
    """Energy error of the mixed form against the FP64 form: both run `steps`
    steps from the same start; energies are evaluated in FP64 in both forms,
    so the difference is that of the trajectories."""
    out = {}
    for prec, sol in (("fp64", s64), ("mixed", smx)):
        sysg.upload(atoms)
        nl.update(-1.0)
        e0 = _state_energy(sol, sysg)
        Verlet(sol).run(sysg, dt, steps)
        out[prec] = (e0, _state_energy(sol, sysg))
    (p0, _), (p1, t1) = out["fp64"]
    (q0, _), (q1, u1) = out["mixed"]
    return {"at_start_potential_rel": abs(q0 - p0) / abs(p0), "after_steps": steps,
            "potential_rel": abs(q1 - p1) / abs(p1), "total_rel": abs(u1 - t1) / abs(t1)}


def _oracle_rate(atoms, box, params, steps, threads=None):
    """The oracle's driver loop on the same input: (atom-steps/s, seconds, rebuilds, final atoms)."""
    from oracle import mdref as R
    threads = threads or R.hardware_threads()
    ao = np.zeros(len(atoms), dtype=R.ATOM_DTYPE)
    ao.view(np.uint8)[:] = np.ascontiguousarray(atoms).view(np.uint8)
    d = R.Domain(*box)
    for k in range(3):
        d.set_periodic(k, True)
    kind = params["kind"]
    keep = []
    if kind == "lj":
        pot = R.LJsCut(params["a"], params["s"], params["rcut"])
        sol = R.Solver(pot, periodic=d, threads=threads)
        keep.append(pot)
    elif kind == "eam":
        t = params["tables"]
        pot = R.EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
        sol = R.Solver(pot, periodic=d, threads=threads)
        keep.append(pot)
    else:
        sol = R.Solver(None, periodic=d, threads=threads, nkinds=params.get("nkinds", 2))
        for (i, j), t in params["tables"].items():
            pot = R.EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
            sol.add_potential(i, j, pot)
            keep.append(pot)
    nl = R.VerletList(ao, d, threads=threads)
    nl.update(-1.0)
    sol.prepare(ao)
    sol.stages(ao, nl)
    t0 = time.perf_counter()
    rebuilds = sol.run(ao, nl, d, params["dt"], steps)
    dt = time.perf_counter() - t0
    del keep
    return len(ao) * steps / dt, dt, rebuilds, ao, threads


def lj_argon(device=0, steps=1000, cpu=True):
    atoms, box, _, p = W.lj_argon_fcc()
    ctx = Context(device)
    out = {"config": "LJ argon fcc 10^3 = 4000 atoms, a 5.26 A, rc 2.5 sigma, skin 0.3 A, 100 K, dt 2 fs",
           "steps": steps}
    final = {}
    for prec in ("fp64", "mixed"):
        sysg = System(ctx, _domain(box), atoms)
        nl = VerletList(sysg)
        nl.update(-1.0)
        sol, keep = _solver(p, prec)
        sol.prepare(sysg)
        sol.stages(sysg)
        st = Verlet(sol)
        st.run(sysg, p["dt"], 3)  # warm-up (graph instantiation)
        sysg.upload(atoms)
        nl.update(-1.0)
        sol.prepare(sysg)
        sol.stages(sysg)
        e0 = _energy(sol, sysg)["Etot"]
        sol.stages(sysg)
        rb0 = nl.rebuilds()
        sec = _timed_run(ctx, sysg, st, p["dt"], steps)
        e1 = _energy(sol, sysg)["Etot"]
        final[prec] = sysg.download()
        final[prec + "_energy"] = _state_energy(sol, sysg)
        out[prec] = {"value": len(atoms) * steps / sec, "unit": "atom-steps/s", "ms_per_step": 1e3 * sec / steps,
                     "rebuilds": nl.rebuilds() - rb0, "energy_drift_rel": (e1 - e0) / abs(e0)}
        sysg.close()
    (p1, t1), (q1, u1) = final["fp64_energy"], final["mixed_energy"]
    out["energy_error_vs_fp64"] = {"after_steps": steps, "potential_rel": abs(q1 - p1) / abs(p1),
                                   "total_rel": abs(u1 - t1) / abs(t1)}
    if cpu:
        rate, sec, rebuilds, ao, threads = _oracle_rate(atoms, box, p, steps)
        dr = np.abs(final["fp64"]["r"] - ao["r"]).max()
        out["cpu_baseline"] = {"value": rate, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                               "sample": f"the whole run ({steps} steps, {rebuilds} rebuilds)"}
        out["fp64_vs_oracle"] = {"max_abs_dr_nm": float(dr), "max_abs_dv": float(np.abs(final["fp64"]["v"] - ao["v"]).max()),
                                 "rebuilds_equal": bool(rebuilds == out["fp64"]["rebuilds"])}
    return out


def nial(device=0, steps=500, ncell=80, cpu_steps=4):
    atoms, box, _, p = W.eam_nial_b2(ncell=ncell)
    ctx = Context(device)
    sysg = System(ctx, _domain(box), atoms)
    nl = VerletList(sysg)
    nl.update(-1.0)
    s64, k1 = _solver(p, "fp64")
    smx, k2 = _solver(p, "mixed")
    s64.prepare(sysg)
    s64.stages(sysg)
    f64 = sysg.forces()
    smx.prepare(sysg)
    smx.stages(sysg)
    fmx = sysg.forces()
    err = _force_error(fmx, f64)
    L = float((nl.total() - len(atoms)) / len(atoms))
    st64 = Verlet(s64)
    st64.run(sysg, p["dt"], 1)
    sec64 = _timed_run(ctx, sysg, st64, p["dt"], 5)
    # launch shapes of the mixed kernels, measured on this system (state reset after)
    smx.prepare(sysg)
    smx.stages(sysg)
    shapes, _ = tune.tune_shapes(sysg, nl, Verlet(smx), p["dt"], signature=f"nial_{len(atoms)}", device=device,
                                 eam=True)
    sysg.upload(atoms)
    nl.update(-1.0)
    smx.prepare(sysg)
    smx.stages(sysg)
    st = Verlet(smx)
    st.run(sysg, p["dt"], 3)
    rb0 = nl.rebuilds()
    sec = _timed_run(ctx, sysg, st, p["dt"], steps)
    rebuilds = nl.rebuilds() - rb0
    # the same comparison on the thermalised positions after the run (the
    # start is a perfect lattice, whose forces nearly cancel)
    s64.prepare(sysg)
    s64.stages(sysg)
    f64b = sysg.forces()
    smx.prepare(sysg)
    smx.stages(sysg)
    err_run = _force_error(sysg.forces(), f64b)
    eerr = _energy_error(sysg, nl, atoms, s64, smx, p["dt"], 20)
    n = len(atoms)
    out = {"config": f"NiAl B2 {ncell}^3 cells, 0.5% vacancies ({n} atoms), Multi with 3 EAM pair tables, "
                     "rc 6 A, skin 0.5 A, 600 K, dt 1 fs, mixed",
           "atoms": n, "steps": steps, "neighbours_per_atom": L,
           "mixed": {"value": n * steps / sec, "unit": "atom-steps/s", "ms_per_step": 1e3 * sec / steps,
                     "rebuilds": rebuilds},
           "fp64_form": {"value": n * 5 / sec64, "unit": "atom-steps/s", "steps": 5},
           "force_error_vs_fp64": err, "force_error_vs_fp64_after_run": err_run, "energy_error_vs_fp64": eerr,
           "shapes": shapes}
    out["mixed_speedup"] = out["mixed"]["value"] / out["fp64_form"]["value"]
    if cpu_steps:
        rate, secc, rebuilds, _, threads = _oracle_rate(atoms, box, p, cpu_steps)
        out["cpu_baseline"] = {"value": rate, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                               "sample": f"{cpu_steps} steps after one list build ({rebuilds} rebuilds)"}
    sysg.close()
    return out


def lj_liquid(device=0, steps=200, dims=(128, 128, 256), cpu_steps=1):
    atoms, box, _, p = W.lj_liquid(*dims)
    ctx = Context(device)
    sysg = System(ctx, _domain(box), atoms)
    nl = VerletList(sysg)
    nl.update(-1.0)
    s64, k1 = _solver(p, "fp64")
    smx, k2 = _solver(p, "mixed")
    s64.prepare(sysg)
    s64.stages(sysg)
    f64 = sysg.forces()
    smx.prepare(sysg)
    smx.stages(sysg)
    fmx = sysg.forces()
    err = _force_error(fmx, f64)
    del f64, fmx
    # launch shapes of the mixed kernels, measured on this system (state reset after)
    shapes, _ = tune.tune_shapes(sysg, nl, Verlet(smx), p["dt"], signature=f"lj_liquid_{len(atoms)}",
                                 device=device, eam=False)
    sysg.upload(atoms)
    nl.update(-1.0)
    smx.prepare(sysg)
    smx.stages(sysg)
    st = Verlet(smx)
    st.run(sysg, p["dt"], 3)
    rb0 = nl.rebuilds()
    sec = _timed_run(ctx, sysg, st, p["dt"], steps)
    rebuilds = nl.rebuilds() - rb0
    # per-stage device times: the same loop step by step with CUDA events
    # around each stage launch (40 steps)
    ctx.set_timing(True)
    st.run(sysg, p["dt"], 40)
    ctx.synchronize()
    stage = {}
    for k in ("drift", "forces", "rebuild"):
        ms, nlaunch = ctx.stage_time(k)
        stage[k] = {"ms_per_launch": ms / max(nlaunch, 1), "launches": nlaunch}
    ctx.set_timing(False)
    eerr = _energy_error(sysg, nl, atoms, s64, smx, p["dt"], 10)
    n = len(atoms)
    out = {"config": f"LJ liquid rho*=0.8442 T*=0.72, fcc melt start, {n} atoms, rc 2.5 sigma, skin 0.3 sigma, "
                     f"dt*=0.005, mixed", "atoms": n, "steps": steps,
           "mixed": {"value": n * steps / sec, "unit": "atom-steps/s", "ms_per_step": 1e3 * sec / steps,
                     "rebuilds": rebuilds, "stage_ms": stage},
           "force_error_vs_fp64": err, "energy_error_vs_fp64": eerr, "shapes": shapes}
    sysg.close()
    if cpu_steps:
        rate, secc, rebuilds, _, threads = _oracle_rate(atoms, box, p, cpu_steps)
        out["cpu_baseline"] = {"value": rate, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                               "sample": f"{cpu_steps} steps after one list build ({rebuilds} rebuilds)"}
    return out


def nve_drift(device=0, steps=10000, dims=(32, 32, 64), every=1000):
    atoms, box, _, p = W.lj_liquid(*dims)
    ctx = Context(device)
    out = {"config": f"LJ liquid subset {len(atoms)} atoms (4*{dims[0]}*{dims[1]}*{dims[2]}), NVE, "
                     f"{steps} steps of dt*=0.005", "atoms": len(atoms), "steps": steps, "every": every}
    for prec in ("fp64", "mixed"):
        sysg = System(ctx, _domain(box), atoms)
        nl = VerletList(sysg)
        nl.update(-1.0)
        sol, keep = _solver(p, prec)
        sol.prepare(sysg)
        sol.stages(sysg)
        st = Verlet(sol)
        e = [_energy(sol, sysg)["Etot"]]
        sol.stages(sysg)
        t0 = time.perf_counter()
        for _ in range(steps // every):
            st.run(sysg, p["dt"], every)
            e.append(_energy(sol, sysg)["Etot"])
            sol.stages(sysg)
        sec = time.perf_counter() - t0
        e = np.array(e)
        rel = (e - e[0]) / abs(e[0])
        out[prec] = {"E0": float(e[0]), "drift_rel_final": float(rel[-1]), "drift_rel_max_abs": float(np.abs(rel).max()),
                     "series_rel": [float(x) for x in rel], "seconds": sec,
                     "rebuilds": nl.rebuilds()}
        sysg.close()
    return out


CONFIGS = {"lj_argon": lj_argon, "nial": nial, "lj_liquid": lj_liquid, "nve_drift": nve_drift}
