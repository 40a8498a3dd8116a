"""Shared set-up of the GPU parity tests: the same seeded inputs drive the
device engine (through the C-ABI via mdcraft_gb300) and the CPU oracle."""
from __future__ import annotations

import numpy as np

import mdcraft_gb300 as mdg
from oracle import mdref as R

_CTX = None


def ctx():
    global _CTX
    if _CTX is None:
        from mdcraft_gb300 import build
        build.build()
        _CTX = mdg.Context(0)
    return _CTX


def to_oracle_atoms(atoms):
    a = np.zeros(len(atoms), dtype=R.ATOM_DTYPE)
    a.view(np.uint8)[:] = np.ascontiguousarray(atoms).view(np.uint8)
    return a


def domains(box, periodic):
    do = R.Domain(*box)
    dg = mdg.Domain(*box)
    for k in range(3):
        if periodic[k]:
            do.set_periodic(k, True)
            dg.set_periodic(k, True)
    return do, dg


def potentials(params):
    """(oracle solver factory, device solver factory) for a workload's params."""
    kind = params["kind"]
    if kind == "lj":
        return ("lj", (params["a"], params["s"], params["rcut"]))
    if kind == "eam":
        return ("eam", params["tables"])
    return ("multi", params["tables"])


def make_pair(atoms, box, periodic, params, precision="fp64", periodic_boundary=True, threads=None):
    """Returns (oracle dict, device dict) with atoms, domains, lists, solvers."""
    threads = threads or R.hardware_threads()
    do, dg = domains(box, periodic)
    ao = to_oracle_atoms(atoms)
    kind, spec = potentials(params)
    pd_o = do if periodic_boundary else None
    if kind == "lj":
        po = R.LJsCut(*spec)
        so = R.Solver(po, periodic=pd_o, threads=threads)
        pg = mdg.LJsCut(*spec)
        sg = mdg.Single(pg, periodic=periodic_boundary, precision=precision)
        pots = (po, pg)
    elif kind == "eam":
        t = spec
        po = R.EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
        so = R.Solver(po, periodic=pd_o, threads=threads)
        pg = mdg.EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
        sg = mdg.Single(pg, periodic=periodic_boundary, precision=precision)
        pots = (po, pg)
    else:
        nk = params.get("nkinds", 2)
        so = R.Solver(None, periodic=pd_o, threads=threads, nkinds=nk)
        sg = mdg.Multi(nk, periodic=periodic_boundary, precision=precision)
        pots = []
        for (i, j), t in spec.items():
            po = R.EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
            pg = mdg.EAM(t["rcut"], t["Femb"], t["Rho"], t["Vpar"], t["Nr1"], t["dr"], t["Nrh1"], t["drh"])
            so.add_potential(i, j, po)
            sg.add_potential(i, j, pg)
            pots.append((po, pg))
    nlo = R.VerletList(ao, do, threads=threads)
    sysg = mdg.System(ctx(), dg, atoms)
    nlg = mdg.VerletList(sysg)
    o = dict(atoms=ao, dom=do, nl=nlo, solver=so)
    g = dict(sys=sysg, dom=dg, nl=nlg, solver=sg, stepper=mdg.Verlet(sg))
    o["_keep"] = pots
    return o, g


def force_error(f_test, f_ref):
    """(max_i |dF_i| / RMS|F|, ||dF||_2 / ||F||_2)."""
    d = np.linalg.norm(f_test - f_ref, axis=1)
    rms = np.sqrt(np.mean(np.sum(f_ref ** 2, axis=1)))
    return float(d.max() / rms), float(np.linalg.norm(f_test - f_ref) / np.linalg.norm(f_ref))


def same_sets(lists_a, lists_b):
    bad = 0
    for a, b in zip(lists_a, lists_b):
        if not np.array_equal(np.sort(np.asarray(a, dtype=np.uint64)), np.sort(np.asarray(b, dtype=np.uint64))):
            bad += 1
    return bad
