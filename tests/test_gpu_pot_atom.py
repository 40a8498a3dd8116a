"""Potential's per-atom overloads on the GPU (mdg_pot_atom: force, virial
and density of one atom over an explicit list, potential/base.h:44-56)
against the oracle's whole-system FP64 stages. On an open cluster every
listed pair is a raw difference, so calling density(i) for every atom gives
the charge stage's nc, then force(i) the force stage's f, then virial(i)
the virial stage's Ep, Em and V (Single's stage order, single.cxx:11-83).
The half-list rule of LJsCut (LJs-cut.cxx:57-62, 117-125) is checked on a
half list: each pair once, pushed onto both atoms."""
import ctypes as C

import numpy as np
import pytest

import mdcraft_gb300 as mdg
from mdcraft_gb300 import workloads as W
from oracle import mdref as R
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu

REL = 1e-10  # the FP64 tolerance of the parity tests


def _entry():
    fn = mdg.lib().mdg_pot_atom
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p,
                   C.c_size_t, C.c_int]
    fn.restype = C.c_int
    return fn


def _call(fn, pot, what, atoms, i, lst, half=0):
    lst = np.ascontiguousarray(lst, dtype=np.uint64)
    base = atoms.ctypes.data
    rc = fn(H.ctx().h, pot.h, what, base + i * atoms.itemsize, base, len(atoms), lst.ctypes.data, len(lst), half)
    assert rc == 0, mdg.lib().mdg_last_error()


def _open_cluster(workload):
    atoms, box, _, p = workload
    lo = np.array(box[0::2]) - 1.0
    hi = np.array(box[1::2]) + 1.0
    return atoms, (lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]), p


@pytest.mark.parametrize("case", ["eam_cu", "lj_argon"])
def test_per_atom_stages_match_whole_system_stages(case):
    wl = W.eam_cu_fcc(ncell=4) if case == "eam_cu" else W.lj_argon_fcc(ncell=4, jitter=0.01)
    atoms, box, p = _open_cluster(wl)
    o, g = H.make_pair(atoms, box, (0, 0, 0), p, precision="fp64", periodic_boundary=False)
    o["nl"].update(-1.0)
    lists = o["nl"].lists()
    o["solver"].prepare(o["atoms"])
    prepared = o["atoms"].copy()
    o["solver"].stages(o["atoms"], o["nl"])
    o["solver"].virials(o["atoms"], o["nl"])
    ref = o["atoms"]

    pot = o["_keep"][1]
    fn = _entry()
    a = mdg.new_atoms(len(atoms))
    a.view(np.uint8)[:] = prepared.view(np.uint8)
    eam = case == "eam_cu"
    if eam:
        for i in range(len(a)):
            _call(fn, pot, 2, a, i, lists[i])  # density
        np.testing.assert_allclose(a["nc"], ref["nc"], rtol=REL)
    for i in range(len(a)):
        _call(fn, pot, 0, a, i, lists[i])  # force
    err = np.linalg.norm(a["f"] - ref["f"]) / np.linalg.norm(ref["f"])
    assert err <= REL, err
    for i in range(len(a)):
        _call(fn, pot, 1, a, i, lists[i])  # virial
    np.testing.assert_allclose(a["Ep"], ref["Ep"], rtol=REL, atol=1e-14 * np.abs(ref["Ep"]).max())
    if eam:
        np.testing.assert_allclose(a["Em"], ref["Em"], rtol=REL)
    np.testing.assert_allclose(a["V"], ref["V"], rtol=1e-9, atol=1e-12 * np.abs(ref["V"]).max())


def test_ljscut_half_list_pushes_onto_neighbours():
    atoms, box, _, p = W.lj_argon_fcc(ncell=3, jitter=0.02)
    n = len(atoms)
    pot = mdg.LJsCut(p["a"], p["s"], p["rcut"])
    fn = _entry()
    # the half list of every pair once (j > i), from a brute-force search
    r = np.asarray(atoms["r"])
    d2 = ((r[:, None, :] - r[None, :, :]) ** 2).sum(-1)
    half = [np.nonzero((d2[i] <= p["rcut"] ** 2) & (np.arange(n) > i))[0] for i in range(n)]
    full = [np.nonzero((d2[i] <= p["rcut"] ** 2) & (np.arange(n) != i))[0] for i in range(n)]
    a_half = mdg.new_atoms(n)
    a_half.view(np.uint8)[:] = np.ascontiguousarray(atoms).view(np.uint8)
    for f in ("f", "V", "Ep"):
        a_half[f] = 0
    a_full = a_half.copy()
    for i in range(n):
        _call(fn, pot, 0, a_half, i, half[i], half=1)
        _call(fn, pot, 1, a_half, i, half[i], half=1)
        _call(fn, pot, 0, a_full, i, full[i])
        _call(fn, pot, 1, a_full, i, full[i])
    scale = np.abs(a_full["f"]).max()
    assert np.abs(a_half["f"] - a_full["f"]).max() <= 1e-12 * scale
    assert np.abs(a_half["Ep"].sum() - a_full["Ep"].sum()) <= 1e-12 * np.abs(a_full["Ep"]).sum()
    assert np.abs(a_half["V"].sum(0) - a_full["V"].sum(0)).max() <= 1e-11 * np.abs(a_full["V"]).sum()
