"""Test support: restatements of the reference's test utilities
(test/cxx/support/md_test_utils.h) and its fixture loaders, shared by the
oracle pin tests and the GPU parity tests."""
from __future__ import annotations

import lzma
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

kAngstromToNm = 0.1
kBoltzmann = 0.008314462175

# Unit constants of mdcraft/solver/potential/EAM.cxx:8-13
N_a = 6.02214076e23
Qelectron = 1.602176634e-19
UnMass = 1e-3 / N_a
UnLeng = 1e-9
UnTime = 1e-12
UnEnrg = UnMass * (UnLeng / UnTime) * (UnLeng / UnTime)


def atom_array(n: int, dtype) -> np.ndarray:
    a = np.zeros(n, dtype=dtype)
    a["tag"] = 0xFFFF
    return a


def load_lammps_atomic_data(text: str, dtype):
    """load_lammps_atomic_data (md_test_utils.h:71-169). Returns
    (atoms, (xmin, xmax, ymin, ymax, zmin, zmax)) in nm."""
    lines = text.splitlines()
    total = 0
    box = {}
    masses = {}
    i = 0
    while i < len(lines):
        line = lines[i]
        i += 1
        if not line or line[0] == "#":
            continue
        if "atoms" in line and "atom" in line:
            total = int(line.split()[0])
            continue
        for key, tag in (("xlo xhi", "x"), ("ylo yhi", "y"), ("zlo zhi", "z")):
            if key in line:
                lo, hi = line.split()[:2]
                box[tag] = (float(lo), float(hi))
        if "Masses" in line:
            while i < len(lines) and (not lines[i] or lines[i][0] == "#"):
                i += 1
            while i < len(lines) and lines[i] and lines[i][0] != "#":
                t, m = lines[i].split()[:2]
                masses[int(t)] = float(m)
                i += 1
            continue
        if "Atoms" in line:
            while i < len(lines) and (not lines[i] or lines[i][0] == "#"):
                i += 1
            break
    rows = []
    while i < len(lines) and len(rows) < total:
        line = lines[i]
        i += 1
        if not line or line[0] == "#":
            continue
        p = line.split()
        if len(p) < 5:
            continue
        rows.append((int(p[0]), int(p[1]), float(p[2]), float(p[3]), float(p[4])))
    atoms = atom_array(len(rows), dtype)
    arr = np.array(rows, dtype=np.float64)
    atoms["uid"] = arr[:, 0].astype(np.uint32)
    atoms["kind"] = arr[:, 1].astype(np.uint16)
    atoms["r"] = arr[:, 2:5] * kAngstromToNm
    atoms["m"] = np.array([masses.get(int(k), 0.0) for k in arr[:, 1]])
    b = tuple(v * kAngstromToNm for v in (*box["x"], *box["y"], *box["z"]))
    return atoms, b


def argon_ball(dtype):
    with lzma.open(os.path.join(GOLDEN, "lmp_ball_130k_ar.xz"), "rt") as f:
        return load_lammps_atomic_data(f.read(), dtype)


def read_setfl(text: str) -> dict:
    """EAM::EAM(std::string) reader (mdcraft/solver/potential/EAM.cxx:55-87):
    skips 4 lines, reads Nrh1 drh Nr1 dr rcut, Z M Ecoh lattice, then
    Femb[Nrh1], Rho[Nr1], Vpar[Nr1]; converts A->nm and eV->kJ/mol."""
    lines = text.splitlines(True)
    toks = "".join(lines[4:]).split()
    Nrh1, drh, Nr1, dr, rcut = int(toks[0]), float(toks[1]), int(toks[2]), float(toks[3]), float(toks[4])
    pos = 9  # after Z M Ecoh lattice
    vals = np.array([float(t) for t in toks[pos: pos + Nrh1 + 2 * Nr1]], dtype=np.float64)
    Femb = vals[:Nrh1] * (Qelectron / UnEnrg)
    Rho = vals[Nrh1: Nrh1 + Nr1].copy()
    Vpar = vals[Nrh1 + Nr1:] * (Qelectron / (10 * UnEnrg))
    return dict(rcut=rcut / 10, Femb=Femb, Rho=Rho, Vpar=Vpar, Nr1=Nr1, dr=dr / 10, Nrh1=Nrh1, drh=drh)


def al2009():
    with lzma.open(os.path.join(GOLDEN, "al2009_eam_alloy.xz"), "rt") as f:
        return read_setfl(f.read())


def read_pair_file(text: str) -> dict:
    """Pair::Pair(std::string) reader (mdcraft/solver/potential/pair.cxx:36-56):
    skips 4 lines, reads Nr1 dr rcut, then Nr1 values of r*phi(r) in eV*A;
    converts A->nm and eV*A->kJ*nm/mol."""
    lines = text.splitlines(True)
    toks = "".join(lines[4:]).split()
    Nr1, dr, rcut = int(toks[0]), float(toks[1]), float(toks[2])
    Vpar = np.array([float(t) for t in toks[3: 3 + Nr1]], dtype=np.float64) * (Qelectron / (10 * UnEnrg))
    return dict(rcut=rcut / 10, Vpar=Vpar, Nr1=Nr1, dr=dr / 10)


def nialpair_text() -> str:
    with lzma.open(os.path.join(GOLDEN, "nialpair_eam_alloy.xz"), "rt") as f:
        return f.read()


def nialpair():
    return read_pair_file(nialpair_text())


def al2009_text() -> str:
    with lzma.open(os.path.join(GOLDEN, "al2009_eam_alloy.xz"), "rt") as f:
        return f.read()


def set_common_atom_properties(atoms, mass, rcut, skin_factor):
    """set_common_atom_properties (md_test_utils.h:171-184)."""
    n = len(atoms)
    idx = np.arange(n)
    atoms["uid"] = np.where(atoms["uid"] == 0, idx + 1, atoms["uid"])
    atoms["kind"] = np.where(atoms["kind"] == 0, 1, atoms["kind"])
    atoms["m"] = mass
    atoms["rcut"] = rcut
    atoms["rns"] = skin_factor * rcut


def assign_deterministic_velocities(atoms, scale):
    """assign_deterministic_velocities (md_test_utils.h:186-206); sums in
    atom order like the reference."""
    n = len(atoms)
    i = np.arange(n)
    sx = (i % 7).astype(np.float64) - 3
    sy = ((i // 7) % 5).astype(np.float64) - 2
    sz = ((i // 35) % 3).astype(np.float64) - 1
    v = np.stack([scale * sx, scale * sy, scale * sz], axis=1)
    atoms["v"] = v
    mom = np.zeros(3)
    tm = 0.0
    for k in range(n):
        mom = mom + atoms["m"][k] * atoms["v"][k]
        tm += atoms["m"][k]
    com = mom / tm if tm > 0 else np.zeros(3)
    atoms["v"] = atoms["v"] - com


def make_fcc_bulk(nx, ny, nz, a, mass, dtype):
    """make_fcc_bulk (md_test_utils.h:291-344): atoms in (iz, iy, ix, basis)
    order, box centred at the origin, periodic on all axes."""
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]], dtype=np.float64)
    lx, ly, lz = nx * a, ny * a, nz * a
    ox, oy, oz = -0.5 * lx, -0.5 * ly, -0.5 * lz
    n = 4 * nx * ny * nz
    atoms = atom_array(n, dtype)
    r = np.zeros((n, 3))
    k = 0
    for iz in range(nz):
        for iy in range(ny):
            for ix in range(nx):
                co = np.array([ox + ix * a, oy + iy * a, oz + iz * a])
                for b in basis:
                    r[k] = co + a * b
                    k += 1
    atoms["r"] = r
    atoms["uid"] = np.arange(1, n + 1)
    atoms["kind"] = 1
    atoms["m"] = mass
    box = (-0.5 * lx, 0.5 * lx, -0.5 * ly, 0.5 * ly, -0.5 * lz, 0.5 * lz)
    return atoms, box
