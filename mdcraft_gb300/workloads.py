"""Seeded synthetic workloads of the benchmark configurations.

All quantities in MDcraft units (nm, ps, g/mol, kJ/mol). One generator feeds
both the device engine and the CPU oracle, so every comparison runs on
identical inputs.

- lj_argon_fcc     : LJ argon, fcc 10^3 cells (4000 atoms), a = 5.26 A,
                     sigma = 3.405 A, eps = 0.0104 eV, rc = 2.5 sigma,
                     skin 0.3 A, 100 K, dt = 2 fs.
- eam_cu_fcc       : EAM Cu, fcc n^3 cells (63^3 -> 1,000,188 atoms),
                     a = 3.615 A, analytic Finnis-Sinclair-type tables on
                     5000-point grids, rc = 5.0 A, skin 0.5 A, 1% Gaussian
                     jitter (sigma = 0.01 a per component), 300 K, dt = 1 fs.
- eam_nial_b2      : two-species EAM NiAl, B2 n^3 cells with 0.5% vacancies,
                     a = 2.88 A, per-pair analytic tables, rc = 6.0 A,
                     skin 0.5 A, 600 K, dt = 1 fs.
- lj_liquid        : reduced LJ liquid (rho* = 0.8442, T* = 0.72) mapped to
                     argon, fcc start with a bounded uniform jitter (at most
                     0.05 a per component, so no pair starts closer than
                     0.9 sigma), rc = 2.5 sigma, skin 0.3 sigma, dt* = 0.005.
"""
from __future__ import annotations

import math

import numpy as np

from . import ATOM_DTYPE

# 1 eV in kJ/mol, as MDcraft's EAM reader converts it (EAM.cxx:8-13)
_N_a = 6.02214076e23
_Q = 1.602176634e-19
_UnEnrg = (1e-3 / _N_a) * (1e-9 / 1e-12) * (1e-9 / 1e-12)
EV = _Q / _UnEnrg
KB = 0.008314462175  # kJ/mol/K (mdcraft/solver/thermostat/base.h:10)

AR_MASS = 39.948
CU_MASS = 63.546
NI_MASS = 58.6934
AL_MASS = 26.9815


def new_atoms(n: int) -> np.ndarray:
    a = np.zeros(n, dtype=ATOM_DTYPE)
    a["tag"] = 0xFFFF
    return a


def fcc_positions(nx, ny, nz, a, origin=(0.0, 0.0, 0.0)):
    """fcc sites, cell-major order (ix fastest), 4 basis atoms per cell."""
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]], dtype=np.float64)
    iz, iy, ix = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cells = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64)
    pos = (cells[:, None, :] + basis[None, :, :]).reshape(-1, 3) * a
    return pos + np.asarray(origin)


def maxwell_boltzmann(rng, masses, T):
    """Gaussian velocities at temperature T with zero net momentum."""
    n = len(masses)
    v = rng.standard_normal((n, 3)) * np.sqrt(KB * T / masses)[:, None]
    p = (masses[:, None] * v).sum(axis=0)
    v -= p / masses.sum()
    return v


def _finish(atoms, box_lo, box_hi, periodic=True):
    dom = (box_lo[0], box_hi[0], box_lo[1], box_hi[1], box_lo[2], box_hi[2])
    return atoms, dom, periodic


def _wrap_inside(r, lo, L):
    """Wraps into [lo, lo + L) so no atom sits on the upper face."""
    r = lo + np.mod(r - lo, L)
    r = np.where(r >= lo + L, r - L, r)
    return r


def lj_argon_fcc(ncell=10, seed=1, T=100.0, jitter=0.0):
    """Config 1 (LJ argon fcc 10^3 = 4000 atoms; perfect lattice unless a
    Gaussian jitter, as a fraction of a, is asked for)."""
    a = 0.526
    sigma, eps = 0.3405, 0.0104 * EV
    rc = 2.5 * sigma
    skin = 0.03
    L = ncell * a
    rng = np.random.default_rng(seed)
    r = fcc_positions(ncell, ncell, ncell, a) + 0.25 * a
    if jitter:
        r = r + rng.standard_normal(r.shape) * (jitter * a)
    atoms = new_atoms(len(r))
    atoms["r"] = _wrap_inside(r, 0.0, L)
    atoms["m"] = AR_MASS
    atoms["rcut"] = rc
    atoms["rns"] = rc + skin
    atoms["uid"] = np.arange(1, len(r) + 1)
    atoms["kind"] = 0
    atoms["v"] = maxwell_boltzmann(rng, atoms["m"].copy(), T)
    params = dict(kind="lj", a=eps, s=sigma, rcut=rc, skin=skin, dt=0.002, steps=1000)
    return (*_finish(atoms, (0, 0, 0), (L, L, L)), params)


def fs_tables(A_eV, p, re, rc, rho_max, nr=5000, nrho=5000, r_max=None):
    """Analytic Finnis-Sinclair-type EAM tables in MDcraft's array form:
    Rho[k] = exp(-3 (r_k/re - 1)), Vpar[k] = r_k * A exp(-p (r_k/re - 1)) (eV -> kJ/mol),
    Femb[k] = -sqrt(rho_k) (eV -> kJ/mol); r_k = k dr, rho_k = k drh."""
    r_max = r_max if r_max is not None else rc * 1.1
    dr = r_max / (nr - 1)
    drh = rho_max / (nrho - 1)
    r = np.arange(nr) * dr
    rho = np.exp(-3.0 * (r / re - 1.0))
    V = r * A_eV * np.exp(-p * (r / re - 1.0)) * EV
    F = -np.sqrt(np.arange(nrho) * drh) * EV
    return dict(rcut=rc, Femb=F, Rho=rho, Vpar=V, Nr1=nr, dr=dr, Nrh1=nrho, drh=drh)


def fcc_density(a, re, rc, decay=3.0):
    """Host density of a perfect fcc site (for the F table range)."""
    n = int(math.ceil(rc / a)) + 1
    g = np.arange(-n, n + 1)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    pts = (np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)[:, None, :] + basis[None]).reshape(-1, 3) * a
    d = np.linalg.norm(pts, axis=1)
    d = d[(d > 1e-9) & (d <= rc)]
    return float(np.exp(-decay * (d / re - 1.0)).sum())


def eam_cu_fcc(ncell=63, seed=2, T=300.0, jitter=0.01):
    """Config 2 (EAM Cu fcc 63^3 = 1,000,188 atoms)."""
    a = 0.3615
    re = 0.2556
    rc = 0.5
    skin = 0.05
    L = ncell * a
    rho_eq = fcc_density(a, re, rc)
    tab = fs_tables(0.2, 9.0, re, rc, rho_max=2.0 * rho_eq)
    rng = np.random.default_rng(seed)
    r = fcc_positions(ncell, ncell, ncell, a) + 0.25 * a
    r = r + rng.standard_normal(r.shape) * (jitter * a)
    atoms = new_atoms(len(r))
    atoms["r"] = _wrap_inside(r, 0.0, L)
    atoms["m"] = CU_MASS
    atoms["rcut"] = rc
    atoms["rns"] = rc + skin
    atoms["uid"] = np.arange(1, len(r) + 1)
    atoms["kind"] = 0
    atoms["v"] = maxwell_boltzmann(rng, atoms["m"].copy(), T)
    params = dict(kind="eam", tables=tab, rcut=rc, skin=skin, dt=0.001, steps=500)
    return (*_finish(atoms, (0, 0, 0), (L, L, L)), params)


NIAL_PAIRS = {  # (A eV, decay p, re nm) for Ni-Ni, Al-Al, Ni-Al
    (0, 0): (0.25, 8.0, 0.249),
    (1, 1): (0.15, 9.0, 0.286),
    (0, 1): (0.20, 8.5, 0.250),
}


def eam_nial_b2(ncell=80, seed=3, T=600.0, vacancy=0.005):
    """Config 3 (two-species EAM NiAl B2, ncell^3 cells, 0.5% vacancies).
    Ni = kind 0 on the cube corners, Al = kind 1 on the body centres."""
    a = 0.288
    rc = 0.6
    skin = 0.05
    L = ncell * a
    iz, iy, ix = np.meshgrid(np.arange(ncell), np.arange(ncell), np.arange(ncell), indexing="ij")
    cells = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], 1).astype(np.float64)
    pos = np.concatenate([cells[:, None, :] * a, (cells[:, None, :] + 0.5) * a], axis=1).reshape(-1, 3)
    kinds = np.tile(np.array([0, 1], dtype=np.uint16), len(cells))
    rng = np.random.default_rng(seed)
    keep = rng.random(len(pos)) >= vacancy
    pos, kinds = pos[keep] + 0.25 * a, kinds[keep]
    atoms = new_atoms(len(pos))
    atoms["r"] = _wrap_inside(pos, 0.0, L)
    atoms["kind"] = kinds
    masses = np.where(kinds == 0, NI_MASS, AL_MASS)
    atoms["m"] = masses
    atoms["rcut"] = rc
    atoms["rns"] = rc + skin
    atoms["uid"] = np.arange(1, len(pos) + 1)
    atoms["v"] = maxwell_boltzmann(rng, masses.astype(np.float64), T)
    # F range: densest environment over the three pair laws
    rho_max = 2.5 * max(
        fcc_density(a * 2 ** (1 / 3), re, rc) for (_, _, re) in NIAL_PAIRS.values())
    tabs = {k: fs_tables(A, p, re, rc, rho_max=rho_max) for k, (A, p, re) in NIAL_PAIRS.items()}
    params = dict(kind="eam_multi", tables=tabs, rcut=rc, skin=skin, dt=0.001, steps=500, nkinds=2)
    return (*_finish(atoms, (0, 0, 0), (L, L, L)), params)


def lj_liquid(nx=128, ny=128, nz=256, seed=4, rho_star=0.8442, T_star=0.72):
    """Config 4 (reduced LJ liquid, 4*nx*ny*nz atoms; 16,777,216 at the
    default), argon units."""
    sigma, eps = 0.3405, 0.0104 * EV
    a = (4.0 / rho_star) ** (1.0 / 3.0) * sigma
    tau = sigma * math.sqrt(AR_MASS / eps)
    rc, skin = 2.5 * sigma, 0.3 * sigma
    Lx, Ly, Lz = nx * a, ny * a, nz * a
    rng = np.random.default_rng(seed)
    r = fcc_positions(nx, ny, nz, a) + 0.25 * a
    # bounded displacements: a Gaussian tail would put a few pairs nearly on
    # top of each other in a system of millions and blow it apart at step 1
    r = r + rng.uniform(-0.05 * a, 0.05 * a, size=r.shape)
    atoms = new_atoms(len(r))
    atoms["r"] = np.stack([_wrap_inside(r[:, 0], 0, Lx), _wrap_inside(r[:, 1], 0, Ly),
                           _wrap_inside(r[:, 2], 0, Lz)], 1)
    atoms["m"] = AR_MASS
    atoms["rcut"] = rc
    atoms["rns"] = rc + skin
    atoms["uid"] = np.arange(1, len(r) + 1, dtype=np.uint64).astype(np.uint32)
    T = T_star * eps / KB
    atoms["v"] = maxwell_boltzmann(rng, atoms["m"].copy(), T)
    params = dict(kind="lj", a=eps, s=sigma, rcut=rc, skin=skin, dt=0.005 * tau, steps=200)
    return (*_finish(atoms, (0, 0, 0), (Lx, Ly, Lz)), params)


# ---------------------------------------------------------------------------
# Serving stream: independent requests of uneven size
# ---------------------------------------------------------------------------
SERVE_LJ = dict(kind="lj", a=0.526, mass=AR_MASS, eps=0.0104 * EV, sigma=0.3405, rcut=2.5 * 0.3405, skin=0.03,
                dt=0.002)
SERVE_EAM = dict(kind="eam", a=0.3615, mass=CU_MASS, re=0.2556, rcut=0.5, skin=0.05, dt=0.001)


def serve_eam_tables():
    """The EAM Cu tables of the serving stream (those of eam_cu_fcc)."""
    p = SERVE_EAM
    return fs_tables(0.2, 9.0, p["re"], p["rcut"], rho_max=2.0 * fcc_density(p["a"], p["re"], p["rcut"]))


def _serve_dims(n_target, min_cells):
    """fcc nx*ny*nz cells, near-cubic, 4*nx*ny*nz close to n_target, every
    dimension at least min_cells (box edge >= 2 rns)."""
    c = n_target / 4.0
    nx = max(min_cells, int(round(c ** (1.0 / 3.0))))
    ny = max(min_cells, int(round(math.sqrt(c / nx))))
    nz = max(min_cells, int(round(c / (nx * ny))))
    return nx, ny, nz


def serving_stream(count=4096, rate=2000.0, seed=5, steps=1000, n_min=256, n_max=32768, lj_share=0.6):
    """Request specs of the serving workload: Poisson arrivals at `rate`/s,
    60% LJ argon / 40% EAM Cu, atom count log-uniform in [n_min, n_max]
    rounded to fcc nx*ny*nz cells. Atoms are made per request by
    serving_atoms (seeded by the request index)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    kinds = np.where(rng.random(count) < lj_share, "lj", "eam")
    logn = rng.uniform(math.log(n_min), math.log(n_max), size=count)
    out = []
    for i in range(count):
        p = SERVE_LJ if kinds[i] == "lj" else SERVE_EAM
        min_cells = int(math.ceil(2.0 * (p["rcut"] + p["skin"]) / p["a"]))
        dims = _serve_dims(math.exp(logn[i]), min_cells)
        out.append(dict(index=i, kind=str(kinds[i]), dims=dims, n=4 * dims[0] * dims[1] * dims[2],
                        t_arrival=float(t[i]), steps=steps, dt=p["dt"], seed=seed * 1_000_003 + i))
    return out


_SERVE_TEMPLATES = {}


def serving_atoms(spec, jitter=0.01, T=300.0):
    """Atoms and domain of one serving request: fcc lattice with a seeded
    Gaussian jitter (sigma = jitter * a) and Maxwell-Boltzmann velocities."""
    p = SERVE_LJ if spec["kind"] == "lj" else SERVE_EAM
    nx, ny, nz = spec["dims"]
    key = (spec["kind"], nx, ny, nz)
    tpl = _SERVE_TEMPLATES.get(key)
    a = p["a"]
    L = np.array([nx * a, ny * a, nz * a])
    if tpl is None:
        base = fcc_positions(nx, ny, nz, a) + 0.25 * a
        t = new_atoms(len(base))
        t["m"] = p["mass"]
        t["rcut"] = p["rcut"]
        t["rns"] = p["rcut"] + p["skin"]
        t["uid"] = np.arange(1, len(base) + 1)
        t["kind"] = 0
        tpl = (base, t)
        if len(_SERVE_TEMPLATES) < 4096:
            _SERVE_TEMPLATES[key] = tpl
    base, t = tpl
    rng = np.random.default_rng(spec["seed"])
    atoms = t.copy()
    r = base + rng.standard_normal(base.shape) * (jitter * a)
    atoms["r"] = np.stack([_wrap_inside(r[:, k], 0.0, L[k]) for k in range(3)], 1)
    atoms["v"] = maxwell_boltzmann(rng, atoms["m"].copy(), T)
    return atoms, (0.0, L[0], 0.0, L[1], 0.0, L[2])
