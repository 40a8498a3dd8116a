"""ctypes wrapper of the CPU oracle (oracle/mdref.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker, and by bench.py's CPU-baseline leg. The product path (mdcraft_gb300)
never imports this module.

The oracle restates, in plain C with the reference's FP64 operation order,
MDcraft's VerletList (mdcraft/neibs/verlet-list.cxx), Grid
(mdcraft/neibs/grid.cxx), Domain (mdcraft/lattice/domain.cxx), LJsCut
(mdcraft/solver/potential/LJs-cut.cxx), EAM (mdcraft/solver/potential/EAM.cxx),
Single/Multi solvers (mdcraft/solver/{pair,single,multi}.cxx), the Periodic
ghost boundary (mdcraft/solver/boundary/periodic.cxx) and stepper::Verlet
(mdcraft/solver/stepper/verlet.cxx).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "libmdref.so")

# mdcraft::data::Atom (mdcraft/data/atom.h:21-40), 208 bytes; V column-major.
ATOM_DTYPE = np.dtype(
    [
        ("r", "<f8", (3,)),
        ("v", "<f8", (3,)),
        ("f", "<f8", (3,)),
        ("V", "<f8", (9,)),
        ("m", "<f8"),
        ("rcut", "<f8"),
        ("rns", "<f8"),
        ("Ep", "<f8"),
        ("Em", "<f8"),
        ("nc", "<f8"),
        ("bc", "<u2"),
        ("kind", "<u2"),
        ("uid", "<u4"),
        ("tag", "<u2"),
        ("_pad", "<u2", (3,)),
    ]
)
assert ATOM_DTYPE.itemsize == 208


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(
        os.path.getmtime(os.path.join(_HERE, f)) for f in ("mdref.c", "mdref.h")
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        vp, sz, dp, ip = C.c_void_p, C.c_size_t, C.c_double, C.c_int
        L.md_domain_init.argtypes = [vp] + [dp] * 6
        L.md_domain_fit_in_period.argtypes = [vp, vp]
        L.md_domain_shortest.argtypes = [vp, vp]
        L.md_domain_nearest_distance.argtypes = [vp, vp, ip]
        L.md_domain_nearest_distance.restype = dp
        L.md_domain_belong.argtypes = [vp, vp]
        L.md_grid_build.argtypes = [vp, vp, vp, sz]
        L.md_grid_local_index3D.argtypes = [vp, vp, vp, vp]
        L.md_grid_cell_index.argtypes = [vp, vp]
        L.md_grid_cells_number.argtypes = [vp]
        L.md_grid_cell_size.argtypes = [vp]
        L.md_grid_cell_size.restype = dp
        L.md_grid_adjacent_cells.argtypes = [vp, vp, vp, vp, vp]
        L.md_nlist_create.argtypes = [sz, ip, ip, vp]
        L.md_nlist_create.restype = vp
        L.md_nlist_destroy.argtypes = [vp]
        L.md_nlist_update.argtypes = [vp, vp, vp, sz, dp]
        L.md_nlist_decide.argtypes = [vp, vp, vp, sz]
        L.md_nlist_total.argtypes = [vp]
        L.md_nlist_total.restype = sz
        L.md_nlist_export.argtypes = [vp, vp, vp]
        L.md_nlist_list_for.argtypes = [vp, vp, vp, vp, vp, sz]
        L.md_nlist_list_for.restype = sz
        L.md_nlist_grid.argtypes = [vp, vp]
        L.md_sort_atoms.argtypes = [vp, vp, sz, vp]
        L.md_pot_ljcut_create.argtypes = [dp, dp, dp]
        L.md_pot_ljcut_create.restype = vp
        L.md_pot_eam_create.argtypes = [dp, vp, vp, vp, ip, dp, ip, dp]
        L.md_pot_eam_create.restype = vp
        L.md_pot_pair_create.argtypes = [dp, vp, ip, dp]
        L.md_pot_pair_create.restype = vp
        L.md_pot_ljs_create.argtypes = [dp, dp, dp]
        L.md_pot_ljs_create.restype = vp
        L.md_pot_destroy.argtypes = [vp]
        L.md_pot_rcut.argtypes = [vp]
        L.md_pot_rcut.restype = dp
        L.md_eam_init_spline.argtypes = [vp, vp, dp, sz, ip]
        L.md_eam_slopes.argtypes = [vp, vp, vp, vp]
        L.md_eam_embedding.argtypes = [vp, dp, vp, vp]
        L.md_pot_values.argtypes = [vp, vp, sz, vp]
        L.md_solver_single.argtypes = [vp, vp, ip]
        L.md_solver_single.restype = vp
        L.md_solver_multi.argtypes = [ip, vp, ip]
        L.md_solver_multi.restype = vp
        L.md_solver_add_potential.argtypes = [vp, ip, ip, vp]
        L.md_solver_destroy.argtypes = [vp]
        L.md_solver_num_stages.argtypes = [vp]
        for fn in ("md_solver_charge", "md_solver_forces", "md_solver_virials",
                   "md_solver_stages"):
            getattr(L, fn).argtypes = [vp, vp, sz, vp]
        L.md_solver_prepare.argtypes = [vp, vp, sz]
        L.md_verlet_make_step.argtypes = [vp, vp, sz, vp, dp]
        L.md_run.argtypes = [vp, vp, sz, vp, vp, dp, C.c_long]
        L.md_run.restype = C.c_long
        L.md_measure_state.argtypes = [vp, sz, vp]
        L.md_thermo_create.restype = vp
        L.md_thermo_add.argtypes = [vp, vp]
        L.md_thermo_destroy.argtypes = [vp]
        L.md_solver_set_thermostat.argtypes = [vp, vp, C.c_uint32]
        L.md_solver_thermo_calls.argtypes = [vp]
        L.md_solver_thermo_calls.restype = C.c_uint32
        L.md_philox4x32_10.argtypes = [vp, vp, vp]
        L.md_langevin_normals.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, vp]
        L.md_hardware_threads.restype = ip
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def hardware_threads() -> int:
    return lib().md_hardware_threads()


def new_atoms(n: int) -> np.ndarray:
    """Zero atoms with the reference's default tag (uint16 max)."""
    a = np.zeros(n, dtype=ATOM_DTYPE)
    a["tag"] = 0xFFFF
    return a


class Domain:
    """mdcraft::lattice::Domain (mdcraft/lattice/domain.h:77-189)."""

    # md_domain: bmin[3], bmax[3], size[3] (f8), periodic[3], dim (i4)
    _DT = np.dtype([("bmin", "<f8", (3,)), ("bmax", "<f8", (3,)), ("size", "<f8", (3,)),
                    ("periodic", "<i4", (3,)), ("dim", "<i4")])

    def __init__(self, xmin, xmax, ymin, ymax, zmin, zmax):
        self.buf = np.zeros(1, dtype=self._DT)
        lib().md_domain_init(_ptr(self.buf), xmin, xmax, ymin, ymax, zmin, zmax)

    def set_periodic(self, axis: int, val: bool) -> None:
        self.buf["periodic"][0, axis] = int(bool(val))

    @property
    def ptr(self) -> int:
        return _ptr(self.buf)

    @property
    def dim(self) -> int:
        return int(self.buf["dim"][0])

    @property
    def bmin(self):
        return self.buf["bmin"][0].copy()

    @property
    def bmax(self):
        return self.buf["bmax"][0].copy()

    @property
    def size(self):
        return self.buf["size"][0].copy()

    @property
    def periodic(self):
        return [bool(p) for p in self.buf["periodic"][0]]

    def fit_in_period(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64).copy()
        lib().md_domain_fit_in_period(self.ptr, _ptr(v))
        return v

    def shortest(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64).copy()
        lib().md_domain_shortest(self.ptr, _ptr(v))
        return v

    def nearest_distance(self, v, axis: int) -> float:
        v = np.ascontiguousarray(v, dtype=np.float64)
        return lib().md_domain_nearest_distance(self.ptr, _ptr(v), axis)

    def belong(self, v) -> bool:
        v = np.ascontiguousarray(v, dtype=np.float64)
        return bool(lib().md_domain_belong(self.ptr, _ptr(v)))


class Grid:
    """mdcraft::neibs::Grid (mdcraft/neibs/grid.h:55-185)."""

    _DT = np.dtype([("domain_num_cells", "<i4", (3,)), ("_p", "<i4"), ("cell_sizes", "<f8", (3,)),
                    ("grid_offset", "<i4", (3,)), ("num_cells", "<i4", (3,)),
                    ("min_coords", "<f8", (3,)), ("max_coords", "<f8", (3,))])

    def __init__(self, domain: Domain):
        self.domain = domain
        self.buf = np.zeros(1, dtype=self._DT)

    def build(self, atoms: np.ndarray) -> None:
        lib().md_grid_build(_ptr(self.buf), self.domain.ptr, _ptr(atoms), len(atoms))

    def local_index3D(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        out = np.zeros(3, dtype=np.int32)
        lib().md_grid_local_index3D(_ptr(self.buf), self.domain.ptr, _ptr(v), _ptr(out))
        return out

    def cell_index(self, ijk) -> int:
        ijk = np.ascontiguousarray(ijk, dtype=np.int32)
        return lib().md_grid_cell_index(_ptr(self.buf), _ptr(ijk))

    def cells_number(self) -> int:
        return lib().md_grid_cells_number(_ptr(self.buf))

    def cell_size(self) -> float:
        return lib().md_grid_cell_size(_ptr(self.buf))

    def adjacent_cells(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        cells = np.zeros(27, dtype=np.int32)
        edge = np.zeros(3, dtype=np.int32)
        lib().md_grid_adjacent_cells(_ptr(self.buf), self.domain.ptr, _ptr(r), _ptr(cells), _ptr(edge))
        return cells, edge.astype(bool)

    @property
    def fields(self):
        return {k: self.buf[k][0].copy() for k in self._DT.names if k != "_p"}


assert Grid._DT.itemsize == 4 * 3 + 4 + 8 * 3 + 4 * 6 + 8 * 6


def sort_atoms(domain: "Domain", atoms: np.ndarray) -> np.ndarray:
    """md_sort_atoms: VerletList::sort of `atoms` (wrapped in place)."""
    if atoms.dtype != ATOM_DTYPE or not atoms.flags["C_CONTIGUOUS"]:
        raise ValueError("atoms must be a C-contiguous ATOM_DTYPE array")
    out = np.zeros_like(atoms)
    st = lib().md_sort_atoms(domain.ptr, _ptr(atoms), len(atoms), _ptr(out))
    if st not in (0, -4):
        raise RuntimeError(f"md_sort_atoms failed ({st})")
    return out


class VerletList:
    """mdcraft::neibs::VerletList (mdcraft/neibs/verlet-list.h:134-470)."""

    def __init__(self, atoms: np.ndarray, domain: Domain, threads: int = 1, half: bool = False):
        st = C.c_int(0)
        self.h = lib().md_nlist_create(len(atoms), int(half), int(threads), C.byref(st))
        if st.value != 0:
            raise RuntimeError(
                "Half Verlet lists are currently incompatible with multithreaded pair-force evaluation.")
        self.atoms = atoms
        self.domain = domain
        self.last_status = 0

    def __del__(self):
        if getattr(self, "h", None):
            lib().md_nlist_destroy(self.h)
            self.h = None

    def update(self, kbuf: float = -1.0) -> int:
        self.last_status = lib().md_nlist_update(self.h, self.domain.ptr, _ptr(self.atoms), len(self.atoms), kbuf)
        return self.last_status

    def decide(self) -> bool:
        return bool(lib().md_nlist_decide(self.h, self.domain.ptr, _ptr(self.atoms), len(self.atoms)))

    def csr(self):
        n = len(self.atoms)
        tot = lib().md_nlist_total(self.h)
        off = np.zeros(n + 1, dtype=np.uint64)
        idx = np.zeros(max(tot, 1), dtype=np.uint64)
        lib().md_nlist_export(self.h, _ptr(off), _ptr(idx))
        return off, idx[:tot]

    def lists(self):
        off, idx = self.csr()
        return [idx[off[i]:off[i + 1]] for i in range(len(off) - 1)]

    def list_for(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(4096, dtype=np.uint64)
        m = lib().md_nlist_list_for(self.h, self.domain.ptr, _ptr(self.atoms), _ptr(x), _ptr(out), len(out))
        return out[: min(m, len(out))]

    def grid(self):
        g = Grid(self.domain)
        lib().md_nlist_grid(self.h, _ptr(g.buf))
        return g

    def sort(self, atoms: np.ndarray) -> np.ndarray:
        """VerletList::sort (verlet-list.cxx:237-249): wraps `atoms` in place
        and returns a copy ordered by owning cell (x fastest), ascending
        index inside a cell."""
        return sort_atoms(self.domain, atoms)


def pot_values(pot, r2) -> np.ndarray:
    """md_pot_values: Potential::value of each squared distance."""
    r2 = np.ascontiguousarray(r2, dtype=np.float64)
    u = np.zeros(len(r2))
    lib().md_pot_values(pot.h, _ptr(r2), len(r2), _ptr(u))
    return u


class LJsCut:
    """mdcraft::solver::potential::LJsCut (LJs-cut.h:15-19)."""

    type = 1

    def __init__(self, a: float, s: float, rcut: float):
        self.h = lib().md_pot_ljcut_create(a, s, rcut)

    def rcut(self) -> float:
        return lib().md_pot_rcut(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().md_pot_destroy(self.h)
            self.h = None


class EAM:
    """mdcraft::solver::potential::EAM (EAM.h:13-22), array constructor."""

    type = 2

    def __init__(self, rcut, Femb, Rho, Vpar, Nr1, dr, Nrh1, drh):
        self._keep = [np.ascontiguousarray(x, dtype=np.float64) for x in (Femb, Rho, Vpar)]
        self.Nr1, self.Nrh1 = int(Nr1), int(Nrh1)
        self.h = lib().md_pot_eam_create(rcut, _ptr(self._keep[0]), _ptr(self._keep[1]), _ptr(self._keep[2]),
                                         self.Nr1, dr, self.Nrh1, drh)
        if not self.h:
            raise ValueError("bad EAM tables")

    def rcut(self) -> float:
        return lib().md_pot_rcut(self.h)

    def slopes(self):
        dV = np.zeros(self.Nr1)
        dR = np.zeros(self.Nr1)
        dF = np.zeros(self.Nrh1)
        lib().md_eam_slopes(self.h, _ptr(dV), _ptr(dR), _ptr(dF))
        return dV, dR, dF

    def embedding(self, rho: float):
        F = C.c_double(0)
        dF = C.c_double(0)
        lib().md_eam_embedding(self.h, rho, C.byref(F), C.byref(dF))
        return F.value, dF.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().md_pot_destroy(self.h)
            self.h = None


class LJs:
    """mdcraft::solver::potential::LJs (LJs.h:14-18)."""

    type = 4

    def __init__(self, aVr: float, rVr: float, rcut: float):
        self.h = lib().md_pot_ljs_create(aVr, rVr, rcut)

    def rcut(self) -> float:
        return lib().md_pot_rcut(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().md_pot_destroy(self.h)
            self.h = None


class Pair:
    """mdcraft::solver::potential::Pair (pair.h:13-18), array constructor:
    Vpar = r*phi(r) on a uniform grid of step dr."""

    type = 3

    def __init__(self, rcut, Vpar, Nr1, dr):
        self._keep = np.ascontiguousarray(Vpar, dtype=np.float64)
        self.h = lib().md_pot_pair_create(rcut, _ptr(self._keep), int(Nr1), dr)
        if not self.h:
            raise ValueError("bad Pair table")

    def rcut(self) -> float:
        return lib().md_pot_rcut(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().md_pot_destroy(self.h)
            self.h = None


class _Langevin(C.Structure):
    _fields_ = [("beta", C.c_double), ("temperature", C.c_double), ("time_step", C.c_double),
                ("heat", C.c_double * 3), ("U", C.c_double * 3), ("xmin", C.c_double), ("xmax", C.c_double),
                ("seed", C.c_uint64)]


class Thermostat:
    """thermostat::Langevin terms applied in order (langevin.cxx:29-42,
    compound.h); each term is a dict of Langevin's constructor arguments
    plus `seed`."""

    def __init__(self, *terms):
        self.h = lib().md_thermo_create()
        for t in terms:
            self.add(**t)

    def add(self, beta, temperature, time_step, heat_x=1, heat_y=1, heat_z=1, Ux=0.0, Uy=0.0, Uz=0.0,
            xmin=-1e15, xmax=1e15, seed=0):
        L = _Langevin(beta, temperature, time_step, (C.c_double * 3)(heat_x, heat_y, heat_z),
                      (C.c_double * 3)(Ux, Uy, Uz), xmin, xmax, seed)
        if lib().md_thermo_add(self.h, C.byref(L)) != 0:
            raise ValueError("too many thermostat terms")

    def __del__(self):
        if getattr(self, "h", None):
            lib().md_thermo_destroy(self.h)
            self.h = None


def philox4x32_10(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().md_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return out


def langevin_normals(seed, atom, call, term):
    z = np.zeros(3)
    lib().md_langevin_normals(seed, atom, call, term, _ptr(z))
    return z


class Solver:
    """Single (single.h:22-166) or Multi (multi.h:27-174) with an optional
    Periodic boundary (periodic.h:29)."""

    def __init__(self, pot=None, periodic: Domain | None = None, threads: int = 1, nkinds: int = 0):
        self._pots = []
        pd = periodic.ptr if periodic is not None else None
        if nkinds:
            self.h = lib().md_solver_multi(nkinds, pd, threads)
        else:
            self.h = lib().md_solver_single(pot.h, pd, threads)
            self._pots.append(pot)

    def add_potential(self, i, j, pot):
        self._pots.append(pot)
        return lib().md_solver_add_potential(self.h, i, j, pot.h)

    def set_thermostat(self, thermo: "Thermostat | None", calls: int = 0):
        self._thermo = thermo
        lib().md_solver_set_thermostat(self.h, thermo.h if thermo is not None else None, calls)

    def thermo_calls(self) -> int:
        return lib().md_solver_thermo_calls(self.h)

    def num_stages(self) -> int:
        return lib().md_solver_num_stages(self.h)

    def prepare(self, atoms):
        lib().md_solver_prepare(self.h, _ptr(atoms), len(atoms))

    def charge(self, atoms, nl: VerletList):
        lib().md_solver_charge(self.h, _ptr(atoms), len(atoms), nl.h)

    def forces(self, atoms, nl: VerletList):
        lib().md_solver_forces(self.h, _ptr(atoms), len(atoms), nl.h)

    def virials(self, atoms, nl: VerletList):
        lib().md_solver_virials(self.h, _ptr(atoms), len(atoms), nl.h)

    def stages(self, atoms, nl: VerletList):
        lib().md_solver_stages(self.h, _ptr(atoms), len(atoms), nl.h)

    def make_step(self, atoms, nl: VerletList, dt: float):
        lib().md_verlet_make_step(self.h, _ptr(atoms), len(atoms), nl.h, dt)

    def run(self, atoms, nl: VerletList, domain: Domain, dt: float, steps: int) -> int:
        r = lib().md_run(self.h, _ptr(atoms), len(atoms), nl.h, domain.ptr, dt, steps)
        if r < 0:
            raise RuntimeError(f"md_run failed: {r}")
        return r

    def __del__(self):
        if getattr(self, "h", None):
            lib().md_solver_destroy(self.h)
            self.h = None


def measure_state(atoms) -> dict:
    out = np.zeros(8)
    lib().md_measure_state(_ptr(atoms), len(atoms), _ptr(out))
    return {"Ep": out[0], "Em": out[1], "KE": out[2], "Etot": out[3], "virial": out[4],
            "vcom": out[5:8].copy()}


def recompute_state(solver: Solver, atoms, nl: VerletList) -> dict:
    """recompute_state (test/cxx/support/md_test_utils.h:241-253)."""
    solver.prepare(atoms)
    solver.stages(atoms, nl)
    solver.virials(atoms, nl)
    return measure_state(atoms)


def run_md_steps(solver: Solver, atoms, nl: VerletList, dt: float, steps: int, interval: int):
    """run_md_steps (test/cxx/support/md_test_utils.h:255-279)."""
    hist = []
    nl.update(-1.0)
    hist.append(recompute_state(solver, atoms, nl))
    for step in range(1, steps + 1):
        solver.make_step(atoms, nl, dt)
        if interval > 0 and step % interval == 0:
            nl.update(-1.0)
        hist.append(recompute_state(solver, atoms, nl))
    return hist
