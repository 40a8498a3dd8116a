"""mdcraft_gb300 — GB300-native MD step engine (Python host over libmdg).

Python mirror of MDcraft's neighbour / potential / solver / stepper API
(python/mdcraft/{neibs,solver,solver/potential,solver/stepper} bindings of the
reference) on top of the C-ABI in include/mdg.h. Atoms live on the device in
cell-sorted order; every index crossing this API is a caller index, and atom
records use MDcraft's 208-byte Atom layout (mdcraft/data/atom.h:21-40).

There is no CPU fallback: importing works without a GPU, but creating a
Context raises when libmdg.so is missing or no CUDA device is present.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

__all__ = [
    "ATOM_DTYPE", "Context", "Domain", "System", "VerletList", "LJsCut", "EAM", "Single", "Multi", "Verlet",
    "MDGError", "new_atoms", "lib", "lib_path", "PREC_FP64", "PREC_MIXED", "Server", "Pair", "LJs",
    "Langevin", "Compound",
]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libmdg.so")

PREC_FP64 = 0
PREC_MIXED = 1

ATOM_DTYPE = np.dtype(
    [("r", "<f8", (3,)), ("v", "<f8", (3,)), ("f", "<f8", (3,)), ("V", "<f8", (9,)), ("m", "<f8"),
     ("rcut", "<f8"), ("rns", "<f8"), ("Ep", "<f8"), ("Em", "<f8"), ("nc", "<f8"), ("bc", "<u2"),
     ("kind", "<u2"), ("uid", "<u4"), ("tag", "<u2"), ("_pad", "<u2", (3,))]
)
assert ATOM_DTYPE.itemsize == 208

_ERRORS = {
    -1: "invalid argument", -2: "out of memory", -3: "neighbour overflow", -4: "out of range",
    -5: "timeout", -6: "CUDA error", -7: "bad state", -8: "no CUDA device", -9: "I/O error",
}


class MDGError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"mdg error {code} ({_ERRORS.get(code, '?')}): {msg}")
        self.code = code


_lib = None


def lib_path() -> str:
    return _LIB


def lib():
    """Loads libmdg.so (built by mdcraft_gb300.build). Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB):
        raise RuntimeError(f"libmdg.so not built ({_LIB}); run `python -m mdcraft_gb300.build`")
    L = C.CDLL(_LIB)
    vp, sz, dp, ip, u64p = C.c_void_p, C.c_size_t, C.c_double, C.c_int, C.POINTER(C.c_uint64)
    pp = C.POINTER(C.c_void_p)
    sig = {
        "mdg_last_error": ([], C.c_char_p), "mdg_version": ([], C.c_char_p),
        "mdg_ctx_create": ([ip, pp], ip), "mdg_ctx_destroy": ([vp], ip), "mdg_ctx_synchronize": ([vp], ip),
        "mdg_ctx_launch_count": ([vp, u64p], ip), "mdg_ctx_set_timing": ([vp, ip], ip),
        "mdg_ctx_stream": ([vp, pp], ip),
        "mdg_ctx_stage_time": ([vp, ip, C.POINTER(C.c_double), u64p], ip),
        "mdg_system_create": ([vp, vp, sz, pp], ip), "mdg_system_destroy": ([vp], ip),
        "mdg_system_size": ([vp, C.POINTER(C.c_size_t)], ip),
        "mdg_system_upload_atoms": ([vp, vp, sz], ip), "mdg_system_download_atoms": ([vp, vp, sz], ip),
        "mdg_system_set_positions": ([vp, vp], ip), "mdg_system_get_positions": ([vp, vp], ip),
        "mdg_system_set_velocities": ([vp, vp], ip), "mdg_system_get_velocities": ([vp, vp], ip),
        "mdg_system_get_forces": ([vp, vp], ip),
        "mdg_nlist_update": ([vp, dp, ip], ip), "mdg_nlist_decide": ([vp, C.POINTER(C.c_int)], ip),
        "mdg_nlist_total": ([vp, C.POINTER(C.c_size_t)], ip), "mdg_nlist_export": ([vp, vp, vp, sz], ip),
        "mdg_nlist_list_for": ([vp, vp, vp, sz, C.POINTER(C.c_size_t)], ip),
        "mdg_nlist_sort": ([vp, vp, sz, vp], ip),
        "mdg_nlist_grid": ([vp, vp, vp], ip), "mdg_nlist_rebuilds": ([vp, u64p], ip),
        "mdg_grid_build": ([vp, vp, vp], ip),
        "mdg_pot_atom": ([vp, vp, ip, vp, vp, sz, vp, sz, ip], ip),
        "mdg_pot_ljcut_create": ([dp, dp, dp, pp], ip),
        "mdg_pot_eam_create": ([dp, vp, vp, vp, ip, dp, ip, dp, pp], ip),
        "mdg_pot_eam_create_from_file": ([C.c_char_p, pp], ip), "mdg_pot_destroy": ([vp], ip),
        "mdg_pot_rcut": ([vp, C.POINTER(C.c_double)], ip),
        "mdg_pot_values": ([vp, vp, vp, sz, vp], ip),
        "mdg_pot_embedding": ([vp, vp, vp, sz, vp, vp], ip),
        "mdg_solver_single": ([vp, ip, pp], ip), "mdg_solver_multi": ([ip, ip, pp], ip),
        "mdg_solver_add_potential": ([vp, ip, ip, vp], ip), "mdg_solver_destroy": ([vp], ip),
        "mdg_solver_num_stages": ([vp, C.POINTER(C.c_int)], ip), "mdg_solver_set_precision": ([vp, ip], ip),
        "mdg_solver_prepare": ([vp, vp], ip), "mdg_solver_charge": ([vp, vp], ip),
        "mdg_solver_forces": ([vp, vp], ip), "mdg_solver_virials": ([vp, vp], ip),
        "mdg_solver_stages": ([vp, vp], ip), "mdg_verlet_make_step": ([vp, vp, dp], ip),
        "mdg_run": ([vp, vp, dp, C.c_long], ip), "mdg_run_host": ([vp, vp, dp, C.c_long, vp, vp, vp], ip),
        "mdg_system_measure": ([vp, vp], ip), "mdg_system_flags": ([vp, C.POINTER(C.c_uint32)], ip),
        "mdg_server_create": ([ip, vp, pp], ip), "mdg_server_destroy": ([vp], ip),
        "mdg_server_submit": ([vp, vp, vp, vp, sz, dp, C.c_long, u64p], ip),
        "mdg_server_progress": ([vp, C.POINTER(C.c_size_t)], ip),
        "mdg_server_poll": ([vp, vp, sz, C.POINTER(C.c_size_t)], ip),
        "mdg_server_wait": ([vp, C.c_uint64, dp], ip),
        "mdg_server_result": ([vp, C.c_uint64, vp, sz, vp], ip),
        "mdg_server_stats_get": ([vp, vp], ip), "mdg_server_clock": ([vp, C.POINTER(C.c_double)], ip),
        "mdg_server_footprint": ([sz, ip], sz),
        "mdg_pot_pair_create": ([dp, vp, ip, dp, pp], ip), "mdg_pot_ljs_create": ([dp, dp, dp, pp], ip),
        "mdg_pot_pair_create_from_file": ([C.c_char_p, pp], ip),
        "mdg_thermo_langevin_create": ([vp, pp], ip), "mdg_thermo_langevin_set": ([vp, vp], ip),
        "mdg_thermo_langevin_get": ([vp, vp], ip), "mdg_thermo_compound_create": ([pp], ip),
        "mdg_thermo_compound_add": ([vp, vp], ip), "mdg_thermo_destroy": ([vp], ip),
        "mdg_solver_set_thermostat": ([vp, vp], ip),
        "mdg_system_thermo_calls": ([vp, C.POINTER(C.c_uint32)], ip),
        "mdg_system_set_thermo_calls": ([vp, C.c_uint32], ip),
        "mdg_system_set_shape": ([vp, ip, ip], ip), "mdg_system_get_shape": ([vp, ip, C.POINTER(C.c_int)], ip),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(rc: int, allow=()) -> int:
    if rc != 0 and rc not in allow:
        raise MDGError(rc, lib().mdg_last_error().decode(errors="replace"))
    return rc


def _ptr(a: np.ndarray) -> int:
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data


def new_atoms(n: int) -> np.ndarray:
    """Zeroed atoms with the reference's default tag (uint16 max)."""
    a = np.zeros(n, dtype=ATOM_DTYPE)
    a["tag"] = 0xFFFF
    return a


class Context:
    """One CUDA device and one stream."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        _check(lib().mdg_ctx_create(device, C.byref(h)))
        self.h = h
        self.device = device

    def synchronize(self):
        _check(lib().mdg_ctx_synchronize(self.h))

    def launches(self) -> int:
        v = C.c_uint64()
        _check(lib().mdg_ctx_launch_count(self.h, C.byref(v)))
        return v.value

    def stream_handle(self) -> int:
        """The engine's cudaStream_t as an integer handle."""
        p = C.c_void_p()
        _check(lib().mdg_ctx_stream(self.h, C.byref(p)))
        return p.value or 0

    STAGES = {"drift": 0, "density": 1, "forces": 2, "kick": 3, "rebuild": 4}

    def set_timing(self, on: bool = True):
        """Brackets each stage launch of the step loop with CUDA events."""
        _check(lib().mdg_ctx_set_timing(self.h, int(on)))

    def stage_time(self, which: str):
        """(total ms, launches) of one stage since set_timing(True)."""
        ms = C.c_double()
        n = C.c_uint64()
        _check(lib().mdg_ctx_stage_time(self.h, self.STAGES[which], C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def close(self):
        if getattr(self, "h", None):
            lib().mdg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Domain:
    """mdcraft::lattice::Domain (mdcraft/lattice/domain.h:84-108)."""

    class _C(C.Structure):
        _fields_ = [("bmin", C.c_double * 3), ("bmax", C.c_double * 3), ("periodic", C.c_int32 * 3)]

    def __init__(self, xmin, xmax, ymin, ymax, zmin, zmax):
        self.c = Domain._C()
        self.c.bmin[:] = [xmin, ymin, zmin]
        self.c.bmax[:] = [xmax, ymax, zmax]

    def set_periodic(self, axis: int, val: bool = True):
        self.c.periodic[axis] = 1 if val else 0

    @property
    def size(self):
        return np.array([self.c.bmax[k] - self.c.bmin[k] for k in range(3)])


class System:
    """Device-resident atoms + domain (the Atoms vector every reference class binds)."""

    def __init__(self, ctx: Context, domain: Domain, atoms: np.ndarray | int):
        n = atoms if isinstance(atoms, int) else len(atoms)
        h = C.c_void_p()
        _check(lib().mdg_system_create(ctx.h, C.byref(domain.c), n, C.byref(h)))
        self.h, self.ctx, self.domain, self.n = h, ctx, domain, n
        if not isinstance(atoms, int):
            self.upload(atoms)

    def upload(self, atoms: np.ndarray):
        a = np.ascontiguousarray(atoms, dtype=ATOM_DTYPE)
        _check(lib().mdg_system_upload_atoms(self.h, _ptr(a), len(a)))

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        out = np.zeros(self.n, dtype=ATOM_DTYPE) if out is None else out
        _check(lib().mdg_system_download_atoms(self.h, _ptr(out), self.n))
        return out

    def _vec(self, fn, arr=None):
        out = np.zeros((self.n, 3)) if arr is None else np.ascontiguousarray(arr, dtype=np.float64)
        _check(fn(self.h, _ptr(out)))
        return out

    def grid_build(self) -> dict:
        """Grid::build (grid.cxx:43-95) over the system's atoms, on the device
        and without a list (positions are wrapped into the period as by a
        rebuild)."""
        ints = np.zeros(9, dtype=np.int32)
        dbl = np.zeros(3)
        _check(lib().mdg_grid_build(self.h, _ptr(ints), _ptr(dbl)))
        return {"domain_num_cells": ints[0:3], "grid_offset": ints[3:6], "num_cells": ints[6:9],
                "cell_sizes": dbl}

    def positions(self):
        return self._vec(lib().mdg_system_get_positions)

    def velocities(self):
        return self._vec(lib().mdg_system_get_velocities)

    def forces(self):
        return self._vec(lib().mdg_system_get_forces)

    def set_positions(self, xyz):
        self._vec(lib().mdg_system_set_positions, xyz)

    def set_velocities(self, xyz):
        self._vec(lib().mdg_system_set_velocities, xyz)

    SHAPES = {"list_cells_per_block": 0, "force_blocks_per_sm": 1, "density_blocks_per_sm": 2}

    def set_shape(self, name: str, value: int):
        """A launch shape of this system's kernels (0 = the measured default);
        chosen by mdcraft_gb300.tune.tune_shapes."""
        _check(lib().mdg_system_set_shape(self.h, self.SHAPES[name], int(value)))

    def get_shape(self, name: str) -> int:
        v = C.c_int()
        _check(lib().mdg_system_get_shape(self.h, self.SHAPES[name], C.byref(v)))
        return v.value

    def thermo_calls(self) -> int:
        v = C.c_uint32()
        _check(lib().mdg_system_thermo_calls(self.h, C.byref(v)))
        return v.value

    def set_thermo_calls(self, calls: int):
        _check(lib().mdg_system_set_thermo_calls(self.h, int(calls)))

    def measure(self) -> dict:
        """FP64 totals of measure_state (test/cxx/support/md_test_utils.h:214-239)."""
        buf = (C.c_double * 8)()
        _check(lib().mdg_system_measure(self.h, buf))
        v = list(buf)
        return {"Ep": v[0], "Em": v[1], "KE": v[2], "Etot": v[3], "virial": v[4], "vcom": np.array(v[5:8])}

    def flags(self) -> int:
        f = C.c_uint32()
        _check(lib().mdg_system_flags(self.h, C.byref(f)))
        return f.value

    def close(self):
        if getattr(self, "h", None):
            lib().mdg_system_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class VerletList:
    """mdcraft::neibs::VerletList (mdcraft/neibs/verlet-list.h:158-245) on a System."""

    def __init__(self, system: System, half: bool = False):
        self.sys = system
        self.half = bool(half)
        self.last_status = 0

    def update(self, kbuf: float = -1.0) -> int:
        self.last_status = _check(lib().mdg_nlist_update(self.sys.h, kbuf, int(self.half)), allow=(-4,))
        return self.last_status

    def decide(self) -> bool:
        v = C.c_int()
        _check(lib().mdg_nlist_decide(self.sys.h, C.byref(v)))
        return bool(v.value)

    def total(self) -> int:
        """Entries of the whole list, self entries included (mdg_nlist_total)."""
        tot = C.c_size_t()
        _check(lib().mdg_nlist_total(self.sys.h, C.byref(tot)))
        return tot.value

    def csr(self):
        tot = C.c_size_t()
        _check(lib().mdg_nlist_total(self.sys.h, C.byref(tot)))
        off = np.zeros(self.sys.n + 1, dtype=np.uint64)
        idx = np.zeros(max(tot.value, 1), dtype=np.uint64)
        _check(lib().mdg_nlist_export(self.sys.h, _ptr(off), _ptr(idx), tot.value))
        return off, idx[: tot.value]

    def lists(self):
        off, idx = self.csr()
        return [idx[off[i]: off[i + 1]] for i in range(self.sys.n)]

    def list_for(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(65536, dtype=np.uint64)
        cnt = C.c_size_t()
        _check(lib().mdg_nlist_list_for(self.sys.h, _ptr(x), _ptr(out), len(out), C.byref(cnt)))
        return out[: min(cnt.value, len(out))]

    def sort(self, atoms: np.ndarray) -> np.ndarray:
        """VerletList::sort (mdcraft/neibs/verlet-list.cxx:237-249): wraps
        `atoms` (a C-contiguous ATOM_DTYPE array) into the period in place and
        returns a copy ordered by owning cell (x fastest), ascending index
        inside a cell. Computed on the device; this list is not changed."""
        if atoms.dtype != ATOM_DTYPE or not atoms.flags["C_CONTIGUOUS"]:
            raise ValueError("atoms must be a C-contiguous ATOM_DTYPE array")
        out = np.zeros_like(atoms)
        _check(lib().mdg_nlist_sort(self.sys.h, _ptr(atoms), len(atoms), _ptr(out)), allow=(-4,))
        return out

    def grid(self) -> dict:
        ints = np.zeros(9, dtype=np.int32)
        dbl = np.zeros(3)
        _check(lib().mdg_nlist_grid(self.sys.h, _ptr(ints), _ptr(dbl)))
        return {"domain_num_cells": ints[0:3], "grid_offset": ints[3:6], "num_cells": ints[6:9],
                "cell_sizes": dbl}

    def rebuilds(self) -> int:
        v = C.c_uint64()
        _check(lib().mdg_nlist_rebuilds(self.sys.h, C.byref(v)))
        return v.value


class _Pot:
    def rcut(self) -> float:
        v = C.c_double()
        _check(lib().mdg_pot_rcut(self.h, C.byref(v)))
        return v.value

    def values(self, ctx: "Context", r2) -> np.ndarray:
        """Potential::value of each squared distance, on ctx's device
        (mdg_pot_values)."""
        r2 = np.ascontiguousarray(r2, dtype=np.float64).ravel()
        u = np.zeros(len(r2))
        _check(lib().mdg_pot_values(ctx.h, self.h, _ptr(r2), len(r2), _ptr(u)))
        return u

    def embedding(self, ctx: "Context", rho):
        """EAM::embeddingEnergy: (F, F') of each density (mdg_pot_embedding)."""
        rho = np.ascontiguousarray(rho, dtype=np.float64).ravel()
        F = np.zeros(len(rho))
        dF = np.zeros(len(rho))
        _check(lib().mdg_pot_embedding(ctx.h, self.h, _ptr(rho), len(rho), _ptr(F), _ptr(dF)))
        return F, dF

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().mdg_pot_destroy(self.h)
                self.h = None
        except Exception:
            pass


class LJsCut(_Pot):
    """LJsCut(a, s, rcut) (mdcraft/solver/potential/LJs-cut.h:15-19)."""

    def __init__(self, a: float, s: float, rcut: float):
        h = C.c_void_p()
        _check(lib().mdg_pot_ljcut_create(a, s, rcut, C.byref(h)))
        self.h = h


class EAM(_Pot):
    """EAM(rcut, Femb, Rho, Vpar, Nr1, dr, Nrh1, drh) (EAM.h:13-21)."""

    def __init__(self, rcut, Femb, Rho, Vpar, Nr1, dr, Nrh1, drh):
        F = np.ascontiguousarray(Femb, dtype=np.float64)
        R = np.ascontiguousarray(Rho, dtype=np.float64)
        V = np.ascontiguousarray(Vpar, dtype=np.float64)
        h = C.c_void_p()
        _check(lib().mdg_pot_eam_create(rcut, _ptr(F), _ptr(R), _ptr(V), int(Nr1), dr, int(Nrh1), drh,
                                        C.byref(h)))
        self.h = h

    @classmethod
    def from_file(cls, path: str) -> "EAM":
        """EAM(std::string filename) (EAM.cxx:55-87)."""
        obj = cls.__new__(cls)
        h = C.c_void_p()
        _check(lib().mdg_pot_eam_create_from_file(path.encode(), C.byref(h)))
        obj.h = h
        return obj


class LJs(_Pot):
    """LJs(aVr, rVr, Rcutoff) (LJs.h:14-18): smoothed Lennard-Jones."""

    def __init__(self, aVr: float, rVr: float, rcut: float):
        h = C.c_void_p()
        _check(lib().mdg_pot_ljs_create(aVr, rVr, rcut, C.byref(h)))
        self.h = h


class Pair(_Pot):
    """Pair(Rcutoff, pairPotential, NrPot, drPot) (pair.h:13-18): tabulated
    r*phi(r) on a uniform grid."""

    def __init__(self, rcut, Vpar, Nr1, dr):
        V = np.ascontiguousarray(Vpar, dtype=np.float64)
        h = C.c_void_p()
        _check(lib().mdg_pot_pair_create(rcut, _ptr(V), int(Nr1), dr, C.byref(h)))
        self.h = h

    @classmethod
    def from_file(cls, path: str) -> "Pair":
        """Pair(std::string filename) (pair.cxx:36-56)."""
        obj = cls.__new__(cls)
        h = C.c_void_p()
        _check(lib().mdg_pot_pair_create_from_file(path.encode(), C.byref(h)))
        obj.h = h
        return obj


class _LangevinParams(C.Structure):
    _fields_ = [("beta", C.c_double), ("temperature", C.c_double), ("time_step", C.c_double),
                ("heat", C.c_int32 * 3), ("_pad", C.c_int32), ("U", C.c_double * 3), ("xmin", C.c_double),
                ("xmax", C.c_double), ("seed", C.c_uint64)]


class _Thermo:
    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().mdg_thermo_destroy(self.h)
                self.h = None
        except Exception:
            pass


class Langevin(_Thermo):
    """thermostat::Langevin(beta, temperature, time_step, heat_x, heat_y,
    heat_z, Ux, Uy, Uz, xmin, xmax) (langevin.h:17-29); `seed` keys the
    Philox stream of the random force."""

    def __init__(self, beta, temperature, time_step, heat_x=1, heat_y=1, heat_z=1, Ux=0.0, Uy=0.0, Uz=0.0,
                 xmin=-1e15, xmax=1e15, seed=0):
        p = _LangevinParams(beta, temperature, time_step, (C.c_int32 * 3)(heat_x, heat_y, heat_z), 0,
                            (C.c_double * 3)(Ux, Uy, Uz), xmin, xmax, seed)
        h = C.c_void_p()
        _check(lib().mdg_thermo_langevin_create(C.byref(p), C.byref(h)))
        self.h = h

    def _get(self) -> _LangevinParams:
        p = _LangevinParams()
        _check(lib().mdg_thermo_langevin_get(self.h, C.byref(p)))
        return p

    def _set(self, p: _LangevinParams):
        _check(lib().mdg_thermo_langevin_set(self.h, C.byref(p)))

    def set_friction(self, beta):
        p = self._get()
        p.beta = beta
        self._set(p)

    def set_temperature(self, T):
        p = self._get()
        p.temperature = T
        self._set(p)

    def set_average_velocity(self, U):
        p = self._get()
        p.U = (C.c_double * 3)(*U)
        self._set(p)

    def set_heating_axes(self, heat_x=1, heat_y=1, heat_z=1):
        p = self._get()
        p.heat = (C.c_int32 * 3)(heat_x, heat_y, heat_z)
        self._set(p)

    def set_dimensions(self, xmin, xmax):
        p = self._get()
        p.xmin, p.xmax = xmin, xmax
        self._set(p)

    def friction(self):
        return self._get().beta

    def temperature(self):
        return self._get().temperature

    def average_velocity(self):
        return np.array(self._get().U[:])

    def xmin(self):
        return self._get().xmin

    def xmax(self):
        return self._get().xmax


class Compound(_Thermo):
    """thermostat::Compound (compound.h:12-24): parts apply in order."""

    def __init__(self, *parts):
        h = C.c_void_p()
        _check(lib().mdg_thermo_compound_create(C.byref(h)))
        self.h = h
        self._parts = []
        for q in parts:
            self.add(q)

    def add(self, part: _Thermo):
        self._parts.append(part)
        _check(lib().mdg_thermo_compound_add(self.h, part.h))


class _Solver:
    def __init__(self):
        self._pots = []
        self._thermo = None

    def set_thermostat(self, thermo: "_Thermo | None"):
        """The thermostat argument of Single / Multi (None: no thermostat)."""
        self._thermo = thermo
        _check(lib().mdg_solver_set_thermostat(self.h, thermo.h if thermo is not None else None))
        return self

    def num_stages(self) -> int:
        v = C.c_int()
        _check(lib().mdg_solver_num_stages(self.h, C.byref(v)))
        return v.value

    def set_precision(self, precision):
        p = {"fp64": PREC_FP64, "mixed": PREC_MIXED}.get(precision, precision)
        _check(lib().mdg_solver_set_precision(self.h, int(p)))
        return self

    def prepare(self, sys: System):
        _check(lib().mdg_solver_prepare(self.h, sys.h))

    def charge(self, sys: System):
        _check(lib().mdg_solver_charge(self.h, sys.h))

    def forces(self, sys: System):
        _check(lib().mdg_solver_forces(self.h, sys.h))

    def virials(self, sys: System):
        _check(lib().mdg_solver_virials(self.h, sys.h))

    def stages(self, sys: System):
        _check(lib().mdg_solver_stages(self.h, sys.h))

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().mdg_solver_destroy(self.h)
                self.h = None
        except Exception:
            pass


class Single(_Solver):
    """Single(pot, boundary) (mdcraft/solver/single.h:37-42); periodic=True
    selects boundary::Periodic(domain)."""

    def __init__(self, pot: _Pot, periodic: bool = False, precision="fp64"):
        super().__init__()
        h = C.c_void_p()
        _check(lib().mdg_solver_single(pot.h, int(periodic), C.byref(h)))
        self.h = h
        self._pots.append(pot)
        self.set_precision(precision)


class Multi(_Solver):
    """Multi(boundary, thermostat, nkinds) (mdcraft/solver/multi.h:42-47)."""

    def __init__(self, nkinds: int, periodic: bool = False, precision="fp64"):
        super().__init__()
        h = C.c_void_p()
        _check(lib().mdg_solver_multi(nkinds, int(periodic), C.byref(h)))
        self.h = h
        self.set_precision(precision)

    def add_potential(self, i: int, j: int, pot: _Pot):
        self._pots.append(pot)
        _check(lib().mdg_solver_add_potential(self.h, i, j, pot.h))


class Verlet:
    """stepper::Verlet (mdcraft/solver/stepper/verlet.h:34-64)."""

    def __init__(self, solver: _Solver):
        self.solver = solver

    def make_step(self, sys: System, dt: float):
        _check(lib().mdg_verlet_make_step(self.solver.h, sys.h, dt))

    def run(self, sys: System, dt: float, steps: int):
        """steps x {make_step; if decide(): update(-1)} fused on the device."""
        _check(lib().mdg_run(self.solver.h, sys.h, dt, int(steps)), allow=(-4,))

    def run_host(self, sys: System, dt: float, steps: int, pos, vel, force=None):
        fp = _ptr(force) if force is not None else None
        _check(lib().mdg_run_host(self.solver.h, sys.h, dt, int(steps), _ptr(pos), _ptr(vel), fp), allow=(-4,))


class _ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_int), ("hbm_budget", C.c_size_t), ("max_atoms", C.c_size_t),
                ("block_threads", C.c_int), ("order", C.c_int)]


class _RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("done", C.c_int), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("rebuilds", C.c_uint64), ("footprint", C.c_size_t),
                ("service_s", C.c_double)]


class _ServerStats(C.Structure):
    _fields_ = [("budget", C.c_size_t), ("used", C.c_size_t), ("peak", C.c_size_t), ("queued", C.c_size_t),
                ("running", C.c_size_t), ("finished", C.c_size_t), ("admitted", C.c_uint64),
                ("launches", C.c_uint64), ("host_admit_s", C.c_double), ("host_graph_s", C.c_double),
                ("host_retire_s", C.c_double), ("rechecked", C.c_uint64), ("host_detail_s", C.c_double * 4),
                ("live_blocks", C.c_size_t), ("busy_blocks", C.c_size_t), ("block_slots", C.c_size_t),
                ("alloc_slots", C.c_size_t), ("kernel_launches", C.c_uint64)]


class Server:
    """Continuous batching of independent systems on one GPU (mdg_server_*).

    Each request is a whole driver loop (``steps`` velocity-Verlet steps with
    the list rebuilt on decide()) over its own atoms, domain and solver. Up to
    ``slots`` requests run at once, each on its own stream, admitted in FIFO
    order (or largest first, or largest first on the tail of a backlog) as
    slots and device memory (``hbm_budget`` bytes) free up.
    """

    ORDERS = {"fifo": 0, "largest": 1, "balanced": 2}

    def __init__(self, device: int = 0, slots: int = 16, hbm_budget: int = 0, max_atoms: int = 1 << 16,
                 block_threads: int = 0, order: str = "fifo"):
        """block_threads: threads of the fused per-request block (256, 512, 640, 768, 896, 1024; 0 = 768);
        -1 runs every request as a graph loop on its slot's stream instead. order: "fifo"
        admits waiting requests in arrival order, "largest" the one with the most
        atom-steps first, "balanced" in arrival order except that the largest
        waiting request goes first once its atom-steps reach the waiting
        atom-steps per block of the fused kernel (per request slot without it)."""
        cfg = _ServerConfig(slots, hbm_budget, max_atoms, block_threads, self.ORDERS[order])
        h = C.c_void_p()
        _check(lib().mdg_server_create(device, C.byref(cfg), C.byref(h)))
        self.h = h
        self._solvers = {}  # keep solvers alive while their requests run
        self._sizes = {}

    def submit(self, solver: "_Solver", domain: Domain, atoms: np.ndarray, dt: float, steps: int) -> int:
        atoms = np.ascontiguousarray(atoms, dtype=ATOM_DTYPE)
        rid = C.c_uint64()
        _check(lib().mdg_server_submit(self.h, solver.h, C.byref(domain.c), _ptr(atoms), len(atoms), dt, steps,
                                       C.byref(rid)))
        self._solvers[rid.value] = solver
        self._sizes[rid.value] = len(atoms)
        return rid.value

    def progress(self) -> int:
        k = C.c_size_t()
        _check(lib().mdg_server_progress(self.h, C.byref(k)))
        return k.value

    def poll(self, cap: int = 1024) -> list:
        ids = np.zeros(cap, dtype=np.uint64)
        k = C.c_size_t()
        _check(lib().mdg_server_poll(self.h, _ptr(ids), cap, C.byref(k)))
        return [int(x) for x in ids[:k.value]]

    def wait(self, rid: int, timeout: float = 60.0):
        _check(lib().mdg_server_wait(self.h, rid, timeout))

    def result(self, rid: int, atoms: bool = True):
        """(atoms or None, info dict) of a finished request; forgets it."""
        info = _RequestInfo()
        out = new_atoms(self._sizes[rid]) if atoms else None
        _check(lib().mdg_server_result(self.h, rid, _ptr(out) if atoms else None, len(out) if atoms else 0,
                                       C.byref(info)))
        self._solvers.pop(rid, None)
        self._sizes.pop(rid, None)
        d = {k: getattr(info, k) for k, _ in _RequestInfo._fields_}
        return out, d

    def stats(self) -> dict:
        st = _ServerStats()
        _check(lib().mdg_server_stats_get(self.h, C.byref(st)))
        d = {k: getattr(st, k) for k, _ in _ServerStats._fields_}
        d["host_detail_s"] = list(d["host_detail_s"])
        return d

    def clock(self) -> float:
        t = C.c_double()
        _check(lib().mdg_server_clock(self.h, C.byref(t)))
        return t.value

    @staticmethod
    def footprint(n: int, neighbours: int) -> int:
        return int(lib().mdg_server_footprint(n, neighbours))

    def close(self):
        if getattr(self, "h", None):
            lib().mdg_server_destroy(self.h)
            self.h = None
            self._solvers.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
