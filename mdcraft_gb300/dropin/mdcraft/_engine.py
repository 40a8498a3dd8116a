"""The device context and host<->device coupling shared by the drop-in modules."""
from __future__ import annotations

import numpy as np

import mdcraft_gb300 as _mdg

_CTX = None


def context():
    global _CTX
    if _CTX is None:
        _CTX = _mdg.Context(0)
    return _CTX


def engine_view(data: np.ndarray) -> np.ndarray:
    """The records as the engine's flat dtype (same bytes)."""
    return data.view(_mdg.ATOM_DTYPE)


class DeviceAtoms:
    """The device system of one Atoms object (created by a VerletList, which
    knows the domain)."""

    def __init__(self, atoms, domain):
        self.atoms = atoms
        self.domain = domain
        self.n = len(atoms)
        self.sys = _mdg.System(context(), domain._d, self.n)
        self.nl = None

    def push(self):
        if len(self.atoms) != self.n:
            raise RuntimeError("atoms were resized after the VerletList was made: make a new VerletList")
        self.sys.upload(engine_view(self.atoms.data))

    def pull(self):
        out = engine_view(self.atoms.data)
        self.sys.download(out)


def device_of(atoms):
    dev = getattr(atoms, "_device", None)
    if dev is None:
        raise RuntimeError("atoms have no VerletList yet: make one (it binds the atoms to the GPU)")
    return dev
