"""mdcraft.solver.thermostat (python/mdcraft/solver/thermostat/_thermostat.cxx):
Thermostat (no-op), Langevin and Compound on the GPU engine.

The reference seeds each Langevin from std::random_device, so no two runs
repeat; here each object draws from a Philox stream keyed by `seed`, a fresh
random key unless one is given (pass `seed=` to repeat a run)."""
from __future__ import annotations

import os

import mdcraft_gb300 as _mdg


class Thermostat:
    """thermostat::Base: applies nothing."""

    _t = None


class Langevin(Thermostat):
    def __init__(self, beta, temperature, time_step, heat_x=1, heat_y=1, heat_z=1, Ux=0.0, Uy=0.0, Uz=0.0,
                 xmin=-1e15, xmax=1e15, seed=None):
        if seed is None:
            seed = int.from_bytes(os.urandom(8), "little")
        self._t = _mdg.Langevin(beta, temperature, time_step, heat_x, heat_y, heat_z, Ux, Uy, Uz, xmin, xmax,
                                seed)

    @property
    def temperature(self) -> float:
        return self._t.temperature()

    @property
    def friction(self) -> float:
        return self._t.friction()

    @property
    def Ux(self) -> float:
        return float(self._t.average_velocity()[0])

    @property
    def Uy(self) -> float:
        return float(self._t.average_velocity()[1])

    @property
    def Uz(self) -> float:
        return float(self._t.average_velocity()[2])

    @property
    def xmin(self) -> float:
        return self._t.xmin()

    @property
    def xmax(self) -> float:
        return self._t.xmax()

    def set_average_velocity(self, Ux=0.0, Uy=0.0, Uz=0.0):
        self._t.set_average_velocity((Ux, Uy, Uz))

    def set_temperature(self, T):
        self._t.set_temperature(T)

    def set_friction(self, beta):
        self._t.set_friction(beta)

    def set_heating_axes(self, heat_x=1, heat_y=1, heat_z=1):
        self._t.set_heating_axes(heat_x, heat_y, heat_z)

    def set_dimensions(self, xmin=-1e15, xmax=1e15):
        self._t.set_dimensions(xmin, xmax)


class Compound(Thermostat):
    def __init__(self):
        self._t = _mdg.Compound()
        self._parts = []

    def add(self, thermostat: Thermostat):
        if thermostat._t is None:
            return  # the no-op thermostat adds nothing
        self._parts.append(thermostat)
        self._t.add(thermostat._t)
