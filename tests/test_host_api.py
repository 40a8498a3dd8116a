"""CPU checks of the host-only parts of the C-ABI (no GPU is touched):
potential constructors, thermostat records and compounds, solver set-up.
Errors come back as status codes, as include/mdg.h documents."""
import numpy as np
import pytest

import mdcraft_gb300 as mdg
from tests import mdsupport as S


@pytest.fixture(scope="module", autouse=True)
def _lib():
    from mdcraft_gb300 import build
    build.build()


def test_potential_constructors_validate():
    with pytest.raises(mdg.MDGError):
        mdg.LJsCut(1.0, 0.3, 0.0)
    with pytest.raises(mdg.MDGError):
        mdg.LJs(1.0, 0.0, 0.8)
    with pytest.raises(mdg.MDGError):
        mdg.Pair(0.6, np.zeros(2), 2, 0.01)
    assert mdg.LJs(0.9, 0.26, 0.62).rcut() == 0.62
    t = S.nialpair()
    assert mdg.Pair(t["rcut"], t["Vpar"], t["Nr1"], t["dr"]).rcut() == t["rcut"]


def test_langevin_parameters_round_trip():
    with pytest.raises(mdg.MDGError):
        mdg.Langevin(0.5, 300.0, 0.0)  # time_step must be positive
    with pytest.raises(mdg.MDGError):
        mdg.Langevin(-1.0, 300.0, 0.004)
    lg = mdg.Langevin(0.5, 300.0, 0.004, heat_y=0, Ux=0.1, xmin=-2.0, xmax=3.0, seed=77)
    assert lg.friction() == 0.5 and lg.temperature() == 300.0
    assert lg.xmin() == -2.0 and lg.xmax() == 3.0
    assert list(lg.average_velocity()) == [0.1, 0.0, 0.0]
    lg.set_temperature(150.0)
    lg.set_friction(2.0)
    lg.set_average_velocity((0.0, 0.2, 0.0))
    lg.set_dimensions(-1.0, 1.0)
    lg.set_heating_axes(1, 1, 0)
    assert (lg.temperature(), lg.friction(), lg.xmin(), lg.xmax()) == (150.0, 2.0, -1.0, 1.0)
    assert list(lg.average_velocity()) == [0.0, 0.2, 0.0]
    p = lg._get()
    assert list(p.heat) == [1, 1, 0] and p.seed == 77


def test_compound_and_solver_attachment():
    a = mdg.Langevin(0.5, 300.0, 0.004, seed=1)
    b = mdg.Langevin(0.2, 100.0, 0.004, seed=2)
    c = mdg.Compound(a, b)
    L = mdg.lib()
    assert L.mdg_thermo_compound_add(c.h, c.h) != 0  # a compound cannot contain itself
    assert L.mdg_thermo_compound_add(a.h, b.h) != 0  # a Langevin term is not a compound
    sol = mdg.Single(mdg.LJsCut(1.0, 0.3, 0.8), periodic=True)
    sol.set_thermostat(c)
    sol.set_thermostat(None)
    m = mdg.Multi(2, periodic=True)
    m.add_potential(0, 0, mdg.LJs(0.9, 0.26, 0.62))
    m.add_potential(1, 1, mdg.LJsCut(1.0, 0.3, 0.8))
    t = S.nialpair()
    m.add_potential(0, 1, mdg.Pair(t["rcut"], t["Vpar"], t["Nr1"], t["dr"]))
    assert m.num_stages() == 1  # all pair-type: one force stage (multi.cxx:28-49)
    m.add_potential(1, 1, mdg.EAM(*[S.al2009()[k] for k in ("rcut", "Femb", "Rho", "Vpar", "Nr1", "dr", "Nrh1",
                                                               "drh")]))
    assert m.num_stages() == 2  # an EAM pair adds the charge stage
