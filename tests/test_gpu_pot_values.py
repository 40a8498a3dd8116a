"""Potential::value and EAM::embeddingEnergy through the C-ABI
(mdg_pot_values, mdg_pot_embedding) against the oracle's restatement of
EAM.cxx:141-174 / 562-601, pair.cxx:81-114 and LJs.cxx:61-71, on the
reference's own Al2009 setfl and NiAl pair tables: distances across the
whole table and past it, densities inside, below and above the embedding
table. Also the Python drop-in's value() / embeddingEnergy()."""
import os
import sys

import numpy as np
import pytest

import mdcraft_gb300 as mdg
from oracle import mdref as R
from tests import gpu_helpers as H
from tests import mdsupport as S

pytestmark = pytest.mark.gpu

# FP64 on both sides in the same operation order; the device contracts some
# multiply-adds, so values that cancel to near zero (the potential crossing
# zero) differ at the level of the spline terms' rounding (~1e-16 absolute)
RTOL, ATOL = 1e-12, 1e-13


def _pots():
    al = S.al2009()
    pt = S.nialpair()
    eam = (R.EAM(al["rcut"], al["Femb"], al["Rho"], al["Vpar"], al["Nr1"], al["dr"], al["Nrh1"], al["drh"]),
           mdg.EAM(al["rcut"], al["Femb"], al["Rho"], al["Vpar"], al["Nr1"], al["dr"], al["Nrh1"], al["drh"]))
    pair = (R.Pair(pt["rcut"], pt["Vpar"], pt["Nr1"], pt["dr"]), mdg.Pair(pt["rcut"], pt["Vpar"], pt["Nr1"], pt["dr"]))
    ljs = (R.LJs(0.99, 0.3405, 0.85), mdg.LJs(0.99, 0.3405, 0.85))
    lj = (R.LJsCut(0.99, 0.3405, 0.85), mdg.LJsCut(0.99, 0.3405, 0.85))
    return {"eam": (eam, al), "pair": (pair, pt), "ljs": (ljs, None), "ljcut": (lj, None)}


@pytest.mark.parametrize("kind", ["eam", "pair", "ljs", "ljcut"])
def test_values_match_oracle(kind):
    ctx = H.ctx()
    (po, pg), t = _pots()[kind]
    rng = np.random.default_rng(4)
    rmax = (t["Nr1"] + 3) * t["dr"] if t else 1.2
    r = np.concatenate([rng.uniform(0.15, rmax, 4000), [0.2, 0.85, rmax]])
    r2 = r * r
    got = pg.values(ctx, r2)
    want = R.pot_values(po, r2)
    np.testing.assert_allclose(got, want, rtol=RTOL, atol=ATOL)
    if kind == "ljcut":
        assert np.all(got == 0.0)  # Base::value
    else:
        assert np.count_nonzero(got) > 3000


def test_embedding_matches_oracle():
    ctx = H.ctx()
    (po, pg), t = _pots()["eam"]
    rng = np.random.default_rng(6)
    top = t["Nrh1"] * t["drh"]
    rho = np.concatenate([rng.uniform(0.0, top, 3000), [-0.5, -1e-9, top * 1.5, top + t["drh"]]])
    F, dF = pg.embedding(ctx, rho)
    for k, x in enumerate(rho):
        Fo, dFo = po.embedding(float(x))
        assert F[k] == pytest.approx(Fo, rel=RTOL, abs=ATOL)
        assert dF[k] == pytest.approx(dFo, rel=RTOL, abs=ATOL)
    with pytest.raises(mdg.MDGError):
        _pots()["pair"][0][1].embedding(ctx, rho)


def test_dropin_value_and_embedding(tmp_path):
    ctx = H.ctx()
    here = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "mdcraft_gb300", "dropin")
    sys.path.insert(0, here)
    try:
        from mdcraft.solver.potential import EAM, LJs, Pair
    finally:
        sys.path.remove(here)
    setfl = tmp_path / "Al2009.eam.alloy"
    setfl.write_text(S.al2009_text())
    pairfile = tmp_path / "NiAlpair.eam.alloy"
    pairfile.write_text(S.nialpair_text())
    pots = _pots()
    eam_o = pots["eam"][0][0]
    pair_o = pots["pair"][0][0]
    ljs_o = pots["ljs"][0][0]
    e = EAM(str(setfl))
    assert e.value(0.3) == pytest.approx(R.pot_values(eam_o, [0.09])[0], rel=RTOL, abs=ATOL)
    rho = np.linspace(0.0, 0.05, 11)
    assert np.allclose(e.embeddingEnergy(rho), [eam_o.embedding(float(x))[0] for x in rho], rtol=RTOL, atol=ATOL)
    p = Pair(str(pairfile))
    assert p.value(0.25) == pytest.approx(R.pot_values(pair_o, [0.0625])[0], rel=RTOL, abs=ATOL)
    lj = LJs(0.99, 0.3405, 0.85)
    r2 = np.array([0.1, 0.2, 0.3])
    np.testing.assert_allclose(lj.value(r2), R.pot_values(ljs_o, r2), rtol=RTOL, atol=ATOL)
    assert lj.value(0.4) == pytest.approx(R.pot_values(ljs_o, [0.16])[0], rel=RTOL, abs=ATOL)
    del ctx
