"""Parity at the benchmark sizes: EAM Cu fcc 63^3 (1,000,188 atoms) and the
two-species EAM NiAl B2 80^3 with 0.5% vacancies (1,018,903 atoms), the
configurations the throughput is quoted on. The cell grid (41^3 and 35^3
cells here) differs from every scaled-down case, so these run at full size.

Bars, against the oracle (the C restatement of the reference, all host
threads) on the same seeded inputs:
- neighbour sets bit-identical (sorted per atom, self included;
  mdcraft/neibs/verlet-list.cxx:306-400) and wrapped positions identical;
- FP64 forces, Ep, Em, nc and V within 1e-10 relative;
- mixed-precision forces within ||dF||_2/||F||_2 <= 1e-5, the max over atoms
  of |dF_i| / RMS|F| reported (and bounded), and the energies of the mixed
  form (evaluated in FP64 on its positions) equal to the FP64 form's."""
import numpy as np
import pytest

from mdcraft_gb300 import workloads as W
from oracle import mdref as R
from tests import gpu_helpers as H

pytestmark = pytest.mark.gpu

FP64_REL = 1e-10
MIXED_L2 = 1e-5
MIXED_MAX = 5e-5

CASES = [("eam_cu_63", lambda: W.eam_cu_fcc(ncell=63)), ("nial_b2_80", lambda: W.eam_nial_b2(ncell=80))]


def _sorted_entries(off, idx):
    """Per-atom segments of a CSR list sorted ascending, as one array."""
    off = off.astype(np.int64)
    owner = np.repeat(np.arange(len(off) - 1, dtype=np.uint64), np.diff(off))
    return np.sort((owner << np.uint64(32)) | idx.astype(np.uint64))


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_full_size_parity(case):
    atoms, box, per, p = case[1]()
    o, g = H.make_pair(atoms, box, (1, 1, 1), p, precision="fp64")
    o["nl"].update(-1.0)
    g["nl"].update(-1.0)

    # neighbour sets and wrapped positions
    off_o, idx_o = o["nl"].csr()
    off_g, idx_g = g["nl"].csr()
    assert np.array_equal(off_o, off_g), "per-atom list lengths differ from the oracle"
    assert np.array_equal(_sorted_entries(off_o, idx_o), _sorted_entries(off_g, idx_g))
    del idx_o, idx_g
    assert np.array_equal(g["sys"].positions(), o["atoms"]["r"])

    # FP64 form against the oracle
    so, ao = o["solver"], o["atoms"]
    so.prepare(ao)
    so.stages(ao, o["nl"])
    so.virials(ao, o["nl"])
    sg, sysg = g["solver"], g["sys"]
    sg.prepare(sysg)
    sg.stages(sysg)
    sg.virials(sysg)
    a = sysg.download()
    fo = ao["f"]
    scale = np.sqrt(np.mean(np.sum(fo ** 2, axis=1)))
    assert np.max(np.abs(a["f"] - fo)) <= FP64_REL * scale
    for key in ("Ep", "Em", "nc"):
        ref = ao[key]
        assert np.max(np.abs(a[key] - ref)) <= FP64_REL * np.max(np.abs(ref))
    assert np.max(np.abs(a["V"] - ao["V"])) <= FP64_REL * np.max(np.abs(ao["V"]))
    mo = R.measure_state(ao)
    m64 = sysg.measure()
    for key in ("Ep", "Em", "virial"):
        assert m64[key] == pytest.approx(mo[key], rel=FP64_REL)

    # mixed form at the same positions
    sg.set_precision("mixed")
    sg.prepare(sysg)
    sg.stages(sysg)
    f = sysg.forces()
    emax, el2 = H.force_error(f, fo)
    sg.virials(sysg)
    mmx = sysg.measure()
    e_ref = abs(mo["Ep"] + mo["Em"])
    e_err = abs((mmx["Ep"] + mmx["Em"]) - (mo["Ep"] + mo["Em"])) / e_ref
    print(f"{case[0]}: n={len(atoms)} mixed force error L2 {el2:.3e} max/RMS {emax:.3e}; "
          f"energy error {e_err:.2e}")
    assert el2 <= MIXED_L2
    assert emax <= MIXED_MAX
    assert e_err <= FP64_REL
