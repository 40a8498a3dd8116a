"""mdg_measure_static — the measurement reduction for callers that cannot
allocate device memory (a foreign pool owns the heap, no allocation may
synchronise, or only pre-registered buffers are handed out). It must return
what mdg_system_measure returns for the same atoms, call after call, using
only its static device scratch and the caller's arrays.

Named to be collected last: it shares device state (the static scratch) with
nothing else, and a failure here leaves every other test already run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-10  # the FP64 tolerance of the parity tests


def _entry():
    import mdcraft_gb300 as mdg

    fn = mdg.lib().mdg_measure_static
    fn.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def test_measure_static_matches_measure_on_two_calls():
    import torch

    from mdcraft_gb300 import workloads as W
    from tests import gpu_helpers as H

    atoms, box, per, p = W.eam_cu_fcc(ncell=10)
    _, g = H.make_pair(atoms, box, (1, 1, 1), p, precision="fp64")
    g["nl"].update(-1.0)
    g["solver"].prepare(g["sys"])
    g["solver"].stages(g["sys"])
    g["solver"].virials(g["sys"])
    ref = g["sys"].measure()  # the existing entry point
    a = g["sys"].download()
    n = len(a)

    dev = torch.device("cuda", 0)
    m = torch.tensor(a["m"], dtype=torch.float64, device=dev)
    v = torch.tensor(np.ascontiguousarray(a["v"].T), dtype=torch.float64, device=dev)
    Ep = torch.tensor(a["Ep"], dtype=torch.float64, device=dev)
    Em = torch.tensor(a["Em"], dtype=torch.float64, device=dev)
    V = torch.tensor(np.ascontiguousarray(a["V"].T), dtype=torch.float64, device=dev)
    out = torch.full((8,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    fn = _entry()
    want = [ref["Ep"], ref["Em"], ref["KE"], ref["Etot"], ref["virial"]]
    for _ in range(2):
        out.fill_(float("nan"))
        rc = fn(m.data_ptr(), v.data_ptr(), Ep.data_ptr(), Em.data_ptr(), V.data_ptr(), n, out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize(dev)
        o = out.cpu().numpy()
        assert o[:5] == pytest.approx(want, rel=REL)
        assert np.abs(o[5:8] - ref["vcom"]).max() <= 1e-12


def test_measure_static_rejects_oversize():
    import torch

    fn = _entry()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float64, device=dev)
    p = buf.data_ptr()
    rc = fn(p, p, p, p, p, 8_388_609, p, None)
    assert rc == -1
