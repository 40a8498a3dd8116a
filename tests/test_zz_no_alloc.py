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
    free0 = None
    for call in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize(dev)
        if call == 1:
            free0 = torch.cuda.mem_get_info(dev)[0]
        rc = fn(m.data_ptr(), v.data_ptr(), Ep.data_ptr(), Em.data_ptr(), V.data_ptr(), n, out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize(dev)
        if call == 1:
            # nothing was allocated on the device by the second call
            assert torch.cuda.mem_get_info(dev)[0] >= free0
        o = out.cpu().numpy()
        assert o[:5] == pytest.approx(want, rel=REL)
        assert np.abs(o[5:8] - ref["vcom"]).max() <= 1e-12


def _reference(m, v, Ep, Em, V):
    """The same totals in numpy FP64."""
    tm = m.sum()
    vcom = (m[:, None] * v).sum(axis=0) / tm if tm > 0 else np.zeros(3)
    ke = 0.5 * (m * ((v - vcom) ** 2).sum(axis=1)).sum()
    return np.array([Ep.sum(), Em.sum(), ke, Ep.sum() + Em.sum() + ke, (V[:, 0] + V[:, 4] + V[:, 8]).sum(),
                     *vcom])


@pytest.mark.parametrize("n", [0, 8_388_608], ids=["empty", "max_atoms"])
def test_measure_static_edge_sizes(n):
    """No atoms (all totals zero) and the largest accepted input (every one
    of the 4096 partials in use), against a numpy FP64 reduction."""
    import torch

    rng = np.random.default_rng(17)
    m = rng.uniform(1.0, 60.0, n)
    v = rng.standard_normal((n, 3))
    Ep = rng.standard_normal(n)
    Em = -rng.uniform(0.5, 2.0, n)
    V = rng.standard_normal((n, 9))
    dev = torch.device("cuda", 0)
    td = lambda x: torch.tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)  # noqa: E731
    tm, tv, tEp, tEm, tV = td(m), td(v.T), td(Ep), td(Em), td(V.T)
    out = torch.full((8,), float("nan"), dtype=torch.float64, device=dev)
    fn = _entry()
    rc = fn(tm.data_ptr(), tv.data_ptr(), tEp.data_ptr(), tEm.data_ptr(), tV.data_ptr(), n, out.data_ptr(),
            torch.cuda.current_stream(dev).cuda_stream)
    assert rc == 0
    torch.cuda.synchronize(dev)
    o = out.cpu().numpy()
    want = _reference(m, v, Ep, Em, V)
    if n == 0:
        assert np.array_equal(o, np.zeros(8))
    else:
        scale = np.array([np.abs(Ep).sum(), np.abs(Em).sum(), want[2], np.abs(want[3]) + want[2],
                          np.abs(V).sum(), 1.0, 1.0, 1.0])
        assert np.all(np.abs(o - want) <= REL * scale)


def test_measure_static_rejects_oversize():
    import torch

    fn = _entry()
    dev = torch.device("cuda", 0)
    buf = torch.zeros(16, dtype=torch.float64, device=dev)
    p = buf.data_ptr()
    rc = fn(p, p, p, p, p, 8_388_609, p, None)
    assert rc == -1
