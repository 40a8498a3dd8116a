"""CPU checks of the drop-in boundary: libmdg.so builds, loads and exports
every entry point declared in include/mdg.h; without a GPU, creating a
context fails loudly (no CPU fallback)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "mdg.h")).read()
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(mdg_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "mdg_nlist_update" in syms and "mdg_run" in syms and len(syms) > 40


def test_library_exports_every_declared_symbol():
    from mdcraft_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_context_without_gpu_raises():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import mdcraft_gb300 as mdg
    from mdcraft_gb300 import build
    build.build()
    with pytest.raises(mdg.MDGError) as e:
        mdg.Context(0)
    assert e.value.code == -8
