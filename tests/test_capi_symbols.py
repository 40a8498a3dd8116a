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


FIELDS = ["r", "v", "f", "V", "m", "rcut", "rns", "Ep", "Em", "nc", "bc", "kind", "uid", "tag"]


def test_atom_record_layouts_agree(tmp_path):
    """mdg_atom of the C-ABI, the C++ drop-in's mdcraft::data::Atom, the
    binding's ATOM_DTYPE, the Python drop-in's nested record
    (mdcraft.data.Atoms) and the oracle's record place every field of
    mdcraft/data/atom.h:21-40 at the same byte offset, 208 bytes in all."""
    import shutil
    import subprocess
    import sys

    dropin = os.path.join(ROOT, "mdcraft_gb300", "dropin")
    sys.path.insert(0, dropin)
    try:
        from mdcraft.data import ATOM as DROPIN_ATOM
    finally:
        sys.path.remove(dropin)

    import mdcraft_gb300 as mdg
    from oracle import mdref as R
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    lines = ["#include <cstddef>", "#include <cstdio>", "#include <mdcraft/data/atom.h>", "int main() {"]
    for name in FIELDS:
        lines.append(f'  std::printf("{name} %zu %zu\\n", offsetof(mdg_atom, {name}), '
                     f'offsetof(mdcraft::data::Atom, {name}));')
    lines.append('  std::printf("size %zu %zu\\n", sizeof(mdg_atom), sizeof(mdcraft::data::Atom));')
    lines.append("  return 0;\n}")
    src = tmp_path / "layout.cpp"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([gxx, "-std=c++17", "-Wno-invalid-offsetof", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "mdcraft_gb300", "cxx", "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    got = {}
    for row in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n"):
        if row:
            name, c_off, cxx_off = row.split()
            got[name] = (int(c_off), int(cxx_off))
    assert got.pop("size") == (208, 208)
    for name in FIELDS:
        want = mdg.ATOM_DTYPE.fields[name][1]
        assert got[name] == (want, want), name
        assert R.ATOM_DTYPE.fields[name][1] == want, name
        assert DROPIN_ATOM.fields[name][1] == want, name
    assert mdg.ATOM_DTYPE.itemsize == R.ATOM_DTYPE.itemsize == DROPIN_ATOM.itemsize == 208
