"""C++ drop-in on the GPU: MDcraft-style C++ host code (the reference tests'
call sequences) compiled against mdcraft_gb300/cxx/include and linked with
libmdg must reproduce the reference tests' golden values."""
import lzma
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _compile(out):
    from mdcraft_gb300 import build as B

    lib = B.build()
    cxx = shutil.which("g++") or "g++"
    cuda = os.path.dirname(os.path.dirname(B.nvcc()))
    cmd = [cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "mdcraft_gb300", "cxx", "include"),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
           os.path.join(ROOT, "mdcraft_gb300", "cxx", "tests", "dropin_test.cpp"),
           "-L", os.path.dirname(lib), "-lmdg", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           f"-Wl,-rpath,{os.path.dirname(lib)}", "-o", out]
    subprocess.run(cmd, check=True)


def test_cxx_dropin_compiles_on_cpu(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    _compile(str(tmp_path / "dropin_test"))


@pytest.mark.gpu
def test_cxx_dropin_reference_tests_on_gpu(tmp_path):
    exe = str(tmp_path / "dropin_test")
    _compile(exe)
    ball = tmp_path / "LMP_BALL_130k_Ar"
    al = tmp_path / "Al2009.eam.alloy"
    pair = tmp_path / "NiAlpair.eam.alloy"
    ball.write_bytes(lzma.decompress(open(os.path.join(GOLDEN, "lmp_ball_130k_ar.xz"), "rb").read()))
    al.write_bytes(lzma.decompress(open(os.path.join(GOLDEN, "al2009_eam_alloy.xz"), "rb").read()))
    pair.write_bytes(lzma.decompress(open(os.path.join(GOLDEN, "nialpair_eam_alloy.xz"), "rb").read()))
    r = subprocess.run([exe, str(ball), str(al), str(pair)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failures" in r.stdout
