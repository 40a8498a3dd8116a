"""Regenerates the golden input fixtures in this folder from the reference's
own test fixtures (run in a container where the reference is checked out).

- lmp_ball_130k_ar.xz   <- test/cxx/LMP_BALL_130k_Ar (LAMMPS data, 130,124 Ar
  atoms) used by test/cxx/solver/test_argon_ball_md.cxx
- al2009_eam_alloy.xz   <- test/python/solver/Al2009.eam.alloy (setfl EAM Al)
  used by test/cxx/solver/test_aluminum_bulk_eam.cxx
- nialpair_eam_alloy.xz <- problems/NiAl/NiAlpair.eam.alloy (tabulated Ni-Al
  pair term read by Pair(filename)) used by problems/NiAl/test-NiAl.py

The files are byte-identical copies, xz-compressed, so the tests parse them
exactly as the reference's loaders do. The golden VALUES the tests check are
the constants asserted in those reference test files (cited in the tests).

usage: python tests/golden/make_golden.py /path/to/reference
"""
import lzma
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref: str) -> None:
    pairs = [
        (os.path.join(ref, "test", "cxx", "LMP_BALL_130k_Ar"), "lmp_ball_130k_ar.xz"),
        (os.path.join(ref, "test", "python", "solver", "Al2009.eam.alloy"), "al2009_eam_alloy.xz"),
        (os.path.join(ref, "problems", "NiAl", "NiAlpair.eam.alloy"), "nialpair_eam_alloy.xz"),
    ]
    for src, dst in pairs:
        raw = open(src, "rb").read()
        with open(os.path.join(HERE, dst), "wb") as f:
            f.write(lzma.compress(raw, preset=9))
        print(f"{dst}: {len(raw)} -> {os.path.getsize(os.path.join(HERE, dst))} bytes")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/reference")
    main(sys.argv[1])
