"""Writes tests/golden/water3_two_frames.pdb: the two-model, three-molecule
PDB text that the reference's reader test parses (NBodySimulator.jl
test/water_test.jl, the IOBuffer of "Load water molecules from a PDB file"),
copied as text from the reference checkout given as the first argument.

Usage: python tests/golden/make_pdb_fixture.py /path/to/NBodySimulator.jl
"""
import os
import sys


def main(ref):
    src = open(os.path.join(ref, "test", "water_test.jl")).read()
    start = src.index('IOBuffer("MODEL') + len('IOBuffer("')
    end = src.index('")', start)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "water3_two_frames.pdb")
    with open(out, "w") as f:
        f.write(src[start:end] + "\n")
    print(out)


if __name__ == "__main__":
    main(sys.argv[1])
