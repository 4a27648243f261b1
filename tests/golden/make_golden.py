"""Regenerates the golden fixtures in this directory from the reference tree.

Run where the reference checkout exists, with its path as the one required
argument:  python tests/golden/make_golden.py <reference tree>.  The
reference's sphere table
(src/exshalos/cells_in_spheres.c:4) is read as text and written as one
integer per line; the oracle and the CUDA library must reproduce it.
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = None


def cells_in_spheres():
    src = open(os.path.join(REF, "src/exshalos/cells_in_spheres.c")).read()
    body = src[src.index("{") + 1: src.rindex("}")]
    vals = [int(v) for v in re.findall(r"-?\d+", body)]
    with open(os.path.join(HERE, "cells_in_spheres.txt"), "w") as f:
        f.write("# CELLS_IN_SPHERES, src/exshalos/cells_in_spheres.c:4 (%d entries)\n" % len(vals))
        for v in vals:
            f.write("%d\n" % v)
    return len(vals)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference tree>")
    REF = sys.argv[1]
    print("cells_in_spheres:", cells_in_spheres())
