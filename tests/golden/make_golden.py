"""Regenerates the golden fixtures in this directory from the reference tree.

Run in a container that has the reference checkout (its path is the first
argument, default /root/reference).  The reference's sphere table
(src/exshalos/cells_in_spheres.c:4) is read as text and written as one
integer per line; the oracle and the CUDA library must reproduce it.
"""
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
HERE = os.path.dirname(os.path.abspath(__file__))


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
    print("cells_in_spheres:", cells_in_spheres())
