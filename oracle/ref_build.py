"""REFERENCE BUILD recipe — test infrastructure only.

Compiles the reference's own C for the mock path, unmodified and where it
lies in the reference tree, into oracle/_ref/ (git-ignored):

  libref_exshalos.so  src/exshalos/{exshalos_h,density_grid,find_halos,lpt,
                      box,cells_in_spheres,fftlog}.c + oracle/ref_driver_exshalos.c
  libref_spectrum.so  src/spectrum/{spectrum_h,gridmodule,powermodule}.c
                      + oracle/ref_driver_spectrum.c

The reference links against FFTW3 (single precision) and GSL, neither of
which exists in this image.  Their entry points are supplied by the
project-written stand-ins in oracle/ref_shim/ (headers) and oracle/ref_shim.c,
which call the oracle's own restatements (oracle/orc_fft.c in float,
orc_rng.c, orc_spline.c).  The libraries therefore pin the oracle's
restatement of the reference's loops (mode loop, peaks, quicksort, growth,
masses, LPT stencils, CIC, binning), not FFTW's or GSL's arithmetic.
Flags follow the reference's setup.py (-fopenmp) with contraction off, as on
its x86-64 build.  The reference tree is read from the first argument, the
EXH_REFERENCE_TREE environment variable, or the default path below; without
it nothing is built (the GPU machine has no reference tree).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
DEFAULT_TREE = "/root/reference"

EXSHALOS = ["exshalos_h.c", "density_grid.c", "find_halos.c", "lpt.c", "box.c", "cells_in_spheres.c", "fftlog.c"]
SPECTRUM = ["spectrum_h.c", "gridmodule.c", "powermodule.c"]
ORACLE = ["ref_shim.c", "orc_fft.c", "orc_rng.c", "orc_spline.c"]


def tree(arg=None):
    t = arg or os.environ.get("EXH_REFERENCE_TREE") or DEFAULT_TREE
    return t if os.path.isfile(os.path.join(t, "src", "exshalos", "find_halos.c")) else None


def _needs(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(ref_tree=None, verbose=False):
    """Build both libraries (when the reference tree exists); returns their
    paths, or None."""
    t = tree(ref_tree)
    if t is None:
        return None
    os.makedirs(OUT, exist_ok=True)
    libs = {
        "exshalos": ([os.path.join(t, "src", "exshalos", f) for f in EXSHALOS], "ref_driver_exshalos.c",
                     os.path.join(t, "include", "exshalos")),
        "spectrum": ([os.path.join(t, "src", "spectrum", f) for f in SPECTRUM], "ref_driver_spectrum.c",
                     os.path.join(t, "include", "spectrum")),
    }
    shim_hdrs = [os.path.join(r, f) for r, _, fs in os.walk(os.path.join(HERE, "ref_shim")) for f in fs]
    out, procs = {}, []
    for name, (srcs, driver, inc) in libs.items():
        so = os.path.join(OUT, f"libref_{name}.so")
        out[name] = so
        mine = [os.path.join(HERE, f) for f in ORACLE + [driver]]
        if not _needs(so, srcs + mine + shim_hdrs + [os.path.join(HERE, "orc.h"), __file__]):
            continue
        cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
               "-w", "-DORC_REAL=float", "-I", os.path.join(HERE, "ref_shim"), "-I", inc, "-I", HERE,
               "-Wl,--no-undefined", "-o", so] + srcs + mine + ["-lm"]
        if verbose:
            print(" ".join(cmd))
        procs.append((so, subprocess.Popen(cmd, stderr=subprocess.PIPE, text=True)))
    for so, pr in procs:
        _, err = pr.communicate()
        if pr.returncode != 0:
            raise RuntimeError(f"reference build failed for {so}:\n{err}")
    return out


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, verbose=True))
