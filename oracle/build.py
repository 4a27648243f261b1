"""ORACLE build recipe — test infrastructure only.

Compiles the C restatement in this directory twice into oracle/_build/:
  liborc_f32.so  (ORC_REAL=float: the reference's own precision)
  liborc_f64.so  (ORC_REAL=double: the FP64 oracle)
Floating-point contraction is disabled so that float/double rounding follows
the C expressions one operation at a time on both x86-64 and aarch64.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = ["orc_rng.c", "orc_spline.c", "orc_setup.c", "orc_fft.c", "orc_field.c",
        "orc_halos.c", "orc_lpt.c", "orc_spectrum.c", "orc_pipeline.c", "orc_hod.c"]
OUT = os.path.join(HERE, "_build")


def _needs(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    deps = [os.path.join(HERE, s) for s in SRCS] + [os.path.join(HERE, "orc.h")]
    outs = {}
    procs = []
    for tag, real in (("f32", "float"), ("f64", "double")):
        so = os.path.join(OUT, f"liborc_{tag}.so")
        outs[tag] = so
        if not _needs(so, deps):
            continue
        cmd = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp",
               "-ffp-contract=off", "-fno-fast-math", f"-DORC_REAL={real}",
               "-o", so] + deps[:-1] + ["-lm"]
        if verbose:
            print(" ".join(cmd))
        procs.append((so, subprocess.Popen(cmd, stderr=subprocess.PIPE, text=True)))
    for so, pr in procs:
        _, err = pr.communicate()
        if pr.returncode != 0:
            raise RuntimeError(f"oracle build failed for {so}:\n{err}")
    return outs


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
