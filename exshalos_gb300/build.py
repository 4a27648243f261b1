"""In-tree build of libexh_gb300.so (sm_103a).

Every translation unit under csrc/ is compiled in parallel with nvcc for
compute_103a/sm_103a only, then linked into exshalos_gb300/_lib/.  Host code
is compiled with floating-point contraction off: the halo-finder tables must
round exactly like the reference's C expressions.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(HERE, "_lib", "obj")
INC = os.path.join(os.path.dirname(HERE), "include")
LIBNAME = "libexh_gb300.so"

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
          f"-I{INC}", f"-I{CSRC}"]


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(INC, "exh_gb300.h"))
    return hs


def lib_path():
    return os.path.join(OUT, LIBNAME)


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose):
    obj = os.path.join(OBJ, src + ".o")
    deps = [os.path.join(CSRC, src)] + headers() + [__file__]
    if not _stale(obj, deps):
        return obj
    cmd = [NVCC] + ARCH + COMMON + ["-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-warn-spills"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr)
    return obj


def build(verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=jobs or min(16, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    so = lib_path()
    if _stale(so, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", so] + objs + ["-lcuda"] * 0
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return so


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
