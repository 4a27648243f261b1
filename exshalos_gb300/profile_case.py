"""One stage of the box_256 workload, for profiling the library's kernels.

    python -m exshalos_gb300.profile_case halos  [--timing]   # field, peaks, sort, growth, masses, (2)LPT
    python -m exshalos_gb300.profile_case pk     [--timing]   # CIC of the halos, then the 128-bin P(k)
    python -m exshalos_gb300.profile_case ladder [--timing]   # the 50-radius smoothing ladder
    python -m exshalos_gb300.profile_case fft                 # one 256^3 r2c + c2r round trip
    python -m exshalos_gb300.profile_case grid512             # CIC of 512^3 particles, 256-bin P(k)

Each runs one realisation of nd = 256, Lc = 2 Mpc/h (L = 512), 2LPT, barrier
a = 1, beta = 0.12, seed 1 (about 1.5 GB on the device; every field and work
array exceeds L2), after one untimed warm-up call of the same stage.
grid512 runs the CIC and P(k) stage of the nd = 512 box (L = 1024 Mpc/h):
512^3 particles in Lagrangian order at their cell centres moved by
Gaussian displacements of 2 Mpc/h rms per axis (torch generator seeded 3),
as the box's 2LPT particles arrive (about 4 GB on the device), the 512^3
CIC grid, then P(k) in 256 bins.  With
--timing the library's per-kernel-class timing is on: the quicksort levels
and the growth rounds are then launched one by one from the host instead of
as CUDA graphs, so a profiler can filter their kernels by name.
"""
import argparse
import ctypes as C
import sys

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("stage", choices=("halos", "pk", "ladder", "fft", "grid512"))
    ap.add_argument("--timing", action="store_true", help="per-kernel-class timing on (host-driven loops)")
    a = ap.parse_args(argv)
    import torch
    from exshalos_gb300 import _capi
    from exshalos_gb300.workloads import synthetic_pk
    k, P = synthetic_pk()
    k, P = k.astype(np.float32), P.astype(np.float32)
    nd, Lc, nk = 256, 2.0, 128
    L = nd * Lc
    ng = nd ** 3
    lib = _capi.load(build_if_missing=False)
    ctx = _capi.context()
    if a.timing:
        _capi.timing_enable(True)
    prm = _capi.default_params(ndx=nd, ndy=nd, ndz=nd, Lc=Lc, seed=1, DO_2LPT=1, a=1.0, beta=0.12, alpha=0.0)
    nh = C.c_int64(0)
    posh = torch.empty(3 * ng // 2, dtype=torch.float32, device="cuda")
    grid = torch.empty(ng, dtype=torch.float32, device="cuda")
    kmin, kmax = np.float32(2 * np.pi / L), np.float32(np.pi / L * nd)
    ko = np.zeros(nk, np.float32)
    po = np.zeros(nk, np.float32)
    co = np.zeros(nk, np.int64)
    cross = torch.empty(ng, dtype=torch.uint8, device="cuda")

    def halos():
        _capi.check(lib.exh_halos_box_from_pk(ctx, _capi.ptr(k), _capi.ptr(P), k.size, prm, C.byref(nh), None))

    def pk():
        _capi.check(lib.exh_halos_fetch(ctx, _capi.ptr(posh), None, None, None, None, None, None, None, None,
                                        _capi.EXH_MEM_DEVICE, None))
        _capi.check(lib.exh_grid_compute(ctx, _capi.ptr(posh), nh.value, nd, float(L), 2, 1, _capi.ptr(grid),
                                         _capi.EXH_MEM_DEVICE, None))
        _capi.check(lib.exh_power_compute(ctx, _capi.ptr(grid), nd, float(L), 2, nk, float(kmin), float(kmax),
                                          _capi.ptr(ko), _capi.ptr(po), _capi.ptr(co), _capi.EXH_MEM_DEVICE, None))

    def ladder():
        _capi.check(lib.exh_smoothing_ladder(ctx, _capi.ptr(k), _capi.ptr(P), k.size, prm, 50, 30.0,
                                             _capi.ptr(cross), None, None, _capi.EXH_MEM_DEVICE, None))

    def fft():
        x = torch.randn(ng, device="cuda")
        c = torch.empty(nd * nd * (nd // 2 + 1) * 2, device="cuda")
        _capi.check(lib.exh_fft_r2c_3d(ctx, nd, nd, nd, _capi.ptr(x), _capi.ptr(c), None))
        _capi.check(lib.exh_fft_c2r_3d(ctx, nd, nd, nd, _capi.ptr(c), _capi.ptr(x), None))

    def grid512():
        n5, Lc5, nk5 = 512, 2.0, 256
        L5 = n5 * Lc5
        g5 = torch.Generator(device="cuda").manual_seed(3)
        q5 = (torch.arange(n5, device="cuda", dtype=torch.float32) + 0.5) * Lc5
        pos5 = torch.empty((n5, n5, n5, 3), dtype=torch.float32, device="cuda")
        pos5[..., 0] = q5.view(n5, 1, 1)
        pos5[..., 1] = q5.view(1, n5, 1)
        pos5[..., 2] = q5.view(1, 1, n5)
        for s5 in range(0, n5, 64):                  # displacements slab by slab (small temporaries)
            sl = pos5[s5:s5 + 64]
            sl += torch.randn(sl.shape, generator=g5, device="cuda") * 2.0
            sl.remainder_(L5)
        pos5 = pos5.view(-1)
        grid5 = torch.empty(n5 ** 3, dtype=torch.float32, device="cuda")
        kmin5, kmax5 = np.float32(2 * np.pi / L5), np.float32(np.pi / L5 * n5)
        ko5, po5, co5 = np.zeros(nk5, np.float32), np.zeros(nk5, np.float32), np.zeros(nk5, np.int64)

        def run5():
            _capi.check(lib.exh_grid_compute(ctx, _capi.ptr(pos5), n5 ** 3, n5, float(L5), 2, 1, _capi.ptr(grid5),
                                             _capi.EXH_MEM_DEVICE, None))
            _capi.check(lib.exh_power_compute(ctx, _capi.ptr(grid5), n5, float(L5), 2, nk5, float(kmin5),
                                              float(kmax5), _capi.ptr(ko5), _capi.ptr(po5), _capi.ptr(co5),
                                              _capi.EXH_MEM_DEVICE, None))
        return run5

    if a.stage == "pk":
        halos()
        run = pk
    elif a.stage == "grid512":
        run = grid512()
    else:
        run = {"halos": halos, "ladder": ladder, "fft": fft}[a.stage]
    run()                     # warm-up: tables, plans and buffers settle
    torch.cuda.synchronize()
    run()
    torch.cuda.synchronize()
    if a.timing:
        _capi.timing_enable(False)
    print(f"profile_case {a.stage}: done", flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
