"""Times the reference's own CUDA build beside this library on the plain FP64
single-solve configuration (TEST INFRASTRUCTURE: run by hand on a GPU machine;
prints one JSON line).

Workload: N = 1000 point forces uniform in the unit cube, forces N(0, 1),
alpha 10, eps 0.01, splitting d = 0.125 (xi = 8), targets = sources.
* reference: kernelFourier + kernelReal of cuda/periodicBrinkman.h:219-425,
  built from the reference's sources into oracle/_ref/ref_kernels.* and
  launched as its periodicBrinkman() does (oracle/ref_launch.cpp), filling
  the 3000 x 3000 dense matrix; velocities are A f (the caller's job in the
  reference: one cuBLAS-free torch matvec here, timed with it);
* dense drop-in: pb_periodic_brinkman on the same matrix;
* spectral: pb_solve, mixed precision and FP64 (grid 64^3, support 16, the
  configuration's k-space parameters), plans replayed.
Real shells M = 1 (27 images, erfc(1/0.125) ~ 1e-29) and Fourier shells
N = 15 (31^3 wave vectors) are the converged dense sums.  Usage:
    python oracle/time_ref_cuda.py [--reps 3]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--n", type=int, default=1000)
    args = ap.parse_args()
    import torch

    import oracle
    import periodicbrinkman_gb300 as pb
    from periodicbrinkman_gb300.api import Plan, make_params

    n, L, a, e, d, M, N = args.n, 1.0, 10.0, 0.01, 0.125, 1, 15
    rng = np.random.default_rng(1000)
    x = rng.random((n, 3))
    f = rng.standard_normal((n, 3))
    xd, fd = torch.from_numpy(x).cuda(), torch.from_numpy(f).cuda()
    fv = fd.reshape(-1)

    def dense(fn):
        A = torch.zeros((3 * n, 3 * n), dtype=torch.float64, device="cuda").t()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn(A)
        u = (A @ fv).reshape(n, 3)
        torch.cuda.synchronize()
        return time.perf_counter() - t0, u

    def ref_fn(A):
        oracle.ref_gpu_periodic_brinkman(A.data_ptr(), xd.data_ptr(), n, xd.data_ptr(), n, a, d, e, M, N, (L, L, L))

    def ours_fn(A):
        pb.periodicBrinkman(A, xd, xd, a, d, e, M, N, (L, L, L))

    out = {"workload": f"plain FP64 single solve N={n} alpha={a} eps={e} d={d} L={L}, dense shells M={M} N={N}"}
    t_ref, u_ref = min((dense(ref_fn) for _ in range(args.reps)), key=lambda t: t[0])
    t_our, u_our = min((dense(ours_fn) for _ in range(args.reps)), key=lambda t: t[0])
    out["reference_cuda_dense_s"] = t_ref
    out["dense_drop_in_s"] = t_our
    out["dense_rel_diff"] = float((u_our - u_ref).abs().max() / u_ref.abs().max())
    for prec in ("mixed", "fp64"):
        p = make_params(n, L, a, e, tol=1e-6 if prec == "mixed" else 1e-10, M=64, P=16, precision=prec)
        with Plan(p) as plan:
            U = torch.empty_like(xd)
            for _ in range(3):
                plan.execute(xd, fd, U=U)
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            torch.cuda.synchronize()
            ev[0].record()
            for _ in range(20):
                plan.execute(xd, fd, U=U)
            ev[1].record()
            torch.cuda.synchronize()
            out[f"spectral_{prec}_s"] = ev[0].elapsed_time(ev[1]) / 20 / 1e3
            out[f"spectral_{prec}_rel_diff_vs_reference"] = float((U - u_ref).abs().max() / u_ref.abs().max())
    print(json.dumps(out))


if __name__ == "__main__":
    main()
