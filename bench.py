"""Benchmark: Brinkman solves/s on one GB300 (and N independent replicas).

Workload (one "step" = one full solve): the single large solve of N = 100,000
point forces uniform in the unit cube, forces N(0,1), alpha = 20,
eps = 0.005, 128^3 grid, P = 12, max relative error <= 1e-6, mixed precision
(FP32 bulk), splitting and cutoff chosen by the autotuner.  Synthetic seeded
inputs stand in for the reference's (unpublished) data.

  value : solves/s with inputs resident in HBM (plan graph replay), device
          time by CUDA events; L2 flushed (256 MB write) between steps.
  e2e   : the same through the public API with pinned HOST buffers, the
          host->device input copies and device->host velocity copy inside
          the timed region.
  roofline : the dominant kernel (largest share of a solve).
  cpu_baseline : the FP64 oracle (C, OpenMP, all host threads) on a bounded
          sample (all sources, a subset of targets), extrapolated to a full
          solve.

--impl reference times the reference's algorithm on the host cores (the
oracle port of its direct-Ewald sums; its own host code cannot be built on
the GPU machine because its sources stay out of this repository).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="single_solve_N1e5_uniform_alpha20_eps0.005_grid128_P12_tol1e-6_mixed", n=100_000, L=1.0,
                alpha=20.0, eps=0.005, M=128, P=12, tol=1e-6, seed=2000)
METRIC = "Brinkman solves/s at <=1e-6 max rel err (mixed precision, single solve, N=1e5)"


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[3 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def make_inputs(w):
    rng = np.random.default_rng(w["seed"])
    x = rng.random((w["n"], 3)) * w["L"]
    f = rng.standard_normal((w["n"], 3))
    return x, f


def cpu_baseline(w, budget_s=20.0):
    """FP64 oracle on a bounded sample: all n sources, m1 and m2 targets;
    a full solve is extrapolated linearly in the number of targets."""
    import oracle

    x, f = make_inputs(w)
    n = w["n"]
    th = oracle.num_threads()
    rng = np.random.default_rng(1)
    idx = rng.choice(n, 256, replace=False)
    times = {}
    d = oracle.choose_split(n, 128, w["L"])
    for m in (64, 128):
        t0 = time.perf_counter()
        oracle.ewald_velocity(x[idx[:m]], x, f, w["L"], w["alpha"], w["eps"], d=d)
        times[m] = time.perf_counter() - t0
    per_t = max((times[128] - times[64]) / 64, 1e-12)
    fixed = max(times[64] - 64 * per_t, 0.0)
    t_full = fixed + per_t * n
    return {"value": 1.0 / t_full, "unit": "solves/s", "cores": th, "kind": "port",
            "sample": f"FP64 oracle (C/OpenMP, {th} threads), all {n} sources, 64 and 128 of {n} targets at "
                      f"d={d:.4f}; full solve extrapolated linearly in targets: {t_full:.1f} s"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle

    w = WORKLOAD
    x, f = make_inputs(w)
    n = w["n"]
    th = oracle.num_threads()
    d = oracle.choose_split(n, 32, w["L"])
    rng = np.random.default_rng(3)
    times = []
    for k in range(args.warmup + args.steps):
        idx = rng.choice(n, 32, replace=False)
        t0 = time.perf_counter()
        oracle.ewald_velocity(x[idx], x, f, w["L"], w["alpha"], w["eps"], d=d)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
    # the structure factor over all sources is the fixed part; targets scale linearly
    t_sample = float(np.mean(times))
    t0 = time.perf_counter()
    oracle.ewald_velocity(x[:1], x, f, w["L"], w["alpha"], w["eps"], d=d)
    t_one = time.perf_counter() - t0
    per_t = max((t_sample - t_one) / 31, 1e-12)
    t_full = t_one + per_t * (n - 1)
    v = 1.0 / t_full
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_full * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy)",
            "config": {"workload": w["name"], "n": n, "sample_targets_per_step": 32},
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": th, "kind": "port",
                             "sample": f"FP64 direct-Ewald oracle restating the reference's sums, {th} threads, all "
                                       f"{n} sources, 32 targets per step, extrapolated to {n} targets"},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="run the workload's plan twice (eager, then capture+replay) and exit: for ncu")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return

    import torch

    import periodicbrinkman_gb300 as pb
    from periodicbrinkman_gb300.api import Plan, make_params

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    w = WORKLOAD
    x, f = make_inputs(w)
    p = make_params(w["n"], w["L"], w["alpha"], w["eps"], tol=w["tol"], M=w["M"], P=w["P"], precision="mixed")
    plan = Plan(p)
    info = plan.info(0)
    xd = torch.from_numpy(x).cuda()
    fd = torch.from_numpy(f).cuda()
    Ud = torch.empty_like(xd)
    if args.profile:
        plan.execute(xd, fd, U=Ud)
        plan.execute(xd, fd, U=Ud)
        torch.cuda.synchronize()
        print(json.dumps({"profile": w["name"], "info": info, "kernels_per_solve": plan.kernel_count}))
        plan.close()
        return
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    stream = torch.cuda.current_stream()
    for _ in range(max(args.warmup, 3)):
        plan.execute(xd, fd, U=Ud, stream=stream)
    torch.cuda.synchronize()
    # stage breakdown (eager, events between stages)
    plan.set_timing(True)
    plan.execute(xd, fd, U=Ud, stream=stream)
    stages = plan.stage_ms()
    plan.set_timing(False)
    plan.execute(xd, fd, U=Ud, stream=stream)  # graph replay again
    nk = plan.kernel_count
    torch.cuda.synchronize()

    # accuracy of this very solve against the FP64 oracle on a target sample
    err = None
    if rank == 0:
        try:
            import oracle

            idx = np.random.default_rng(5).choice(w["n"], 96, replace=False)
            u_ref = oracle.ewald_velocity(x[idx], x, f, w["L"], w["alpha"], w["eps"])
            err = oracle.rel_errors(Ud.cpu().numpy()[idx], u_ref)
        except Exception as exc:  # pragma: no cover
            err = (None, str(exc))

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            flush.zero_()
            evs[k][0].record(stream)
            plan.execute(xd, fd, U=Ud, stream=stream)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in evs]
    t_dev = float(np.sum(step_ms)) / 1e3
    # e2e: public API with pinned host buffers, copies inside the timed region
    xh = torch.from_numpy(x).pin_memory()
    fh = torch.from_numpy(f).pin_memory()
    Uh = torch.empty_like(xh).pin_memory()
    xn, fn, Un = xh.numpy(), fh.numpy(), Uh.numpy()
    for _ in range(2):
        plan.execute(xn, fn, U=Un)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        plan.execute(xn, fn, U=Un)
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    if dist:
        tt = torch.tensor([t_dev, t_e2e], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_dev, t_e2e = float(tt[0]), float(tt[1])
        dist.barrier()
    value = world * args.steps / t_dev
    e2e = world * args.steps / t_e2e
    if rank != 0:
        return
    # roofline of the dominant stage
    names = ["sort", "real", "spread", "fft_green", "gather", "combine"]
    share = {names[i]: stages[i] / max(sum(stages), 1e-9) for i in range(6)}
    dom = max(share, key=share.get)
    pk = peaks()
    M3 = float(np.prod(info["M"]))
    n = w["n"]
    if dom == "real":
        # algorithmic work: 64 flop per pair inside rc (distance 8, kernel 32, tensor apply 12, Kahan 12)
        flops = 64.0 * info["pairs_est"]
        ach = flops / (stages[1] * 1e-3) / 1e12
        nsm = torch.cuda.get_device_properties(local).multi_processor_count
        fp32_peak = nsm * 128 * 2 * (pk.get("sm_max_mhz", 2070.0) * 1e6) / 1e12
        roof = {"bound": "fp32", "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak,
                "traffic": None, "kernel": "k_real_mixed",
                "note": "FP32 SIMT kernel; peak = SMs x 128 lanes x 2 flop x max SM clock (nominal, not measured)"}
    else:
        # k-space algorithmic bytes per solve: 4 B x 3 comps x M^3 x 6 + 36 N + 24 m
        by = 4.0 * 3 * M3 * 6 + 36.0 * n + 24.0 * n
        stage_idx = names.index(dom)
        ach = by / (stages[stage_idx] * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s", "frac": ach / pk["hbm_gbs"],
                "traffic": None, "kernel": dom}
    cb = None
    if not args.no_cpu_baseline:
        try:
            cb = cpu_baseline(w)
        except Exception as exc:  # pragma: no cover
            cb = {"value": None, "error": str(exc)}
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded numpy)",
        "config": {"workload": w["name"], "n": n, "L": w["L"], "alpha": w["alpha"], "eps": w["eps"], "grid": info["M"],
                   "P": info["P"], "d": info["d"], "rc": info["rc"], "npoly": info["npoly"],
                   "pairs_est": info["pairs_est"], "l2": "flushed (256 MB write) between steps",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": 2 * 3 * n * 8, "d2h_bytes_per_step": 3 * n * 8},
        "gpu_launches": nk * args.steps,
        "roofline": roof,
        "stage_ms": dict(zip(names, stages)),
        "max_rel_err": err[0] if err else None, "rms_rel_err": err[1] if err else None,
        "clocks": clk.summary(),
        "cpu_baseline": cb,
    }
    print(json.dumps(line))
    plan.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
