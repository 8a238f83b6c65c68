"""Throughput benchmark of the batched recursive Green sweep on one GB300.

Workload (the batched-uniform configuration): Dirichlet waveguide, W = 1,
kW/pi = 64.5 (wol = 32.25, M = N = 64 modes), L/W = 1, Nx = 2000 slices,
L/l_s = 10, eps = 0, U iid normal on a 2000 x 256 grid, seeds 1..4096, one
realization per seed.  A step is one persistent launch over the whole batch
(potential generation + sweep + Fisher-Lee + eigenvalues of t^H t); its
working set (4096 potentials, 16.8 GB) is far larger than L2, so no L2 flush
is needed between steps.

Metric: realizations/s (higher is better).  `value` is device-timed with the
seeds already in HBM; `e2e` goes through the C ABI with host buffers
(seeds copied in, eigenvalues and statuses copied out, inside the timing).

`--impl reference` times the reference's CPU algorithm (the oracle's C
restatement with LAPACK, OpenMP over seeds) on all host cores, on a bounded
sample of the same workload; gfortran is absent so the Fortran program itself
cannot be built here.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(boundtype="dirichlet", nxdiso=2000, nxfree=0, wol=32.25, exfac=1.0, aratio=1.0, dscat=10.0,
                dabso=0.0, napera=1.0, naperb=1.0, ny=256)
NSEED = 4096
METRIC = "realizations/s, N=256: batched vs per-realization FP64 GPU, t rel err≤1e-10"
UNIT = "realizations/s"


def flops_per_realization(M: int, nx: int) -> float:
    """FP64 flops of the reference's slice solve (src/waveguide.f90:426-440):
    16 M^3 per slice (complex inverse 8 M^3 + complex product 8 M^3) for
    slices 2..Nx plus 8 M^3 for the first inverse.  The pivoted kernel's
    Gauss-Jordan on [X | B Gs1] does the same 16 M^3 per slice."""
    return 16.0 * M ** 3 * (nx - 1) + 8.0 * M ** 3


def flops_symmetric(M: int, nx: int) -> float:
    """FP64 flops of the symmetric sweep: per slice, M pivot steps each update
    the M(M+1)/2 stored elements of W and the M x M elements of B Gs1 with one
    complex FMA (8 flops): 8 M (M(M+1)/2 + M^2) = 12 M^3 + 4 M^2."""
    return (12.0 * M ** 3 + 4.0 * M ** 2) * nx


KERNEL_NAMES = {"symmetric": "sweep_sym_kernel<64,256,2>", "pivoted": "sweep_kernel<64,256,2>",
                "blocked": "sweep_large_kernel"}


def config(batch: int) -> dict:
    nx = WORKLOAD["nxdiso"]
    return {"workload": f"batched-uniform: M=64 modes (kW/pi=64.5), Nx={nx}, ny=256, L/l_s=10, eps=0, "
                        f"{batch} realizations (seeds 1..{batch})",
            "modes": 64, "nx": nx, "ny": 256, "realizations_per_step": batch,
            "l2": "working set (potentials) 16.8 GB >> L2; no flush needed"}


class ClockSampler:
    """nvidia-smi clock and throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-i", "0", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.f.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_fp64_peak(torch) -> tuple[float, str]:
    """FP64 peak measured live: cuBLAS DGEMM 8192^3 (best of 5)."""
    a = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    b = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return 2.0 * 8192 ** 3 / best / 1e12, "cuBLAS DGEMM 8192^3 measured in this run (no FP64 entry in MEASURED_PEAKS.json)"


def cpu_baseline(sample: int, threads: int) -> dict:
    import oracle as O

    w = O.Waveguide(**WORKLOAD)
    seeds = list(range(1, sample + 1))
    t0 = time.perf_counter()
    w.tdistrib_batch(seeds, nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": sample / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{sample} realizations (seeds 1..{sample}) of the same workload, OpenMP over seeds, "
                      f"OpenBLAS 1 thread per worker; {dt:.1f} s"}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sample = args.ref_sample
    import oracle as O

    w = O.Waveguide(**WORKLOAD)
    seeds = list(range(1, sample + 1))
    for _ in range(args.warmup):
        w.tdistrib_batch(seeds[: max(threads, 1)], nthreads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        w.tdistrib_batch(seeds, nthreads=threads)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = sample * args.steps / tot
    out = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": config(sample),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"{sample} realizations per step (seeds 1..{sample}); the reference's "
                                      "algorithm restated in C with zgetrf/zgetri/zgesvd/zgemm from OpenBLAS"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=NSEED)
    ap.add_argument("--cpu-sample", type=int, default=48)
    ap.add_argument("--ref-sample", type=int, default=48)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--nx", type=int, default=WORKLOAD["nxdiso"],
                    help="slices (profiling runs only; the workload is Nx=2000)")
    args = ap.parse_args()
    WORKLOAD["nxdiso"] = args.nx
    if args.impl == "reference":
        run_reference(args)
        return

    import numpy as np
    import torch
    import torch.distributed as dist

    import recurgreen_gb300 as rg

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    torch.cuda.init()

    w = rg.Waveguide(**WORKLOAD)
    n = args.batch
    # Replicas: rank r takes seeds r*n+1 .. (r+1)*n (realizations are independent).
    seeds_h = np.arange(rank * n + 1, (rank + 1) * n + 1, dtype=np.int32)
    seeds_d = torch.from_numpy(seeds_h).cuda()
    out_d = torch.empty(n * w.neigv, dtype=torch.float64, device="cuda")
    st_d = torch.empty(n, dtype=torch.int32, device="cuda")
    L = rg.lib()
    stream = torch.cuda.Stream()  # the library enqueues on this stream; the events below bracket its work
    stream.wait_stream(torch.cuda.current_stream())

    def device_step():
        rc = L.rg_tdistrib_batch_device(w._h, seeds_d.data_ptr(), n, out_d.data_ptr(), st_d.data_ptr(),
                                        stream.cuda_stream)
        if rc:
            raise rg.RecurGreenError(rc, L.rg_last_error().decode())

    for _ in range(args.warmup):
        device_step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = ClockSampler()
    clk.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    sweep_ms = []
    fms = __import__("ctypes").c_float()
    e0.record(stream)
    for _ in range(args.steps):
        device_step()
        if L.rg_last_sweep_time(w._h, __import__("ctypes").byref(fms)) == 0:
            sweep_ms.append(fms.value)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = clk.stop()
    dt = e0.elapsed_time(e1) / 1e3
    if world > 1:
        t = torch.tensor([dt], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dt = float(t.item())
        dist.barrier()
    bad = int((st_d != 0).sum().item())

    # End to end through the C ABI with host buffers.
    tall = np.zeros(n * w.neigv)
    status = np.zeros(n, np.int32)
    ip = __import__("ctypes").POINTER(__import__("ctypes").c_int32)
    dp = __import__("ctypes").POINTER(__import__("ctypes").c_double)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rc = L.rg_tdistrib_batch(w._h, seeds_h.ctypes.data_as(ip), n, tall.ctypes.data_as(dp),
                                 status.ctypes.data_as(ip))
        if rc:
            raise rg.RecurGreenError(rc, L.rg_last_error().decode())
    e2e_dt = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_dt], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_dt = float(t.item())

    info = w.last_batch_info()
    fl = flops_per_realization(w.nmu, w.nx)
    if info["kernel"] == "symmetric":  # re-run items also cost a pivoted sweep
        fl_exec = flops_symmetric(w.nmu, w.nx) + fl * info["rerun"] / n
    else:
        fl_exec = fl
    value = world * n * args.steps / dt
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded potentials)",
           "config": config(n),
           "e2e": {"value": world * n * args.steps / e2e_dt, "unit": UNIT, "h2d_bytes_per_step": 4 * n,
                   "d2h_bytes_per_step": 8 * n * w.neigv + 4 * n},
           "gpu_launches": args.steps, "bad_status": bad}
    if rank == 0:
        peak, peak_src = measured_fp64_peak(torch)
        # the sweep kernel's own duration: CUDA events recorded around its
        # launch inside the library, on the same stream (rg_last_sweep_time)
        sweep_s = (sum(sweep_ms) / len(sweep_ms) / 1e3) if len(sweep_ms) == args.steps else dt / args.steps
        achieved = fl_exec * n / sweep_s / 1e12
        out["roofline"] = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                           "frac": achieved / peak, "traffic": None, "peak_source": peak_src,
                           "algorithmic_flops_per_launch": fl_exec * n,
                           "kernel": KERNEL_NAMES.get(info["kernel"], info["kernel"]), "launch": info,
                           "dense_equivalent_tflops": fl * n / sweep_s / 1e12,
                           "kernel_ms_per_launch": 1e3 * sweep_s,
                           "kernel_timing": "CUDA events around the sweep launch" if len(sweep_ms) == args.steps
                           else "whole step (potential + sweep)"}
        out["slice_solves_per_s"] = value * (w.nx)
        if clocks:
            out["clocks"] = clocks
        if not args.no_cpu:
            out["cpu_baseline"] = cpu_baseline(args.cpu_sample, os.cpu_count() or 1)
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
