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

`per_realization` times the drop-in path on a few of the same seeds: one
rg_compute_tdistrib call per seed (the reference's unit of work,
src/main.f90:156), so `batched_over_per_realization` is the batching gain.

`--impl reference` times the reference's CPU algorithm (the oracle's C
restatement with LAPACK, OpenMP over seeds) on all host cores, on a bounded
sample of the same workload; gfortran is absent so the Fortran program itself
cannot be built here.

`--workload` selects a secondary measurement instead of the default line:
  n256   M=256 modes (kW/pi=256.5, wol=128.25), Nx=2000, ny=1024: batched
         (--batch realizations, default 152) vs per-realization calls;
  uneven 2048 guides with N in {32,...,256}, Nx in [500,5000], L/l_s in
         [1,20], absorption on half (numpy default_rng(0)), ny=4N, through
         rg_tdistrib_multi, plus per-N histograms;
  diff   M=128, Nx=1000, ny=512, 256 realizations: Tr(t^H t), Tr((t^H t)^2)
         and both gradients w.r.t. U through the adjoint sweep (both
         cotangent chains in one reverse sweep);
  large  M=512, Nx=10^4 (or --nx, then also extrapolated to 10^4 by slice
         count), ny=2048, --batch realizations (default 152, one wave);
  tprofile  the default guide (M=64, Nx=2000, ny=256, L/l_s=10): transmission-
         eigenstate profiles for 0.9 <= T <= 1 (compute_tprofile) of --batch
         realizations (default 304) through rg_tprofile_batch, against
         per-realization rg_compute_tprofile calls and the oracle's
         solve_block_tridiag + zgesvd path on one host core (--wol changes
         the guide's width: M = floor(2 wol) modes on ny = 4M points).
"""
from __future__ import annotations

import argparse
import json
import math
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
                "blocked": "sweep_large_kernel", "blocked_symmetric": "sweep_large_sym_kernel"}


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


def _sync_time(torch, fn):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    return time.perf_counter() - t0, r


def _per_realization(L, w, seeds, np) -> tuple[float, float]:
    """Drop-in path: one rg_compute_tdistrib call per seed; (realizations/s, seconds)."""
    import ctypes

    tall = np.zeros(max(seeds) * w.neigv)
    dp = ctypes.POINTER(ctypes.c_double)
    t0 = time.perf_counter()
    for s in seeds:
        rc = L.rg_compute_tdistrib(w._h, int(s), tall.ctypes.data_as(dp), tall.size)
        if rc:
            raise RuntimeError(L.rg_last_error().decode())
    dt = time.perf_counter() - t0
    return len(seeds) / dt, dt


def run_workload(args) -> None:
    """Secondary measurements (one JSON line each); see the module docstring."""
    import ctypes

    import numpy as np
    import torch

    import recurgreen_gb300 as rg

    torch.cuda.init()
    L = rg.lib()
    out = {"workload": args.workload, "dtype": "f64", "data": "synthetic", "n_gpus": 1}
    peak, peak_src = measured_fp64_peak(torch)
    out["fp64_peak_tflops"] = peak
    out["fp64_peak_source"] = peak_src
    if args.workload in ("n256", "large"):
        if args.workload == "n256":
            kw = dict(WORKLOAD, wol=128.25, nxdiso=args.nx, ny=1024)
            n = args.batch if args.batch != NSEED else 152
        else:
            kw = dict(WORKLOAD, wol=256.25, nxdiso=args.nx if args.nx != 2000 else 10000, dscat=20.0, ny=2048)
            n = args.batch if args.batch != NSEED else 152
        w = rg.Waveguide(**kw)
        seeds = np.arange(1, n + 1, dtype=np.int32)
        # warm-up: the autotuner's choice depends on (modes, ny, batch size), not on
        # Nx, so a 16-slice copy of the guide tunes this batch outside the timing
        rg.Waveguide(**dict(kw, nxdiso=16)).tdistrib_batch(seeds)
        times = []
        for _ in range(max(args.steps, 1)):
            dt, _ = _sync_time(torch, lambda: w.tdistrib_batch(seeds))
            times.append(dt)
        ms = ctypes.c_float()
        L.rg_last_sweep_time(w._h, ctypes.byref(ms))
        info = w.last_batch_info()
        dt = min(times)
        fl = flops_per_realization(w.nmu, w.nx)
        out.update({"modes": w.nmu, "nx": w.nx, "ny": w.ny, "realizations": n, "launch": info,
                    "batched_realizations_per_s": n / dt, "batched_seconds": dt,
                    "sweep_kernel_seconds": ms.value / 1e3,
                    "dense_equivalent_tflops": fl * n / (ms.value / 1e3) / 1e12})
        out["frac_of_fp64_peak"] = out["dense_equivalent_tflops"] / peak
        if args.workload == "large" and w.nx != 10000:
            # the sweep time is linear in Nx; the per-realization epilogue is
            # below 1 % of a 10^4-slice guide at these sizes
            out["extrapolated_realizations_per_s_at_nx_10000"] = out["batched_realizations_per_s"] * w.nx / 10000
        if args.per_sample > 0:
            pr, pdt = _per_realization(L, w, list(range(1, args.per_sample + 1)), np)
            out["per_realization_per_s"] = pr
            out["per_realization_sample"] = f"{args.per_sample} seeds, one rg_compute_tdistrib call each, {pdt:.1f} s"
            out["batched_over_per_realization"] = out["batched_realizations_per_s"] / pr
    elif args.workload == "uneven":
        rng = np.random.default_rng(0)
        Ns = [32, 48, 64, 96, 128, 192, 256]
        n = args.batch if args.batch != NSEED else 2048
        guides, items, fl = {}, [], 0.0
        t0 = time.perf_counter()
        for k in range(n):
            N = int(rng.choice(Ns))
            nx = int(rng.integers(500, 5001))
            ds = float(rng.uniform(1, 20))
            wol = (N + 0.5) / 2
            dabso = 0.02 * math.pi * wol if rng.random() < 0.5 else 0.0
            g = rg.Waveguide("dirichlet", nxdiso=nx, nxfree=0, wol=wol, exfac=1.0, aratio=1.0, dscat=ds,
                             dabso=dabso, ny=4 * N)
            guides[k] = g
            items.append((g, k + 1))
            fl += flops_per_realization(g.nmu, nx)
        t_init = time.perf_counter() - t0
        dt, (res, st) = _sync_time(torch, lambda: rg.tdistrib_multi(items, return_status=True))
        # per-N histograms of T on the tdistrib task's Chebyshev edges (src/main.f90:233)
        from recurgreen_gb300.tdistrib import chebyshev_bins
        t1 = time.perf_counter()
        hist = {}
        for N in Ns:
            sel = [T for (g, _), T in zip(items, res) if g.nmu == N]
            if sel:
                h, miss = rg.histogram(np.concatenate(sel), chebyshev_bins(100))
                hist[N] = {"guides": len(sel), "samples": int(sum(x.size for x in sel)), "missing": miss}
        t_hist = time.perf_counter() - t1
        out.update({"guides": n, "guides_per_s": n / dt, "seconds": dt, "init_seconds": t_init,
                    "histogram_seconds": t_hist, "bad_status": int((st != 0).sum()),
                    "dense_equivalent_tflops": fl / dt / 1e12, "total_tflop": fl / 1e12, "per_N": hist})
        out["frac_of_fp64_peak"] = out["dense_equivalent_tflops"] / peak
    elif args.workload == "tprofile":
        import oracle as O

        kw = dict(WORKLOAD, nxdiso=args.nx)
        if args.wol:
            kw.update(wol=args.wol, ny=4 * int(2 * args.wol))  # M = floor(2 wol) modes on a 4M grid
        w = rg.Waveguide(**kw)
        n = args.batch if args.batch != NSEED else 304
        seeds = np.arange(1, n + 1, dtype=np.int32)
        w.tprofile_batch(seeds[:8], "tprofile", [0.9], [1.0])  # warm-up
        times = []
        for _ in range(max(args.steps, 1)):
            dt, (prof, nt, _) = _sync_time(torch, lambda: w.tprofile_batch(seeds, "tprofile", [0.9], [1.0]))
            times.append(dt)
        dt = min(times)
        M, nx = w.nmu, w.nx
        ksel = float(nt.mean())
        fl = flops_per_realization(M, nx) + 16.0 * M * M * ksel * nx  # forward sweep + back-substitution
        out.update({"modes": M, "nx": nx, "ny": w.ny, "realizations": n, "window": [0.9, 1.0],
                    "mean_eigenstates_in_window": ksel, "realizations_per_s": n / dt, "seconds": dt,
                    "dense_equivalent_tflops": fl * n / dt / 1e12,
                    "dump_bytes_per_realization": 2 * nx * M * M * 16})
        out["frac_of_fp64_peak"] = out["dense_equivalent_tflops"] / peak
        if args.per_sample > 0:
            t0 = time.perf_counter()
            for s in range(1, args.per_sample + 1):
                w.compute_tprofile(s, 0.9, 1.0)
            pdt = time.perf_counter() - t0
            out["per_realization_per_s"] = args.per_sample / pdt
            out["batched_over_per_realization"] = out["realizations_per_s"] / out["per_realization_per_s"]
        o = O.Waveguide(**kw)
        cs = 2
        t0 = time.perf_counter()
        for s in range(1, cs + 1):
            o.tprofile_upot(o.potential(s), 0.9, 1.0)
        cdt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": cs / cdt, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"{cs} realizations (seeds 1..{cs}): solve_block_tridiag with "
                                         f"zgetrf/zgetri/zgemm, zgesvd('N','A'), profile loop; {cdt:.1f} s"}
    elif args.workload == "diff":
        from recurgreen_gb300.adjoint import transmission_losses, transmission_losses_and_grads

        kw = dict(WORKLOAD, wol=64.25, nxdiso=args.nx if args.nx != 2000 else 1000, dscat=5.0, ny=512)
        w = rg.Waveguide(**kw)
        n = args.batch if args.batch != NSEED else 256
        gen = torch.Generator(device="cuda")
        gen.manual_seed(0)
        U = (torch.randn(n, w.nxdiso, w.ny, dtype=torch.float64, device="cuda", generator=gen) * w.stdu)
        U.requires_grad_(True)
        K = max(1, int(round(math.sqrt(w.nx))))

        def fwd():
            return transmission_losses(U, w, K)

        def step():  # both losses and both gradients, one reverse sweep for the two
            _, _, g1, g2 = transmission_losses_and_grads(U.detach(), w, K)
            return g1, g2

        fwd()
        t_fwd, _ = _sync_time(torch, fwd)
        t_all, (g1, g2) = _sync_time(torch, step)
        fl = flops_per_realization(w.nmu, w.nx)
        from recurgreen_gb300.adjoint import _method
        out.update({"adjoint_method": _method(w, U, "auto")})
        out.update({"modes": w.nmu, "nx": w.nx, "ny": w.ny, "realizations": n, "checkpoint_every": K,
                    "forward_seconds": t_fwd, "forward_and_two_gradients_seconds": t_all,
                    "realizations_per_s_with_gradients": n / t_all,
                    "forward_dense_equivalent_tflops": fl * n / t_fwd / 1e12,
                    "gradient_finite": bool(torch.isfinite(g1).all().item() and torch.isfinite(g2).all().item())})
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
    ap.add_argument("--per-sample", type=int, default=4,
                    help="seeds timed through the per-realization drop-in call (0: skip)")
    ap.add_argument("--wol", type=float, default=0.0,
                    help="tprofile workload: W/lambda instead of 32.25 (M = floor(2 wol) modes, ny = 4M)")
    ap.add_argument("--workload", default="uniform", choices=["uniform", "n256", "uneven", "diff", "large", "tprofile"])
    args = ap.parse_args()
    if args.impl == "reference":
        WORKLOAD["nxdiso"] = args.nx
        run_reference(args)
        return
    if args.workload != "uniform":
        run_workload(args)
        return
    WORKLOAD["nxdiso"] = args.nx

    import numpy as np
    import torch
    import torch.distributed as dist

    import recurgreen_gb300 as rg
    from recurgreen_gb300 import replicas

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)  # before the NCCL group, which binds to the current device
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
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
        dt = replicas.max_over_ranks(dt)
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
        e2e_dt = replicas.max_over_ranks(e2e_dt)
    per = None
    if args.per_sample > 0 and rank == 0:
        pr, pdt = _per_realization(L, w, list(seeds_h[: args.per_sample]), np)
        per = {"value": pr, "unit": UNIT,
               "sample": f"seeds {int(seeds_h[0])}..{int(seeds_h[min(args.per_sample, n) - 1])}, one "
                         f"rg_compute_tdistrib call each (host buffers, one CTA per call), {pdt:.1f} s"}

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
           # this library's kernels per step: the sweep, plus the pivoted re-run
           # that follows a symmetric sweep in the same graph (empty when nothing is flagged)
           "gpu_launches": args.steps * (2 if info["kernel"] in ("symmetric", "blocked_symmetric") else 1),
           "bad_status": bad}
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
        if per:
            out["per_realization"] = per
            out["batched_over_per_realization"] = value / per["value"]
        if clocks:
            out["clocks"] = clocks
        if not args.no_cpu:
            out["cpu_baseline"] = cpu_baseline(args.cpu_sample, os.cpu_count() or 1)
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
