"""Throughput benchmark of the batched recursive Green sweep on one GB300.

Default workload (the metric's configuration, `--workload n256`): Dirichlet
waveguide, W = 1, kW/pi = 256.5 (wol = 128.25, M = N = 256 modes), L/W = 1,
Nx = 2000 slices, ny = 1024 transverse points, L/l_s = 10, eps = 0, U iid
normal drawn from each realization's seed.  A step is one batched call over
--batch realizations (seeds 1..B): potential generation, the sweep,
Fisher-Lee and the eigenvalues of t^H t, all inside one persistent launch
(plus the pivoted re-run of flagged items in the same CUDA graph).

Metric: realizations/s (higher is better).  The timed loop makes K calls of
rg_tdistrib_batch, the C-ABI entry point a user calls, with host buffers
(seeds in, eigenvalues and statuses out):
  * `value`  = realizations / the summed device time of the K batches (CUDA
               events recorded by the library around each batch's graph on
               its launching stream; inputs are already in HBM there);
  * `e2e`    = realizations / the host wall time of the same K calls
               (host-to-device and device-to-host copies included).
`per_realization` times the drop-in path (rg_compute_tdistrib, one call per
seed, the reference's unit of work, src/main.f90:156) on the same guide, so
`batched_over_per_realization` is the batching gain the metric names.

`--impl reference` times the reference's CPU algorithm (the oracle's C
restatement with LAPACK, OpenMP over seeds, one seed per host core) on a
bounded sample of the same workload; gfortran is absent, so the Fortran
program itself cannot be built.

Secondary workloads (`--workload`, one JSON line each, clocks sampled):
  uniform  the batched-uniform configuration through the same timed loop:
           M=64 (kW/pi=64.5), Nx=2000, ny=256, seeds 1..4096 per step;
  uneven   2048 guides with N in {32,...,256}, Nx in [500,5000], L/l_s in
           [1,20], absorption on half (numpy default_rng(0)), ny=4N, through
           rg_tdistrib_multi, plus per-N histograms;
  diff     M=128, Nx=1000, ny=512, 256 realizations: Tr(t^H t), Tr((t^H t)^2)
           and both gradients w.r.t. U through the adjoint sweep;
  large    M=512, Nx=10^4 (or --nx), ny=2048, L/l_s=20, --batch
           realizations (default 152, one wave);
  tprofile the batched-uniform guide (M=64, Nx=2000, ny=256): transmission-
           eigenstate profiles for 0.9 <= T <= 1 of --batch realizations;
  probe    pipe rates (rg_probe_rate: FP64 FMA, FP64 mma.sync, FP16 mma.sync,
           FP32 FMA) beside cuBLAS DGEMM 8192^3.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "realizations/s, N=256: batched vs per-realization FP64 GPU, t rel err≤1e-10"
UNIT = "realizations/s"

BASE = dict(boundtype="dirichlet", nxdiso=2000, nxfree=0, wol=128.25, exfac=1.0, aratio=1.0, dscat=10.0,
            dabso=0.0, napera=1.0, naperb=1.0, ny=1024)

# The timed workloads: waveguide parameters, realizations per step, and the
# slices of the reference arm's per-step sample.  N=256: 304 realizations per
# step, one per CTA at two CTAs per SM of the GB300's 152 (one wave), where
# the autotuner's fastest cluster size is one CTA per realization.
SPECS = {
    "n256": dict(kw=dict(BASE), batch=304, ref_nx=200,
                 desc="batched N=256: Dirichlet, kW/pi=256.5 (wol=128.25, M=N=256 modes), L/W=1, Nx=2000, "
                      "ny=1024, L/l_s=10, eps=0"),
    "uniform": dict(kw=dict(BASE, wol=32.25, ny=256), batch=4096, ref_nx=2000,
                    desc="batched-uniform: M=64 modes (kW/pi=64.5), Nx=2000, ny=256, L/l_s=10, eps=0"),
}


def uneven_items(n: int = 2048) -> list[tuple[dict, int]]:
    """The batched-uneven workload: guide k (seed k + 1) has N drawn from
    {32, 48, 64, 96, 128, 192, 256} (kW/pi = N + 0.5, M = N, ny = 4N),
    Nx from [500, 5000], L/l_s from [1, 20], and absorption
    eps = 0.01 k^2 (dabso = 0.02 pi W/lambda) with probability 1/2, all from
    numpy default_rng(0)."""
    import numpy as np

    rng = np.random.default_rng(0)
    Ns = [32, 48, 64, 96, 128, 192, 256]
    out = []
    for k in range(n):
        N = int(rng.choice(Ns))
        nx = int(rng.integers(500, 5001))
        ds = float(rng.uniform(1, 20))
        wol = (N + 0.5) / 2
        dabso = 0.02 * math.pi * wol if rng.random() < 0.5 else 0.0
        out.append((dict(boundtype="dirichlet", nxdiso=nx, nxfree=0, wol=wol, exfac=1.0, aratio=1.0, dscat=ds,
                         dabso=dabso, ny=4 * N), k + 1))
    return out


def flops_per_realization(M: int, nx: int) -> float:
    """Algorithmic FP64 flops of the reference's sweep (src/waveguide.f90:426-440):
    16 M^3 per slice (complex inverse 8 M^3 + complex product 8 M^3) for
    slices 2..Nx plus 8 M^3 for the first inverse.  The pivoted kernels'
    Gauss-Jordan on [X | B Gs1] does the same 16 M^3 per slice."""
    return 16.0 * M ** 3 * (nx - 1) + 8.0 * M ** 3


def executed_flops(M: int, nx: int, kernel: str) -> tuple[float, float]:
    """(FP64 flops, FP16 tensor flops) the sweep executes for one realization:
      * shared-memory symmetric kernel (M <= 64): 12 M^3 + 4 M^2 FP64 per slice;
      * blocked symmetric kernel with the tensor-core propagator product
        (64 < M <= 512): the inverse in FP64 -- 4 M^3 for one Gauss-Jordan
        sweep; each level of the 2 x 2 block form (even sizes >= 128, at most
        two levels) replaces a size-m inverse by two of size m/2 and four
        (m/2)^3 products -- and 26 digit pairs x 4 real products x 2 k^3 FP16
        flops per k x k product: 208 M^3 for the propagator product plus
        4 x 208 (m/2)^3 per block split;
      * otherwise the pivoted reference count 16 M^3 in FP64.
    RG_TENSOR_R=0 / RG_SPLIT_INVERSE=0 or 1 select the other variants."""
    tensor = os.environ.get("RG_TENSOR_R", "1") != "0" and 64 < M <= 512
    want = {"0": 0, "1": 1}.get(os.environ.get("RG_SPLIT_INVERSE", "2"), 2)
    if kernel == "symmetric":
        return flops_symmetric(M, nx), 0.0
    if kernel != "blocked_symmetric":
        return flops_per_realization(M, nx), 0.0
    if not tensor:
        return flops_symmetric(M, nx), 0.0
    fp16 = 208.0 * M ** 3
    m, blocks = M, 1
    while want > 0 and m >= 128 and m % 2 == 0:
        want -= 1
        fp16 += blocks * 4 * 208.0 * (m // 2) ** 3
        m, blocks = m // 2, blocks * 2
    fp64 = blocks * 4.0 * m ** 3
    return fp64 * nx, fp16 * nx


def flops_symmetric(M: int, nx: int) -> float:
    """Executed FP64 flops of the symmetric sweeps: per slice, M pivot steps each
    update the M(M+1)/2 stored elements of W and the M x M elements of B Gs1
    with one complex FMA (8 flops): 8 M (M(M+1)/2 + M^2) = 12 M^3 + 4 M^2."""
    return (12.0 * M ** 3 + 4.0 * M ** 2) * nx


KERNEL_NAMES = {"symmetric": "sweep_sym_kernel<64,256,2>", "pivoted": "sweep_kernel<64,256,2>",
                "blocked": "sweep_large_kernel", "blocked_symmetric": "sweep_large_sym_kernel"}


def config(spec: dict, batch: int, M: int) -> dict:
    kw = spec["kw"]
    ws_mb = 3 * M * M * 16 / 2 ** 20
    return {"workload": f"{spec['desc']}, {batch} realizations per step (seeds 1..{batch})",
            "modes": M, "nx": kw["nxdiso"], "ny": kw["ny"], "realizations_per_step": batch,
            "l2": f"inputs larger than L2: each step draws {batch} potentials of {kw['nxdiso']}x{kw['ny']} "
                  f"doubles in-kernel ({batch * kw['nxdiso'] * kw['ny'] * 8 / 1e9:.1f} GB if materialised) and "
                  f"sweeps {ws_mb:.2f} MB of slice matrices per realization; no flush needed"}


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
        return self

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


def _ref_sample(spec: dict, threads: int, ref_nx: int):
    """The reference arm's bounded sample: one seed per host core (seeds
    1..threads), each sweeping a guide of ref_nx slices with every other
    parameter of the workload (the per-slice work -- projection, inverse,
    product -- is the workload's), so a sample is worth threads * ref_nx / Nx
    realizations of the workload."""
    import oracle as O

    nx = spec["kw"]["nxdiso"]
    w = O.Waveguide(**dict(spec["kw"], nxdiso=min(ref_nx, nx)))
    seeds = list(range(1, threads + 1))
    worth = threads * min(ref_nx, nx) / nx
    desc = (f"{threads} seeds (1..{threads}, one per core) each sweeping the first {min(ref_nx, nx)} of the "
            f"{nx} slices with the workload's modes and grid, counted as {worth:g} realizations; the "
            "reference's algorithm restated in C with zgetrf/zgetri/zgesvd/zgemm from OpenBLAS "
            "(1 BLAS thread per worker); the per-sample zgesvd is included")
    return w, seeds, worth, desc


def cpu_baseline(spec: dict, threads: int, ref_nx: int) -> dict:
    w, seeds, worth, desc = _ref_sample(spec, threads, ref_nx)
    t0 = time.perf_counter()
    w.tdistrib_batch(seeds, nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": worth / dt, "unit": UNIT, "cores": threads, "kind": "port", "sample": f"{desc}; {dt:.1f} s"}


def run_reference(args, spec: dict) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    ref_nx = args.ref_nx or spec["ref_nx"]
    w, seeds, worth, desc = _ref_sample(spec, threads, ref_nx)
    for _ in range(args.warmup):
        w.tdistrib_batch(seeds, nthreads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        w.tdistrib_batch(seeds, nthreads=threads)
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    value = worth * args.steps / tot
    M = int(2 * spec["kw"]["wol"])
    batch = args.batch or spec["batch"]
    out = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded potentials)", "config": config(spec, batch, M),
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": "each step: " + desc},
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
    tall = np.zeros(max(seeds) * w.neigv)
    dp = ctypes.POINTER(ctypes.c_double)
    t0 = time.perf_counter()
    for s in seeds:
        rc = L.rg_compute_tdistrib(w._h, int(s), tall.ctypes.data_as(dp), tall.size)
        if rc:
            raise RuntimeError(L.rg_last_error().decode())
    dt = time.perf_counter() - t0
    return len(seeds) / dt, dt


def run_main(args, spec: dict) -> None:
    """The timed batched path: K host-buffer rg_tdistrib_batch calls."""
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

    kw = dict(spec["kw"])
    if args.nx:
        kw["nxdiso"] = args.nx
    spec = dict(spec, kw=kw)
    w = rg.Waveguide(**kw)
    n = args.batch or spec["batch"]
    L = rg.lib()
    # Replicas: rank r takes seeds r*n+1 .. (r+1)*n (realizations are independent).
    seeds_h = np.arange(rank * n + 1, (rank + 1) * n + 1, dtype=np.int32)
    tall = np.zeros(n * w.neigv)
    status = np.zeros(n, np.int32)
    ip = ctypes.POINTER(ctypes.c_int32)
    dp = ctypes.POINTER(ctypes.c_double)
    fms = ctypes.c_float()

    def step() -> float:
        rc = L.rg_tdistrib_batch(w._h, seeds_h.ctypes.data_as(ip), n, tall.ctypes.data_as(dp),
                                 status.ctypes.data_as(ip))
        if rc:
            raise rg.RecurGreenError(rc, L.rg_last_error().decode())
        rc = L.rg_last_sweep_time(w._h, ctypes.byref(fms))
        if rc:
            raise rg.RecurGreenError(rc, L.rg_last_error().decode())
        return fms.value / 1e3

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = ClockSampler().start()
    torch.cuda.synchronize()
    sweep_s = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sweep_s.append(step())
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    dev = sum(sweep_s)
    if world > 1:
        dev = replicas.max_over_ranks(dev)
        wall = replicas.max_over_ranks(wall)
        dist.barrier()
    bad = int((status != 0).sum())
    info = w.last_batch_info()
    M = w.nmu
    fl = flops_per_realization(M, w.nx)
    fl64, fl16 = executed_flops(M, w.nx, info["kernel"])
    if info["kernel"] in ("symmetric", "blocked_symmetric"):  # re-run items also cost a pivoted sweep
        fl64 += fl * info["rerun"] / n
    value = world * n * args.steps / dev
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * dev / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded potentials)",
           "config": config(spec, n, M),
           "timing": "value: summed CUDA-event device time of the K batches (events recorded around each "
                     "batch's graph on its launching stream); e2e: host wall time of the same K "
                     "rg_tdistrib_batch calls with host buffers",
           "e2e": {"value": world * n * args.steps / wall, "unit": UNIT, "h2d_bytes_per_step": 4 * n,
                   "d2h_bytes_per_step": 8 * n * w.neigv + 4 * n},
           # this library's kernels per step: the sweep, plus the pivoted re-run
           # that follows a symmetric sweep in the same graph (empty when nothing is flagged)
           "gpu_launches": args.steps * (2 if info["kernel"] in ("symmetric", "blocked_symmetric") else 1),
           "bad_status": bad}
    if rank == 0:
        peak, peak_src = measured_fp64_peak(torch)
        mma = ctypes.c_double()
        mma_peak = mma.value if L.rg_probe_rate(3, 100000, ctypes.byref(mma)) == 0 else float("nan")
        per_launch = sum(sweep_s) / len(sweep_s)  # this rank's batches
        achieved = fl * n / per_launch / 1e12
        t64, t16 = fl64 * n / per_launch / 1e12, fl16 * n / per_launch / 1e12
        out["roofline"] = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                           "frac": achieved / peak, "traffic": None, "peak_source": peak_src,
                           "algorithmic_flops_per_launch": fl * n,
                           "algorithmic_count": "16 M^3 per slice-solve (slices 2..Nx) + 8 M^3, per realization: "
                                                "the reference's FP64 work, the numerator of achieved",
                           "executed": {
                               "fp64_flops_per_launch": fl64 * n, "fp64_tflops": t64, "fp64_frac_of_dgemm": t64 / peak,
                               "fp16_tensor_flops_per_launch": fl16 * n, "fp16_tensor_tflops": t16,
                               "fp16_mma_sync_peak_tflops": mma_peak,
                               "fp16_tensor_frac_of_mma_sync": t16 / mma_peak if mma_peak == mma_peak else None,
                               "note": "the FP64 inverse runs on the FP64 pipe; the propagator product (and, in "
                                       "the 2x2 block form, the block products) on the FP16 tensor cores with "
                                       "FP64 accuracy (exact digit products), so achieved above the FP64 peak "
                                       "is work moved off the FP64 pipe"},
                           "kernel": KERNEL_NAMES.get(info["kernel"], info["kernel"]), "launch": info,
                           "kernel_ms_per_launch": 1e3 * per_launch,
                           "kernel_timing": "CUDA events around each batch's graph (sweep + pivoted re-run)"}
        out["slice_solves_per_s"] = value * w.nx
        if args.per_sample > 0:
            pr, pdt = _per_realization(L, w, list(seeds_h[: args.per_sample]), np)
            out["per_realization"] = {
                "value": pr, "unit": UNIT,
                "sample": f"seeds {int(seeds_h[0])}..{int(seeds_h[min(args.per_sample, n) - 1])}, one "
                          f"rg_compute_tdistrib call each (host buffers), {pdt:.1f} s"}
            out["batched_over_per_realization"] = value / pr
        if clocks:
            out["clocks"] = clocks
        if not args.no_cpu:
            out["cpu_baseline"] = cpu_baseline(spec, os.cpu_count() or 1, args.ref_nx or spec["ref_nx"])
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


def run_workload(args) -> None:
    """Secondary measurements (one JSON line each); see the module docstring."""
    import numpy as np
    import torch

    import recurgreen_gb300 as rg

    torch.cuda.init()
    L = rg.lib()
    out = {"workload": args.workload, "dtype": "f64", "data": "synthetic", "n_gpus": 1}
    if args.no_peak:  # profiling runs: no cuBLAS DGEMM in the launch list
        peak, peak_src = float("nan"), "not measured (--no-peak)"
    else:
        peak, peak_src = measured_fp64_peak(torch)
    out["fp64_peak_tflops"] = peak
    out["fp64_peak_source"] = peak_src
    clk = ClockSampler()
    if args.workload == "probe":
        # the denominators of the roofline: pipe rates from register-only probes
        names = {0: ("fp64_fma", 100000), 1: ("fp64_mma_m8n8k4", 20000), 2: ("fp64_mma_m16n8k16", 3000),
                 3: ("fp16_mma_m16n8k16_f32acc", 100000), 4: ("fp32_fma", 1000000)}
        clk.start()
        rates = {}
        for kind, (name, iters) in names.items():
            v = ctypes.c_double()
            rc = L.rg_probe_rate(kind, iters, ctypes.byref(v))
            if rc:
                raise rg.RecurGreenError(rc, L.rg_last_error().decode())
            rates[name] = v.value
        # the tensor-core complex product (rg_zgemm_batched) at the sweep's
        # sizes: 152 independent M x M products per call, FP16 flops counted as
        # 26 digit pairs x 4 real products x 2 M^3
        from recurgreen_gb300.adjoint import _ZGemm
        zrates = {}
        for M in (128, 256, 512):
            nb = 152
            A = torch.randn(nb, M, M, dtype=torch.complex128, device="cuda")
            B = torch.randn(nb, M, M, dtype=torch.complex128, device="cuda")
            C = torch.empty_like(A)
            zg = _ZGemm(M, nb, A.device)
            zg(nb, A, B, C)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(3):
                zg(nb, A, B, C)
            e1.record()
            e1.synchronize()
            sec = e0.elapsed_time(e1) / 3e3
            zrates[f"M{M}"] = {"ms_per_call": 1e3 * sec, "fp16_tflops": 26 * 4 * 2 * M ** 3 * nb / sec / 1e12,
                               "fp64_equivalent_tflops": 8 * M ** 3 * nb / sec / 1e12}
            del A, B, C, zg
        out["clocks"] = clk.stop()
        out["tflops"] = rates
        out["tflops"]["cublas_dgemm_8192"] = peak
        out["zgemm_batched"] = zrates
        out.pop("fp64_peak_tflops")
    elif args.workload == "large":
        kw = dict(BASE, wol=256.25, nxdiso=args.nx or 10000, dscat=20.0, ny=2048)
        n = args.batch or 152
        w = rg.Waveguide(**kw)
        seeds = np.arange(1, n + 1, dtype=np.int32)
        # warm-up: the autotuner's choice depends on (modes, ny, batch size), not on
        # Nx, so a 16-slice copy of the guide tunes this batch outside the timing
        rg.Waveguide(**dict(kw, nxdiso=16)).tdistrib_batch(seeds)
        clk.start()
        dt, T = _sync_time(torch, lambda: w.tdistrib_batch(seeds))
        out["clocks"] = clk.stop()
        ms = ctypes.c_float()
        L.rg_last_sweep_time(w._h, ctypes.byref(ms))
        info = w.last_batch_info()
        fl = flops_per_realization(w.nmu, w.nx)
        out.update({"modes": w.nmu, "nx": w.nx, "ny": w.ny, "realizations": n, "launch": info,
                    "batched_realizations_per_s": n / dt, "batched_seconds": dt,
                    "sweep_kernel_seconds": ms.value / 1e3,
                    "dense_equivalent_tflops": fl * n / (ms.value / 1e3) / 1e12})
        out["frac_of_fp64_peak"] = out["dense_equivalent_tflops"] / peak
        T = T.reshape(n, w.neigv)
        out["smallest_T"] = float(T.min())
        fix = os.path.join(ROOT, "tests", "golden", "oracle_c5.npz")
        if w.nx == 10000 and w.ny == 2048 and os.path.exists(fix):
            # the oracle's eigenvalues of seeds 1..16 (tests/golden/make_large_fixtures.py c5)
            f = np.load(fix)
            k = [int(s) - 1 for s in f["seeds"] if s <= n]
            if k:
                To, Tg = f["T"][: len(k)], T[k]
                big = To >= 1e-12
                out["parity_vs_oracle"] = {
                    "seeds": [int(s) for s in f["seeds"][: len(k)]],
                    "max_abs_T_err": float(np.max(np.abs(Tg - To))),
                    "max_rel_T_err_for_T_ge_1e-12": float(np.max(np.abs(Tg - To)[big] / To[big])),
                    "eigenvalues_with_T_ge_1e-12": int(big.sum()),
                    "smallest_oracle_T": float(To.min())}
        if args.per_sample > 0:
            pr, pdt = _per_realization(L, w, list(range(1, args.per_sample + 1)), np)
            out["per_realization_per_s"] = pr
            out["per_realization_sample"] = f"{args.per_sample} seeds, one rg_compute_tdistrib call each, {pdt:.1f} s"
            out["batched_over_per_realization"] = out["batched_realizations_per_s"] / pr
    elif args.workload == "uneven":
        Ns = [32, 48, 64, 96, 128, 192, 256]
        n = args.batch or 2048
        guides, items, fl = {}, [], 0.0
        t0 = time.perf_counter()
        for k, (kw, seed) in enumerate(uneven_items(n)):
            g = rg.Waveguide(**kw)
            guides[k] = g
            items.append((g, seed))
            fl += flops_per_realization(g.nmu, kw["nxdiso"])
        t_init = time.perf_counter() - t0
        clk.start()
        dt, (res, st) = _sync_time(torch, lambda: rg.tdistrib_multi(items, return_status=True))
        out["clocks"] = clk.stop()
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

        kw = dict(SPECS["uniform"]["kw"], nxdiso=args.nx or 2000)
        if args.wol:
            kw.update(wol=args.wol, ny=4 * int(2 * args.wol))  # M = floor(2 wol) modes on a 4M grid
        w = rg.Waveguide(**kw)
        n = args.batch or 304
        seeds = np.arange(1, n + 1, dtype=np.int32)
        w.tprofile_batch(seeds[:8], "tprofile", [0.9], [1.0])  # warm-up
        clk.start()
        dt, (prof, nt, _) = _sync_time(torch, lambda: w.tprofile_batch(seeds, "tprofile", [0.9], [1.0]))
        out["clocks"] = clk.stop()
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

        kw = dict(BASE, wol=64.25, nxdiso=args.nx or 1000, dscat=5.0, ny=512)
        w = rg.Waveguide(**kw)
        n = args.batch or 256
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
        clk.start()
        t_fwd, _ = _sync_time(torch, fwd)
        t_all, (g1, g2) = _sync_time(torch, step)
        out["clocks"] = clk.stop()
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
    ap.add_argument("--batch", type=int, default=0, help="realizations per step (0: the workload's default)")
    ap.add_argument("--ref-nx", type=int, default=0,
                    help="slices of each seed of the reference arm's sample (0: the workload's default)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-peak", action="store_true",
                    help="secondary workloads: skip the cuBLAS DGEMM peak measurement (profiling runs)")
    ap.add_argument("--nx", type=int, default=0, help="slices (0: the workload's own; other values for profiling)")
    ap.add_argument("--per-sample", type=int, default=1,
                    help="seeds timed through the per-realization drop-in call (0: skip)")
    ap.add_argument("--wol", type=float, default=0.0,
                    help="tprofile workload: W/lambda instead of 32.25 (M = floor(2 wol) modes, ny = 4M)")
    ap.add_argument("--workload", default="n256",
                    choices=["n256", "uniform", "uneven", "diff", "large", "tprofile", "probe"])
    args = ap.parse_args()
    if args.workload in SPECS:
        spec = SPECS[args.workload]
        if args.impl == "reference":
            run_reference(args, spec)
        else:
            run_main(args, spec)
        return
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm is defined for the timed "
                                                              "workloads (n256, uniform) only"}))
        return
    run_workload(args)


if __name__ == "__main__":
    main()
