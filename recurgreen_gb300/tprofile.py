"""The full Green-function tasks: wavefunction, tprofile and tprofile_group.

Host-side mirror of the reference's task drivers (src/main.f90:335-728):
the same namelist groups, the same averages over realizations, and CSV
files in the same layout (`%%` preamble, header line, values written like
Fortran's G0.16).  The per-realization work (the block tridiagonal solve,
the eigenvectors of t^H t and the profiles) runs in the GPU library
(rg_tprofile_batch, rg_compute_wavefunction); the seed loop is one batched
call instead of an OpenMP loop, or, with a process group, one batched call
per GPU on its seed range (replicas: no exchange until the gather).  The
TikZ plots the reference renders after saving (tikz/*.py through
execute_command_line) are not part of this build.
"""
from __future__ import annotations

import os
import time

import numpy as np

from .tdistrib import (_preamble, _waveguide_from, fortran_f, fortran_g0, generate_directory,
                       unique_filename)


def _profiles(w, nseed: int, kind: str, a, b, group=None):
    """Profiles of seeds 1..nseed: (prof (nseed, nprofile, nx), nt (nseed,
    nprofile), tavg (nseed,), seconds).  With a process group (one process per
    GPU) each rank sweeps a contiguous seed range and the results are
    gathered in seed order on every rank; the time is the slowest rank's."""
    a, b = np.atleast_1d(a), np.atleast_1d(b)
    if group is None:
        t0 = time.perf_counter()
        prof, nt, tavg = w.tprofile_batch(np.arange(1, nseed + 1, dtype=np.int32), kind, a, b)
        return prof, nt, tavg, time.perf_counter() - t0
    import torch.distributed as dist

    from . import replicas

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    seeds = replicas.seed_range(rank, world, nseed)
    t0 = time.perf_counter()
    if seeds.size:
        prof, nt, tavg = w.tprofile_batch(seeds, kind, a, b)
    else:
        prof, nt, tavg = np.zeros((0, a.size, w.nx)), np.zeros((0, a.size), np.int32), np.zeros(0)
    tsec = replicas.max_over_ranks(time.perf_counter() - t0, group)
    prof = replicas.gather_values(prof.reshape(-1), group).reshape(nseed, a.size, w.nx)
    nt = replicas.gather_values(nt.reshape(-1).astype(np.float64), group).reshape(nseed, a.size).astype(np.int32)
    tavg = replicas.gather_values(tavg, group)
    return prof, nt, tavg, tsec


def _writer(group) -> bool:
    if group is None:
        return True
    import torch.distributed as dist

    return dist.get_rank(group) == 0


def _header(w, prefix: str = "%%") -> list[str]:
    """print_timestamp and print_parameters (src/base_utils.f90:722-739,
    src/waveguide.f90:1003-1018)."""
    return _preamble(w, 0, 0, 1, 1.0, prefix)[:4]


def _write_rows(f, rows: np.ndarray) -> None:
    """save_real_matrix (src/base_utils.f90:639-657) with 'g0.16' and ', '."""
    for row in np.atleast_2d(rows):
        f.write(", ".join(fortran_g0(float(v)) for v in row) + "\n")


def task_wavefunction(settings: dict, outdir: str = "out") -> str:
    """task_wavefunction and save_wavefunction (src/main.f90:335-398)."""
    wf = settings["wavefunction"]
    iseed, ipos, imode = int(wf.get("iseed", 1)), int(wf.get("ipos", 1)), int(wf.get("imode", 1))
    w = _waveguide_from(settings["waveguide"])
    data = w.compute_wavefunction(iseed, ipos, imode)
    ddir = os.path.join(generate_directory(w, outdir), "wavefun")
    os.makedirs(ddir, exist_ok=True)
    path = unique_filename(os.path.join(ddir, "result_"), ".wavefun.csv")
    with open(path, "w") as f:
        for line in _header(w):
            f.write(line + "\n")
        f.write(f"%% Wavefunction parameters: iseed={iseed}, ipos={ipos}, imode={imode}\n")
        f.write("x, y, repsi, impsi, upot\n")
        _write_rows(f, data)
    return path


def task_tprofile(settings: dict, outdir: str = "out", group=None) -> dict:
    """task_tprofile and save_tprofile (src/main.f90:405-565): the profile of
    every realization (raw file) and their average over the realizations
    with at least one eigenvalue in [tmin, tmax] (avg file).  With a process
    group the seeds are sharded over the ranks and rank 0 writes the files."""
    tp = settings["tprofile"]
    tmin, tmax = float(tp.get("tmin", 0.0)), float(tp.get("tmax", 1.0))
    nseed = int(tp.get("nseed", 0))
    w = _waveguide_from(settings["waveguide"])
    if nseed <= 0:
        raise ValueError(f"Invalid number of disorder realizations (received {nseed}), aborting...")
    prof, nt, _, tsec = _profiles(w, nseed, "tprofile", tmin, tmax, group)
    data = prof[:, 0, :]
    nsample = int(np.count_nonzero(nt[:, 0]))
    avg = np.zeros(w.nx)
    for k in range(nseed):  # seed order, as src/main.f90:476-483
        if nt[k, 0] != 0:
            avg = avg + data[k]
    with np.errstate(invalid="ignore", divide="ignore"):
        avg = avg / nsample
    res = {"raw": None, "avg": None, "nsample": nsample, "time": tsec, "profiles": data, "nt": nt[:, 0]}
    if not _writer(group):
        return res
    ddir = os.path.join(generate_directory(w, outdir), "tprofile")
    os.makedirs(ddir, exist_ok=True)
    params = (f"%% Transmission profile parameters: Found nsample={nsample} / nseed={nseed}, nx={w.nx}, "
              f"tmin={fortran_g0(tmin, 6)}, tmax={fortran_g0(tmax, 6)}, time={fortran_f(tsec, 3)} s.")
    raw = unique_filename(os.path.join(ddir, "result_"), ".raw.csv")
    with open(raw, "w") as f:
        for line in _header(w):
            f.write(line + "\n")
        f.write(params + "\n")
        f.write("%% Here follows, on each line, the function |psi_T(x)|^2 for a given realization of the disorder.\n")
        _write_rows(f, data)
    avgp = unique_filename(os.path.join(ddir, "result_"), ".avg.csv")
    x = w.get_xmesh()
    with open(avgp, "w") as f:
        for line in _header(w):
            f.write(line + "\n")
        f.write(params + "\n")
        f.write("x, tprofile\n")
        for ix in range(w.nx):
            f.write(f"{fortran_g0(float(x[ix]))}, {fortran_g0(float(avg[ix]))}\n")
    res.update(raw=raw, avg=avgp)
    return res


def task_tprofile_group(settings: dict, outdir: str = "out", group=None) -> dict:
    """task_tprofile_group and save_tprofile_group (src/main.f90:572-728):
    four profiles per realization, their averages, and the mean transmission
    Tavg with its uncertainty.  With a process group the seeds are sharded
    over the ranks and rank 0 writes the file."""
    tg = settings["tprofile_group"]
    tm = np.atleast_1d(np.asarray(tg.get("tm", []), np.float64))
    dt = np.atleast_1d(np.asarray(tg.get("dt", []), np.float64))
    nseed = int(tg.get("nseed", 0))
    nprofile = 4
    if tm.size != nprofile or dt.size != nprofile:
        raise ValueError(f"tm and dt need {nprofile} values each, aborting...")
    w = _waveguide_from(settings["waveguide"])
    if nseed <= 0:
        raise ValueError(f"Invalid number of disorder realizations (received {nseed}), aborting...")
    prof, nt, tavgdata, tsec = _profiles(w, nseed, "group", tm, dt, group)
    avg = np.zeros((w.nx, nprofile))
    nsample = np.zeros(nprofile, np.int64)
    for ip in range(nprofile):  # src/main.f90:633-651
        for k in range(nseed):
            if nt[k, ip] != 0:
                avg[:, ip] = avg[:, ip] + prof[k, ip]
                nsample[ip] += 1
        if nsample[ip] != 0:
            avg[:, ip] = avg[:, ip] / nsample[ip]
    tavg = np.sum(tavgdata) / nseed
    uctavg = np.sqrt(np.sum((tavgdata - tavg) ** 2)) / nseed
    res = {"path": None, "nsample": nsample, "tavg": tavg, "uctavg": uctavg, "time": tsec}
    if not _writer(group):
        return res
    ddir = os.path.join(generate_directory(w, outdir), "tprofile_group")
    os.makedirs(ddir, exist_ok=True)
    path = unique_filename(os.path.join(ddir, "result_"), ".csv")
    x = w.get_xmesh()
    g6 = lambda v: fortran_g0(float(v), 6)  # noqa: E731
    with open(path, "w") as f:
        for line in _header(w):
            f.write(line + "\n")
        f.write(f"%% Transmission profile parameters: nx={w.nx}, tm=[{', '.join(g6(v) for v in tm)}], "
                f"dt=[{', '.join(g6(v) for v in dt)}].\n")
        f.write(f"%% Results: Found nsample=[{', '.join(str(int(v)) for v in nsample)}] over nseed={nseed}, "
                f"tavg={g6(tavg)}+-{g6(uctavg)}, time={fortran_f(tsec, 3)} s.\n")
        f.write("x" + "".join(f", tprofile{fortran_f(float(v), 4)}" for v in tm) + "\n")
        for ix in range(w.nx):
            f.write(", ".join(fortran_g0(float(v)) for v in [x[ix], *avg[ix]]) + "\n")
    res["path"] = path
    return res
