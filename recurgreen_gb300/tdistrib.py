"""The tdistrib task and plothisto re-binning on top of the GPU library.

Host-side mirror of the reference's task driver for the transmission-
eigenvalue distribution (src/main.f90:73-328) and of the plothisto program
(src/plot_histogram.f90:7-143): the same namelist input, the same Chebyshev
or linear bins, the same histogram / normalisation / bin-centre steps
(src/base_utils.f90:491-570), and CSV output in the same layout (a `%%`
preamble, a `tm, rho` header, values written like Fortran's G0.16).  The
eigenvalues come from one batched GPU launch (rg_tdistrib_batch) and the
histogram counts from the GPU (rg_histogram).

    python -m recurgreen_gb300.tdistrib settings.nml [--outdir DIR]     (any task of &settings)
    python -m recurgreen_gb300.tdistrib --replot plothisto_settings.nml result_1.eigvals.csv
"""
from __future__ import annotations

import argparse
import datetime
import math
import os
import re
import time

import numpy as np

from . import Waveguide, histogram

PROGRAM = "RecurGreen-GB300 (recursive Green sweep on GB300)"


# ---------------------------------------------------------------------------
# Namelists (the subset the reference's settings files use)
# ---------------------------------------------------------------------------
def _value(tok: str):
    t = tok.strip()
    if not t:
        return None
    if t[0] in "'\"" and t[-1] == t[0]:
        return t[1:-1]
    low = t.lower()
    if low in (".true.", ".t.", "t", "true"):
        return True
    if low in (".false.", ".f.", "f", "false"):
        return False
    try:
        if re.fullmatch(r"[-+]?\d+", t):
            return int(t)
        return float(t.replace("d", "e").replace("D", "e"))
    except ValueError:
        return t


def read_namelists(text: str) -> dict:
    """Groups `&name key = value, ... /` of a Fortran namelist file.  `!`
    starts a comment outside quotes; comma-separated values become lists.
    The first group of a given name wins (Fortran reads the first match)."""
    groups: dict = {}
    cur = None
    body: list[str] = []
    for raw in text.splitlines():
        line, q = "", None
        for ch in raw:
            if q:
                line += ch
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
                line += ch
            elif ch == "!":
                break
            else:
                line += ch
        s = line.strip()
        if not s:
            continue
        if cur is None:
            m = re.match(r"&(\w+)(.*)", s)
            if not m:
                continue
            cur, rest = m.group(1).lower(), m.group(2)
            body = [rest]
            s = ""
        else:
            body.append(s)
        joined = " ".join(body)
        if "/" in joined.replace("'/'", "") and re.search(r"/\s*$", joined):
            joined = joined[: joined.rstrip().rfind("/")]
            kv = {}
            for m in re.finditer(r"(\w+)\s*=\s*((?:'[^']*'|\"[^\"]*\"|[^=])*?)(?=\s*,?\s*\w+\s*=|$)", joined):
                vals = [v for v in re.split(r",(?=(?:[^']*'[^']*')*[^']*$)", m.group(2)) if v.strip()]
                parsed = [_value(v) for v in vals]
                kv[m.group(1).lower()] = parsed[0] if len(parsed) == 1 else parsed
            groups.setdefault(cur, kv)
            cur = None
    return groups


# ---------------------------------------------------------------------------
# Fortran-style numbers
# ---------------------------------------------------------------------------
def fortran_g0(x: float, d: int = 16) -> str:
    """Fortran G0.d output as gfortran writes it: F form with d significant
    digits when 0.1 <= |x| < 10**d, otherwise 0.ddddE+-e."""
    if x != x:
        return "NaN"
    if math.isinf(x):
        return "Infinity" if x > 0 else "-Infinity"
    sign = "-" if (x < 0 or (x == 0 and math.copysign(1.0, x) < 0)) else ""
    ax = abs(x)
    if ax == 0.0:
        return sign + "0." + "0" * (d - 1)
    mant, exp = f"{ax:.{d - 1}e}".split("e")
    e10 = int(exp) + 1                  # ax = 0.DDDD * 10**e10
    digits = mant.replace(".", "")
    if 0 <= e10 <= d:                   # 0.1 <= ax < 10**d after rounding
        if e10 == 0:
            return sign + "0." + digits
        return sign + digits[:e10] + "." + digits[e10:]
    return sign + "0." + digits + "E" + ("-" if e10 < 0 else "+") + str(abs(e10))


def fortran_f(x: float, d: int = 6) -> str:
    """Fortran F0.d output as gfortran writes it: with no field width there is
    no leading zero below one (0.2 -> ".200000"); F0.0 keeps the point."""
    t = f"{x:.{d}f}"
    if t.startswith("0."):
        t = t[1:]
    elif t.startswith("-0."):
        t = "-" + t[2:]
    return t + "." if d == 0 else t


def generate_directory(w: Waveguide, root: str = "out") -> str:
    """generate_directory (src/waveguide.f90:1046-1067):
    root/dscat_X/dabso_Y/wol_Z/boundtype/ with F0.6 values, trailing zeros
    removed (a zero is put before the point of values below one)."""
    p = w.get_parameters()

    def folder(stem, v):
        return (stem + ("0" if v < 1.0 else "") + fortran_f(v)).rstrip("0 ")

    return os.path.join(root, folder("dscat_", p["dscat"]), folder("dabso_", p["dabso"]), folder("wol_", p["wol"]),
                        str(p["boundtype"]).strip()) + os.sep


# ---------------------------------------------------------------------------
# Histogram pipeline (src/main.f90:223-251, src/base_utils.f90:491-570)
# ---------------------------------------------------------------------------
def chebyshev_bins(nbins: int, xmin: float = 0.0, xmax: float = 1.0) -> np.ndarray:
    """Bin edges at the Chebyshev nodes (src/main.f90:233, src/plot_histogram.f90:84)."""
    return np.array([xmin + (xmax - xmin) * (1.0 - math.cos(math.pi * (i - 1) / nbins)) / 2
                     for i in range(1, nbins + 2)], np.float64)


def linear_bins(nbins: int, xmin: float = 0.0, xmax: float = 1.0) -> np.ndarray:
    """Linear bin edges (src/plot_histogram.f90:82)."""
    return np.array([xmin + (xmax - xmin) * (i - 1) / nbins for i in range(1, nbins + 2)], np.float64)


def density_from_counts(histo, bins):
    """eps/10 + normalize_histogram + moving_average (src/main.f90:243-245,
    src/base_utils.f90:524-570) on histogram counts: rho_data[nbins, 2] =
    (centre, density)."""
    histo = np.asarray(histo, np.float64) + np.finfo(np.float64).eps / 10.0
    npoints = 0.0
    for v in histo:  # sum(histo): sequential, as the Fortran intrinsic
        npoints += v
    rho = np.array([histo[j] / (npoints * (bins[j + 1] - bins[j])) for j in range(histo.size)])
    centres = np.array([(0.0 + bins[j] + bins[j + 1]) / 2 for j in range(histo.size)])
    return np.stack([centres, rho], axis=1)


def density(samples, bins):
    """histogram (GPU) then density_from_counts: (rho_data[nbins, 2], missing)."""
    histo, missing = histogram(samples, bins)
    return density_from_counts(histo, bins), missing


def prepare_distrib(tallvals, nbins: int):
    """prepare_distrib (src/main.f90:223-251): Chebyshev bins on [0, 1]."""
    return density(tallvals, chebyshev_bins(nbins))


# ---------------------------------------------------------------------------
# Output files (src/main.f90:257-328, src/base_utils.f90:703-716,825-871)
# ---------------------------------------------------------------------------
def unique_filename(base: str, ext: str) -> str:
    i = 1
    while os.path.exists(f"{base}{i}{ext}"):
        i += 1
    return f"{base}{i}{ext}"


def _preamble(w: Waveguide, nseed: int, nbins: int, nthreads: int, tsec: float, prefix: str = "%%",
              seed0: int = 1) -> list[str]:
    """The reference's header lines; a run that starts at seed0 != 1 adds one
    line naming its seed range, so files of disjoint ranges stay apart."""
    p = w.get_parameters()
    now = datetime.datetime.now().astimezone()
    speed = nseed / tsec if tsec > 0 else float("inf")
    extra = [f"{prefix} Seeds {seed0}..{seed0 + nseed - 1}"] if seed0 != 1 else []
    return extra + [
        f"{prefix} Computed on {now:%Y-%m-%d at %H:%M:%S %z} by {PROGRAM}",
        f"{prefix} Waveguide 2D with boundtype='{p['boundtype']}', W/lambda={fortran_f(p['wol'])}, "
        f"exfac={fortran_f(p['exfac'])}, Nmode={w.nmu}, Nprop={w.nprop}",
        f"{prefix} Filtering: NAper_a={fortran_f(p['napera'])} (Nmode_a={w.jmax - w.jmin + 1}), "
        f"NAper_b={fortran_f(p['naperb'])} (Nmode_b={w.imax - w.imin + 1}), Neigv={w.neigv}",
        f"{prefix} Medium: L/lscat={fortran_f(p['dscat'])}, L/labso={fortran_f(p['dabso'])}, "
        f"Nx_diso={p['nxdiso']}, Nx_free={p['nxfree']}, aratio=L/W={fortran_f(p['aratio'])}",
        f"{prefix} Nseed={nseed}, Nbins={nbins}, Nthreads={nthreads}, Time={fortran_g0(tsec, 6)} s, "
        f"Speed={fortran_g0(speed, 6)} seed/s",
    ]


def save_distrib(path: str, rho_data: np.ndarray, preamble: list[str]) -> None:
    with open(path, "w") as f:
        for line in preamble:
            f.write(line + "\n")
        f.write("tm, rho\n")
        for c, r in rho_data:
            f.write(f"{fortran_g0(c)}, {fortran_g0(r)}\n")


def save_raw_eigvals(path: str, tallvals: np.ndarray, preamble: list[str]) -> None:
    with open(path, "w") as f:
        for line in preamble:
            f.write(line + "\n")
        f.write(f"%% Transmission eigenvalues ({tallvals.size} values)\n")
        for v in tallvals:
            f.write(fortran_g0(float(v)) + "\n")


def read_real_array(path: str) -> np.ndarray:
    """read_real_array (src/base_utils.f90:663-697): one list-directed read
    per line; lines whose first item is not a real number are skipped."""
    out = []
    for line in open(path):
        tok = line.strip().replace(",", " ").split()
        if not tok:
            continue
        t = tok[0]
        if t.lower() in ("nan", "+nan", "-nan"):
            out.append(float("nan"))
        elif re.fullmatch(r"[-+]?(\d+\.?\d*|\.\d+)([eEdD][-+]?\d+)?", t):
            out.append(float(t.replace("d", "e").replace("D", "e")))
    return np.array(out, np.float64)


def task_tdistrib(settings: dict, outdir: str = "out", group=None) -> dict:
    """task_tdistrib (src/main.f90:73-123) with the seed loop as one GPU batch.

    With a torch.distributed process group, each rank (one GPU) takes a
    contiguous range of the seeds; the histogram counts are summed over the
    ranks and rank 0 writes the files (see replicas.py).  Other ranks return
    the same rho and missing values with no file paths.

    The optional key seed0 (default 1, the reference's first seed) starts the
    seeds at seed0: runs on separate machines over disjoint ranges give
    eigenvalue files that together are the run over their union."""
    td = settings["tdistrib"]
    nseed, nbins, seed0 = int(td["nseed"]), int(td["nbins"]), int(td.get("seed0", 1))
    if seed0 < 1:
        raise ValueError(f"Invalid first seed, received seed0={seed0}, expected >0, aborting...")
    if seed0 + nseed - 1 > 2 ** 31 - 1:
        raise ValueError(f"Invalid seed range, seed0+nseed-1={seed0 + nseed - 1} exceeds 2147483647, aborting...")
    w = _waveguide_from(settings["waveguide"])
    if group is not None:
        return _task_tdistrib_replicas(w, td, nseed, nbins, outdir, group, seed0)
    t0 = time.perf_counter()
    tallvals = w.tdistrib_batch(np.arange(seed0, seed0 + nseed, dtype=np.int32))
    tsec = time.perf_counter() - t0
    rho, missing = prepare_distrib(tallvals, nbins)
    ddir = os.path.join(generate_directory(w, outdir), "distrib")
    os.makedirs(ddir, exist_ok=True)
    pre = _preamble(w, nseed, nbins, int(td.get("nthreads", 1)), tsec, seed0=seed0)
    dpath = unique_filename(os.path.join(ddir, "result_"), ".distrib.csv")
    save_distrib(dpath, rho, pre)
    res = {"distrib": dpath, "tallvals": tallvals, "rho": rho, "missing": missing, "time": tsec}
    if td.get("save_eigvals", False):
        epath = unique_filename(os.path.join(ddir, "result_"), ".eigvals.csv")
        save_raw_eigvals(epath, tallvals, pre)
        res["eigvals"] = epath
    return res


def _task_tdistrib_replicas(w: Waveguide, td: dict, nseed: int, nbins: int, outdir: str, group,
                            seed0: int = 1) -> dict:
    import torch.distributed as dist

    from . import replicas

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    seeds = replicas.seed_range(rank, world, nseed) + (seed0 - 1)
    t0 = time.perf_counter()
    local = w.tdistrib_batch(seeds) if seeds.size else np.zeros(0)
    tsec = replicas.max_over_ranks(time.perf_counter() - t0, group)
    bins = chebyshev_bins(nbins)
    histo, missing = histogram(local, bins) if local.size else (np.zeros(nbins), 0.0)
    histo, missing = replicas.sum_counts(histo, missing, group)
    rho = density_from_counts(histo, bins)
    tallvals = replicas.gather_values(local, group) if td.get("save_eigvals", False) else None
    res = {"distrib": None, "tallvals": tallvals, "rho": rho, "missing": missing, "time": tsec}
    if rank == 0:
        ddir = os.path.join(generate_directory(w, outdir), "distrib")
        os.makedirs(ddir, exist_ok=True)
        pre = _preamble(w, nseed, nbins, int(td.get("nthreads", 1)), tsec, seed0=seed0)
        res["distrib"] = unique_filename(os.path.join(ddir, "result_"), ".distrib.csv")
        save_distrib(res["distrib"], rho, pre)
        if tallvals is not None:
            res["eigvals"] = unique_filename(os.path.join(ddir, "result_"), ".eigvals.csv")
            save_raw_eigvals(res["eigvals"], tallvals, pre)
    return res


def _waveguide_from(wg: dict) -> Waveguide:
    return Waveguide(boundtype=str(wg.get("boundtype", "dirichlet")).strip(), nxdiso=int(wg["nxdiso"]),
                     nxfree=int(wg.get("nxfree", 0)), wol=float(wg["wol"]), exfac=float(wg.get("exfac", 1.0)),
                     aratio=float(wg.get("aratio", 1.0)), dscat=float(wg["dscat"]), dabso=float(wg.get("dabso", 0.0)),
                     napera=float(wg.get("napera", 1.0)), naperb=float(wg.get("naperb", 1.0)), ny=int(wg.get("ny", 0)))


def tpattern_probabilities(w: Waveguide, nseed: int, imu: int, probatype: str, chunk: int = 256):
    """The seed loop of task_tpattern (src/main.f90:796-836): the mean over
    seeds 1..nseed of |t_{b,imu}|^2 and |r_{b,imu}|^2 ('incident'), of
    sum_b |t_{ba}|^2 and sum_b |r_{ba}|^2 ('total'), or of |d_{b,imu}|^2 for
    the deposition matrix d at the middle of the medium from the first slice
    ('deposition', rprob zero), from batched GPU calls."""
    M = w.nmu
    tsum, rsum = np.zeros(M), np.zeros(M)
    fpos = w.nxfree + w.nxdiso // 2 + 1  # src/main.f90:769-770
    for s0 in range(1, nseed + 1, chunk):
        seeds = np.arange(s0, min(s0 + chunk, nseed + 1), dtype=np.int32)
        if probatype == "deposition":
            d = w.deposition_batch(seeds, fpos, 1, col=imu)
            tp, rp = np.abs(d) ** 2, np.zeros((seeds.size, M))
        else:
            r, t = w.refl_trans_v1_batch(seeds)
            if probatype == "incident":
                tp, rp = np.abs(t[:, :, imu - 1]) ** 2, np.abs(r[:, :, imu - 1]) ** 2
            else:
                tp, rp = (np.abs(t) ** 2).sum(axis=1), (np.abs(r) ** 2).sum(axis=1)
        for k in range(seeds.size):  # seed order, as the Fortran sum over dim=2
            tsum += tp[k]
            rsum += rp[k]
    return tsum / nseed, rsum / nseed


def task_tpattern(settings: dict, outdir: str = "out") -> str:
    """task_tpattern (src/main.f90:735-838) and save_tpattern
    (src/main.f90:843-877).  Returns the result file."""
    tp = settings["tpattern"]
    nseed, imode = int(tp.get("nseed", 0)), int(tp.get("imode", 1))
    probatype = str(tp.get("probatype", "incident")).strip()
    if nseed <= 0:
        raise ValueError(f"Invalid number of disorder realizations (received {nseed}), aborting...")
    if probatype not in ("incident", "total", "deposition"):
        raise ValueError(f"Invalid probatype, received '{probatype}', expected incident/total/deposition, aborting...")
    w = _waveguide_from(settings["waveguide"])
    M = w.nmu
    imu = (imode + M // 2 - 1) % M + 1 if w.get_parameters()["boundtype"] == "periodic" else imode
    if not 1 <= imu <= M:
        raise ValueError(f"Invalid incident mode imode={imode}, expected in [1, {M}], aborting...")
    t0 = time.perf_counter()
    tprob, rprob = tpattern_probabilities(w, nseed, imu, probatype)
    tsec = time.perf_counter() - t0
    ddir = os.path.join(generate_directory(w, outdir), "tpattern")
    os.makedirs(ddir, exist_ok=True)
    path = unique_filename(os.path.join(ddir, "result_"), ".csv")
    pre = _preamble(w, nseed, 0, 1, tsec)[:4]  # timestamp and the waveguide parameters
    with open(path, "w") as f:
        for line in pre:
            f.write(line + "\n")
        f.write(f"%% Radiation pattern parameters: probatype='{probatype}', nseed={nseed}, imode={imode}, "
                f"time={fortran_f(tsec, 3)} s.\n")
        f.write("imu, tprob, rprob\n")
        for i in range(M):
            f.write(f"{i + 1}, {fortran_g0(tprob[i])}, {fortran_g0(rprob[i])}\n")
    return path


def plot_histo_from_file(settings: dict, datafile: str) -> str:
    """plot_histo_from_file (src/plot_histogram.f90:50-143): re-bin saved
    samples into replot_N.distrib.csv next to the data file."""
    st = settings["settings"]
    bintype = str(st.get("bintype", "chebyshev")).strip()
    nbins, xmin, xmax = int(st["nbins"]), float(st.get("xmin", 0.0)), float(st.get("xmax", 1.0))
    if nbins < 1:
        raise ValueError(f"Invalid number of bins (nbins={nbins} must be positive)")
    if not (xmax > xmin):
        raise ValueError("Invalid binning range")
    if bintype == "linear":
        bins = linear_bins(nbins, xmin, xmax)
    elif bintype == "chebyshev":
        bins = chebyshev_bins(nbins, xmin, xmax)
    else:
        raise ValueError(f"Unknown binning type '{bintype}'")
    samples = read_real_array(datafile)
    rho, _ = density(samples, bins)
    pre = []
    for line in open(datafile):
        if line[:1] in ("%", "#"):
            pre.append(line.rstrip("\n"))
        else:
            break
    out = unique_filename(os.path.join(os.path.dirname(os.path.abspath(datafile)), "replot_"), ".distrib.csv")
    save_distrib(out, rho, pre)
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("settings")
    ap.add_argument("datafile", nargs="?")
    ap.add_argument("--outdir", default="out")
    ap.add_argument("--replot", action="store_true")
    a = ap.parse_args(argv)
    nml = read_namelists(open(a.settings).read())
    if a.replot:
        print(plot_histo_from_file(nml, a.datafile))
    else:
        task = str(nml.get("settings", {}).get("task", "tdistrib")).strip()
        if task == "tpattern":
            print(task_tpattern(nml, a.outdir))
            return
        if task in ("wavefunction", "tprofile", "tprofile_group"):
            from . import tprofile as P

            r = getattr(P, "task_" + task)(nml, a.outdir)
            print(r if isinstance(r, str) else r.get("path") or r["avg"])
            return
        r = task_tdistrib(nml, a.outdir)
        print(r["distrib"], f"{r['time']:.3f} s")


if __name__ == "__main__":
    main()
