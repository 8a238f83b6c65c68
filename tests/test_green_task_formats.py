"""Host logic of the full Green-function tasks without a GPU: a stand-in
waveguide returns fixed profiles, and the task drivers must average them and
write the files as the reference's task_tprofile / task_tprofile_group /
task_wavefunction do (src/main.f90:335-728): nsample counts realizations with
nt != 0, averages run in seed order, Tavg = sum/nseed with uncertainty
sqrt(sum (T - Tavg)^2)/nseed, `%%` preamble, G0.16 rows."""
import math

import numpy as np
import pytest

from recurgreen_gb300 import tdistrib as T
from recurgreen_gb300 import tprofile as P


class StandIn:
    """The attributes and methods the task drivers use, with fixed results."""

    nmu, nprop, neigv, imin, imax, jmin, jmax = 4, 4, 4, 1, 4, 1, 4
    nxdiso, nxfree, ny = 5, 1, 3
    nx = nxdiso + 2 * nxfree

    def get_parameters(self):
        return dict(boundtype="dirichlet", nxdiso=self.nxdiso, nxfree=self.nxfree, wol=2.25, exfac=1.0, aratio=1.0,
                    dscat=3.0, dabso=0.0, napera=1.0, naperb=1.0, ny=self.ny)

    def get_xmesh(self):
        return np.array([(i - 0.5 - self.nxfree) / self.nxdiso for i in range(1, self.nx + 1)])

    def tprofile_batch(self, seeds, kind, a, b):
        seeds = np.asarray(seeds)
        a = np.atleast_1d(a)
        prof = np.array([[[s + 0.25 * w + ix / 7.0 for ix in range(self.nx)] for w in range(a.size)]
                         for s in seeds], np.float64)
        nt = np.array([[0 if (s + w) % 3 == 0 else (s + w) % 4 for w in range(a.size)] for s in seeds], np.int32)
        prof[nt == 0] = 0.0
        tavg = np.array([0.1 * s for s in seeds], np.float64)
        return prof, nt, tavg

    def compute_wavefunction(self, iseed, ipos, imode):
        rows = self.nx * self.ny
        return np.arange(rows * 5, dtype=np.float64).reshape(rows, 5) / 3.0


WG = "&waveguide\n boundtype='dirichlet', wol=2.25, dscat=3.0, nxdiso=5, nxfree=1\n/\n"


@pytest.fixture
def stand_in(monkeypatch):
    w = StandIn()
    monkeypatch.setattr(P, "_waveguide_from", lambda wg: w)
    return w


def test_tprofile_task_files(stand_in, tmp_path):
    w = stand_in
    nml = T.read_namelists("&settings task='tprofile' /\n" + WG + "&tprofile tmin=0.25, tmax=0.75, nseed=7 /\n")
    r = P.task_tprofile(nml, str(tmp_path))
    prof, nt, _ = w.tprofile_batch(np.arange(1, 8), "tprofile", [0.25], [0.75])
    keep = [k for k in range(7) if nt[k, 0] != 0]
    assert r["nsample"] == len(keep)
    raw = open(r["raw"]).read().splitlines()
    assert raw[0].startswith("%% Computed on ")
    assert raw[1] == "%% Waveguide 2D with boundtype='dirichlet', W/lambda=2.250000, exfac=1.000000, Nmode=4, " \
                     "Nprop=4"
    assert raw[4].startswith(f"%% Transmission profile parameters: Found nsample={len(keep)} / nseed=7, nx=7, "
                             "tmin=0.250000, tmax=0.750000, time=")
    assert raw[4].endswith(" s.")
    assert raw[5] == "%% Here follows, on each line, the function |psi_T(x)|^2 for a given realization of the disorder."
    assert raw[6] == ", ".join(T.fortran_g0(float(v)) for v in prof[0, 0])
    assert raw[6:] == [", ".join(T.fortran_g0(float(v)) for v in row) for row in prof[:, 0, :]]
    avg = open(r["avg"]).read().splitlines()
    assert avg[5] == "x, tprofile" and len(avg) == 6 + w.nx
    want = sum(prof[k, 0] for k in keep) / len(keep)
    assert avg[6:] == [f"{T.fortran_g0(float(x))}, {T.fortran_g0(float(v))}" for x, v in zip(w.get_xmesh(), want)]
    assert r["raw"].endswith("tprofile/result_1.raw.csv") and r["avg"].endswith("tprofile/result_1.avg.csv")


def test_tprofile_group_task_file(stand_in, tmp_path):
    w = stand_in
    nml = T.read_namelists("&settings task='tprofile_group' /\n" + WG +
                           "&tprofile_group tm = 0.05, 0.5, 0.75, 1.0, dt = 0.05, 0.1, 0.1, 0.25, nseed = 6 /\n")
    r = P.task_tprofile_group(nml, str(tmp_path))
    prof, nt, tavgs = w.tprofile_batch(np.arange(1, 7), "group", [0.05, 0.5, 0.75, 1.0], [0.05, 0.1, 0.1, 0.25])
    lines = open(r["path"]).read().splitlines()
    assert lines[4] == "%% Transmission profile parameters: nx=7, tm=[0.500000E-1, 0.500000, 0.750000, 1.00000], " \
                       "dt=[0.500000E-1, 0.100000, 0.100000, 0.250000]."
    ns = [int(np.count_nonzero(nt[:, p])) for p in range(4)]
    tavg = np.sum(tavgs) / 6
    unc = math.sqrt(np.sum((tavgs - tavg) ** 2)) / 6
    assert lines[5].startswith(f"%% Results: Found nsample=[{', '.join(map(str, ns))}] over nseed=6, "
                               f"tavg={T.fortran_g0(tavg, 6)}+-{T.fortran_g0(unc, 6)}, time=")
    assert lines[6] == "x, tprofile.0500, tprofile.5000, tprofile.7500, tprofile1.0000"
    want = np.zeros((w.nx, 4))
    for p in range(4):
        keep = [k for k in range(6) if nt[k, p] != 0]
        want[:, p] = sum(prof[k, p] for k in keep) / len(keep)
    assert lines[7:] == [", ".join(T.fortran_g0(float(v)) for v in [x, *row]) for x, row in zip(w.get_xmesh(), want)]
    assert r["nsample"].tolist() == ns


def test_tprofile_group_needs_four_values(stand_in, tmp_path):
    nml = T.read_namelists("&settings task='tprofile_group' /\n" + WG + "&tprofile_group tm = 0.5, dt = 0.1 /\n")
    with pytest.raises(ValueError, match="tm and dt need 4 values each"):
        P.task_tprofile_group(nml, str(tmp_path))


def test_wavefunction_task_file(stand_in, tmp_path):
    w = stand_in
    nml = T.read_namelists("&settings task='wavefunction' /\n" + WG + "&wavefunction iseed=3, ipos=2, imode=4 /\n")
    path = P.task_wavefunction(nml, str(tmp_path))
    lines = open(path).read().splitlines()
    assert lines[4] == "%% Wavefunction parameters: iseed=3, ipos=2, imode=4"
    assert lines[5] == "x, y, repsi, impsi, upot"
    data = w.compute_wavefunction(3, 2, 4)
    assert lines[6] == ", ".join(T.fortran_g0(float(v)) for v in data[0])
    assert len(lines) == 6 + data.shape[0]
    assert path.endswith("wavefun/result_1.wavefun.csv")


@pytest.mark.parametrize("task,group", [
    ("tprofile", "&tprofile tmin=0.25, tmax=0.75, nseed=3 /\n"),
    ("tprofile_group", "&tprofile_group tm = 0.1, 0.4, 0.6, 0.9, dt = 0.1, 0.1, 0.1, 0.1, nseed = 3 /\n"),
    ("wavefunction", "&wavefunction iseed=1, ipos=1, imode=1 /\n"),
])
def test_command_line_dispatches_the_task(stand_in, tmp_path, capsys, task, group):
    """`python -m recurgreen_gb300.tdistrib settings.nml` runs the task that
    &settings names (src/main.f90:41-66) and prints the file it wrote."""
    (tmp_path / "s.nml").write_text(f"&settings task='{task}' /\n" + WG + group)
    T.main([str(tmp_path / "s.nml"), "--outdir", str(tmp_path / "out")])
    printed = capsys.readouterr().out.strip()
    sub = {"tprofile": "tprofile", "tprofile_group": "tprofile_group", "wavefunction": "wavefun"}[task]
    assert f"/{sub}/result_1." in printed and printed.startswith(str(tmp_path / "out"))
