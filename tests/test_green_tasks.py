"""The full Green-function tasks end to end (src/main.f90:335-728): the Python
task driver against the oracle, and the C++ program `recurgreen` against the
Python driver (same rows; the timestamp and time fields aside)."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
from recurgreen_gb300 import build
from recurgreen_gb300 import tdistrib as T
from recurgreen_gb300 import tprofile as P

pytestmark = pytest.mark.gpu

WG = dict(boundtype="dirichlet", nxdiso=40, nxfree=2, wol=3.3, exfac=1.0, aratio=1.0, dscat=2.0, dabso=0.0,
          napera=1.0, naperb=1.0)
WG_NML = ("&waveguide\n    boundtype = 'dirichlet', wol = 3.3, exfac = 1.0, aratio = 1.0\n"
          "    dscat = 2.0, dabso = 0.0, nxdiso = 40, nxfree = 2, napera = 1.0, naperb = 1.0\n/\n")
OUT = os.path.join("out", "dscat_2.", "dabso_0.", "wol_3.3", "dirichlet")
TMIN, TMAX = 0.1234567, 0.9012345
TM, DT = [0.1111, 0.3737, 0.6161, 0.8585], [0.1013, 0.1013, 0.1013, 0.1013]


def _nml(task, group):
    return f"&settings\n    task = '{task}'\n/\n" + WG_NML + group


def _run(tmp_path, text):
    build.build()
    (tmp_path / "s.nml").write_text(text)
    r = subprocess.run([os.path.join(build.BIN, "recurgreen"), "s.nml"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


def _tvals(o, u, window):
    t = o.refl_trans_v1_upot(u)[1]
    if window:
        t = t[o.imin - 1:o.imax, o.jmin - 1:o.jmax]
    return np.linalg.svd(t, compute_uv=False) ** 2


def test_tprofile_task_matches_oracle(tmp_path):
    nseed = 5
    nml = T.read_namelists(_nml("tprofile", f"&tprofile\n tmin = {TMIN}, tmax = {TMAX}, nseed = {nseed}\n/\n"))
    r = P.task_tprofile(nml, str(tmp_path / "py"))
    o = O.Waveguide(**WG)
    ref, nts = [], []
    for s in range(1, nseed + 1):
        u = o.potential(s)
        tv = _tvals(o, u, False)
        assert np.all(np.abs(tv - TMIN) > 1e-8) and np.all(np.abs(tv - TMAX) > 1e-8)
        p, nt = o.tprofile_upot(u, TMIN, TMAX)
        ref.append(p)
        nts.append(nt)
    np.testing.assert_array_equal(r["nt"], nts)
    ref = np.array(ref)
    assert np.max(np.abs(r["profiles"] - ref)) <= 1e-9 * np.max(np.abs(ref))
    lines = open(r["avg"]).read().splitlines()
    assert lines[5] == "x, tprofile" and len(lines) == 6 + o.nx
    avg = np.array([[float(v) for v in l.split(",")] for l in lines[6:]])
    nz = [k for k in range(nseed) if nts[k]]
    want = ref[nz].sum(axis=0) / len(nz)
    assert np.max(np.abs(avg[:, 1] - want)) <= 1e-9 * np.max(np.abs(want))
    assert lines[4].startswith(f"%% Transmission profile parameters: Found nsample={len(nz)} / nseed={nseed}, "
                               f"nx={o.nx}, tmin={T.fortran_g0(TMIN, 6)}, tmax={T.fortran_g0(TMAX, 6)}, time=")
    assert T.fortran_g0(TMIN, 6) == "0.123457"


def test_tprofile_group_task_matches_oracle(tmp_path):
    nseed = 4
    nml = T.read_namelists(_nml("tprofile_group", f"&tprofile_group\n tm = {', '.join(map(str, TM))}\n"
                                                  f" dt = {', '.join(map(str, DT))}\n nseed = {nseed}\n/\n"))
    r = P.task_tprofile_group(nml, str(tmp_path / "py"))
    o = O.Waveguide(**WG)
    acc, ns, tavgs = np.zeros((o.nx, 4)), np.zeros(4, int), []
    for s in range(1, nseed + 1):
        u = o.potential(s)
        tv = _tvals(o, u, True)
        for k in range(4):
            assert np.all(np.abs(np.abs(tv - TM[k]) - DT[k]) > 1e-8)
        p, nt, ta = o.tprofile_group_upot(u, TM, DT)
        tavgs.append(ta)
        for k in range(4):
            if nt[k]:
                acc[:, k] += p[:, k]
                ns[k] += 1
    np.testing.assert_array_equal(r["nsample"], ns)
    assert abs(r["tavg"] - np.mean(tavgs)) < 1e-12
    lines = open(r["path"]).read().splitlines()
    assert lines[4] == f"%% Transmission profile parameters: nx={o.nx}, tm=[0.111100, 0.373700, 0.616100, " \
                       "0.858500], dt=[0.101300, 0.101300, 0.101300, 0.101300]."
    assert lines[5].startswith(f"%% Results: Found nsample=[{', '.join(map(str, ns))}] over nseed={nseed}, tavg=")
    assert lines[6] == "x, tprofile.1111, tprofile.3737, tprofile.6161, tprofile.8585"
    got = np.array([[float(v) for v in l.split(",")] for l in lines[7:]])
    for k in range(4):
        if ns[k]:
            want = acc[:, k] / ns[k]
            assert np.max(np.abs(got[:, 1 + k] - want)) <= 1e-9 * np.max(np.abs(want))


def test_wavefunction_task_matches_oracle(tmp_path):
    nml = T.read_namelists(_nml("wavefunction", "&wavefunction\n iseed = 3, ipos = 20, imode = 2\n/\n"))
    path = P.task_wavefunction(nml, str(tmp_path / "py"))
    lines = open(path).read().splitlines()
    assert lines[4] == "%% Wavefunction parameters: iseed=3, ipos=20, imode=2"
    assert lines[5] == "x, y, repsi, impsi, upot"
    got = np.array([[float(v) for v in l.split(",")] for l in lines[6:]])
    o = O.Waveguide(**WG)
    want = o.wavefunction_upot(o.potential(3), 20, 2)
    # the file holds G0.16, 16 significant digits: x, y and upot to the last one
    np.testing.assert_allclose(got[:, [0, 1, 4]], want[:, [0, 1, 4]], rtol=1e-15, atol=0)
    assert np.max(np.abs(got[:, 2:4] - want[:, 2:4])) <= 1e-10 * np.max(np.abs(want[:, 2:4]))


@pytest.mark.parametrize("task", ["wavefunction", "tprofile", "tprofile_group"])
def test_cpp_program_writes_python_rows(tmp_path, task):
    groups = {
        "wavefunction": "&wavefunction\n iseed = 2, ipos = 1, imode = 1\n/\n",
        "tprofile": f"&tprofile\n tmin = {TMIN}, tmax = {TMAX}, nseed = 6, nthreads = 4\n/\n",
        "tprofile_group": f"&tprofile_group\n tm = {', '.join(map(str, TM))}, dt = {', '.join(map(str, DT))}\n"
                          " nseed = 5, nthreads = 2\n/\n",
    }
    text = _nml(task, groups[task])
    _run(tmp_path, text)
    nml = T.read_namelists(text)
    py = getattr(P, "task_" + task)(nml, str(tmp_path / "py"))
    if task == "wavefunction":
        pairs = [(tmp_path / OUT / "wavefun" / "result_1.wavefun.csv", py)]
    elif task == "tprofile":
        pairs = [(tmp_path / OUT / "tprofile" / "result_1.raw.csv", py["raw"]),
                 (tmp_path / OUT / "tprofile" / "result_1.avg.csv", py["avg"])]
    else:
        pairs = [(tmp_path / OUT / "tprofile_group" / "result_1.csv", py["path"])]
    for cpp, pyf in pairs:
        a, b = open(cpp).read().splitlines(), open(pyf).read().splitlines()
        assert len(a) == len(b)
        assert a[1:4] == b[1:4]  # parameters
        for la, lb in zip(a[4:], b[4:]):
            if la.startswith("%%"):
                # time differs; tavg sums in another order
                assert la.split("time=")[0].split("tavg=")[0] == lb.split("time=")[0].split("tavg=")[0]
            else:
                assert la == lb


@pytest.mark.parametrize("task", ["tprofile", "tprofile_group"])
def test_tprofile_tasks_replica_path_matches(tmp_path, task):
    """The sharded path (a process group; here one gloo rank) writes the
    single-process rows."""
    import torch.distributed as dist

    group_nml = {"tprofile": f"&tprofile\n tmin = {TMIN}, tmax = {TMAX}, nseed = 5\n/\n",
                 "tprofile_group": f"&tprofile_group\n tm = {', '.join(map(str, TM))}, dt = {', '.join(map(str, DT))}\n"
                                   " nseed = 4\n/\n"}[task]
    nml = T.read_namelists(_nml(task, group_nml))
    one = getattr(P, "task_" + task)(nml, str(tmp_path / "one"))
    dist.init_process_group("gloo", store=dist.HashStore(), rank=0, world_size=1)
    try:
        rep = getattr(P, "task_" + task)(nml, str(tmp_path / "rep"), group=dist.group.WORLD)
    finally:
        dist.destroy_process_group()
    files = [("raw", "avg")] if task == "tprofile" else [("path",)]
    for key in files[0]:
        a, b = open(one[key]).read().splitlines(), open(rep[key]).read().splitlines()
        assert a[1:4] == b[1:4] and len(a) == len(b)
        for la, lb in zip(a[4:], b[4:]):
            if la.startswith("%%"):
                assert la.split("time=")[0] == lb.split("time=")[0]
            else:
                assert la == lb
