"""The C++ host programs bin/recurgreen, bin/plothisto and bin/waveguide_test
(src/main.f90, src/plot_histogram.f90, src/waveguide.test.f90) and the C++
interface include/recurgreen.hpp.

CPU tests cover everything the programs do before the first GPU call: the
settings-file checks and their messages, and the Fortran number formats.  GPU
tests run the tdistrib task end to end against the Python task driver and the
oracle, and re-bin the reference's test data into its replot fixture.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from recurgreen_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
STOP = "STOP RecurGreen: Invalid arguments, aborting..."


@pytest.fixture(scope="module")
def progs():
    build.build()
    return {p: os.path.join(build.BIN, p) for p in build.PROGRAMS}


def run(exe, args, cwd):
    r = subprocess.run([exe] + args, cwd=cwd, capture_output=True, text=True, timeout=600)
    return r.returncode, r.stdout, r.stderr


def test_programs_built(progs):
    for exe in progs.values():
        assert os.access(exe, os.X_OK)


def test_settings_errors_stop_like_the_reference(progs, tmp_path):
    exe = progs["recurgreen"]
    cases = {
        "unknown.nml": ("&settings task = 'nosuch' /\n", "Unknown task 'nosuch', aborting..."),
        "wavefunction.nml": ("&settings\n task = 'wavefunction'  !! c\n/\n",
                             "Invalid entry in namelist: group &waveguide not found"),
        "tp_nseed.nml": ("&settings task='tpattern' /\n&tpattern nseed=0, imode=1, probatype='incident' /\n",
                         "Invalid number of disorder realizations (received 0), aborting..."),
        "tp_type.nml": ("&settings task='tpattern' /\n&tpattern nseed=4, imode=1, probatype='side' /\n",
                        "Invalid probatype, received 'side', expected incident/total/deposition, aborting..."),
        "tg_tm.nml": ("&settings task='tprofile_group' /\n&waveguide wol=5.25 /\n"
                      "&tprofile_group\n tm = 0.1, 0.5\n nseed = 3\n/\n", "Invalid entry in namelist: tm = 0.1, 0.5"),
        "tp_key.nml": ("&settings task='tprofile' /\n&waveguide wol=5.25 /\n&tprofile tmin=0.1, tmid=0.5 /\n",
                       "Invalid entry in namelist:"),
        "entry.nml": ("&settings task='tdistrib' /\n&waveguide\n wol = 5.25, bogus = 3\n/\n&tdistrib nseed=2 /\n",
                      "Invalid entry in namelist: wol = 5.25, bogus = 3..."),
        "nogroup.nml": ("&settings task='tdistrib' /\n&tdistrib nseed=2 /\n",
                        "Invalid entry in namelist: group &waveguide not found"),
        "badreal.nml": ("&settings task='tdistrib' /\n&waveguide\n wol = 5.2x5\n/\n&tdistrib nseed=2 /\n",
                        "Invalid entry in namelist: wol = 5.2x5..."),
    }
    for name, (text, msg) in cases.items():
        (tmp_path / name).write_text(text)
        rc, out, err = run(exe, [name], tmp_path)
        assert rc == 1, name
        assert "Reading file: " + name in out
        assert msg in err and STOP in err, (name, err)
    rc, out, err = run(exe, ["missing.nml"], tmp_path)
    assert rc == 1 and "File not found: missing.nml" in err
    rc, out, err = run(exe, [], tmp_path)
    assert "No settings file provided, doing nothing..." in err


def test_plothisto_checks(progs, tmp_path):
    exe = progs["plothisto"]
    (tmp_path / "d.csv").write_text("%% header\n0.5\n")
    cases = {
        "nb.nml": ("&settings bintype='chebyshev', nbins=0 /\n", "Invalid number of bins (nbins=0 must be positive)"),
        "rg.nml": ("&settings bintype='linear', nbins=4, xmin=1.0, xmax=1.0 /\n", "Invalid binning range, aborting..."),
        "bt.nml": ("&settings bintype='log', nbins=4 /\n", "Unknown binning type 'log', aborting..."),
    }
    for name, (text, msg) in cases.items():
        (tmp_path / name).write_text(text)
        rc, out, err = run(exe, [name, "d.csv"], tmp_path)
        assert rc == 1 and msg in err and STOP in err, (name, err)
        assert "Found 1 samples in the data file..." in out
    rc, out, err = run(exe, ["nb.nml"], tmp_path)
    assert rc == 1 and "Two files expected" in err and "Usage: $ ./plothisto" in out


def test_cpp_interface_formats(tmp_path):
    """recurgreen.hpp is self-contained; its F0.d matches gfortran's (no
    leading zero below one) and the Python driver's."""
    from recurgreen_gb300 import tdistrib as T

    src = tmp_path / "f.cpp"
    src.write_text('#include "recurgreen.hpp"\n#include <cstdio>\nint main() {\n'
                   '  const double v[] = {0.2, 32.25, -0.5, 0.0, 1.0, 0.9999996, 10.0};\n'
                   '  for (double x : v) std::printf("%s\\n", recurgreen::format_f0(x).c_str());\n}\n')
    exe = tmp_path / "f"
    subprocess.run([build.cxx(), "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe)], check=True)
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert got == [".200000", "32.250000", "-.500000", ".000000", "1.000000", "1.000000", "10.000000"]
    assert got == [T.fortran_f(x) for x in (0.2, 32.25, -0.5, 0.0, 1.0, 0.9999996, 10.0)]


SETTINGS = """&settings
    task = 'tdistrib'
/
&waveguide
    boundtype = 'dirichlet'
    wol = 5.25, exfac = 1.0
    dscat = 5., dabso = 0.0, aratio = 1.0
    nxdiso = 200, nxfree = 0
    napera = 1.0, naperb = 1.0
/
&tdistrib
    nseed = 40
    nbins = 100
    nthreads = 8
    save_eigvals = .true.
/
"""


@pytest.mark.gpu
def test_recurgreen_tdistrib_matches_python_driver_and_oracle(progs, tmp_path):
    import oracle as O
    from recurgreen_gb300 import tdistrib as T

    (tmp_path / "settings.nml").write_text(SETTINGS)
    rc, out, err = run(progs["recurgreen"], ["settings.nml"], tmp_path)
    assert rc == 0, err
    ddir = tmp_path / "out" / "dscat_5." / "dabso_0." / "wol_5.25" / "dirichlet" / "distrib"
    dist = (ddir / "result_1.distrib.csv").read_text().splitlines()
    eig = (ddir / "result_1.eigvals.csv").read_text().splitlines()
    assert "Result written in file: out/dscat_5./dabso_0./wol_5.25/dirichlet/distrib/result_1.distrib.csv" in out
    assert dist[0].startswith("%% Computed on ") and dist[0].endswith("by RecurGreen-GB300 (recursive Green "
                                                                    "sweep on GB300)")
    assert dist[1] == "%% Waveguide 2D with boundtype='dirichlet', W/lambda=5.250000, exfac=1.000000, Nmode=10, " \
                      "Nprop=10"
    assert dist[2] == "%% Filtering: NAper_a=1.000000 (Nmode_a=10), NAper_b=1.000000 (Nmode_b=10), Neigv=10"
    assert dist[3] == "%% Medium: L/lscat=5.000000, L/labso=.000000, Nx_diso=200, Nx_free=0, aratio=L/W=1.000000"
    assert dist[4].startswith("%% Nseed=40, Nbins=100, Nthreads=8, Time=")
    assert dist[5] == "tm, rho" and len(dist) == 6 + 100
    assert eig[5] == "%% Transmission eigenvalues (400 values)" and len(eig) == 6 + 400
    # the Python task driver on the same settings: identical rows and preamble lines 1-3
    res = T.task_tdistrib(T.read_namelists(SETTINGS), str(tmp_path / "py"))
    pyd = open(res["distrib"]).read().splitlines()
    assert pyd[1:4] == dist[1:4] and pyd[5:] == dist[5:]
    assert open(res["eigvals"]).read().splitlines()[6:] == eig[6:]
    # the eigenvalues against the oracle
    tall = np.array([float(x) for x in eig[6:]])
    o = O.Waveguide(boundtype="dirichlet", nxdiso=200, nxfree=0, wol=5.25, exfac=1.0, aratio=1.0, dscat=5.0)
    ref = o.tdistrib_batch(np.arange(1, 41, dtype=np.int32))
    assert np.max(np.abs(tall - ref)) <= 1e-9


@pytest.mark.gpu
def test_plothisto_reproduces_reference_replot_fixture(progs, tmp_path):
    """test/test_data.csv -> test/replot_1.distrib.csv of the reference, line by line."""
    with open(os.path.join(GOLD, "replot_fixture.json")) as f:
        r = json.load(f)
    data = tmp_path / "data" / "test_data.csv"
    data.parent.mkdir()
    data.write_text("%% samples\n" + "\n".join("Nan" if s is None else repr(s) for s in r["samples"]) + "\n")
    (tmp_path / "p.nml").write_text(f"&settings\n bintype = '{r['bintype']}'\n nbins = {r['nbins']}\n"
                                    f" xmin = {r['xmin']}\n xmax = {r['xmax']}\n/\n")
    rc, out, err = run(progs["plothisto"], ["p.nml", "data/test_data.csv"], tmp_path)
    assert rc == 0, err
    lines = (tmp_path / "data" / "replot_1.distrib.csv").read_text().splitlines()
    assert lines[0] == "%% samples" and lines[1] == "tm, rho"
    assert lines[2:] == r["lines"]
    assert f"Found {len(r['samples'])} samples in the data file..." in out


@pytest.mark.gpu
def test_waveguide_test_program(progs, tmp_path):
    """src/waveguide.test.f90's checks, printed as the reference prints them, all
    near zero: unitarity of v1 and v2 and v1 - v2 for seeds 1..5."""
    rc, out, err = run(progs["waveguide_test"], [], tmp_path)
    assert rc == 0, err
    lines = out.splitlines()
    assert lines[1] == "| Waveguide 2D with boundtype='dirichlet', W/lambda=4.300000, exfac=1.200000, Nmode=10, Nprop=8"
    heads = [l for l in lines if l.startswith("======")]
    assert heads == ["====== TEST INIT_WAVEGUIDE ======", "====== TEST UNITARITY V1 ======",
                     "====== TEST UNITARITY V2 ======", "====== TEST GREEN V1/V2 ======"]
    tests = [l for l in lines if l.startswith("[TEST] #")]
    assert len(tests) == 20
    assert tests[0].startswith("[TEST] #    1 | norm(t'*t + r'*r - 1) = ") and tests[0].endswith(" (expected 0).")
    for l in tests:
        assert float(l.split(" = ")[1].split(" (")[0]) < 1e-10, l


@pytest.mark.gpu
def test_disjoint_seed_ranges_add_up_to_one_run(progs, tmp_path):
    """&tdistrib seed0 (optional, default 1): runs over seeds 1..10 and 11..20
    give the eigenvalue files of one run over 1..20, and plothisto on their
    concatenation reproduces that run's density rows (the replicas-only
    multi-machine workflow: disjoint seed ranges, merged on the host)."""
    from recurgreen_gb300 import tdistrib as T

    def settings(nseed, seed0=None):
        extra = f", seed0 = {seed0}" if seed0 is not None else ""
        return SETTINGS.replace("nseed = 40", f"nseed = {nseed}{extra}").replace("nbins = 100", "nbins = 16")

    out = {}
    for name, text in (("all", settings(20)), ("lo", settings(10, 1)), ("hi", settings(10, 11))):
        d = tmp_path / name
        d.mkdir()
        (d / "s.nml").write_text(text)
        rc, _, err = run(progs["recurgreen"], ["s.nml"], d)
        assert rc == 0, err
        ddir = d / "out" / "dscat_5." / "dabso_0." / "wol_5.25" / "dirichlet" / "distrib"
        ev, ds = (ddir / "result_1.eigvals.csv").read_text(), (ddir / "result_1.distrib.csv").read_text()
        if name == "hi":  # a run that does not start at seed 1 names its range in the header
            assert ev.splitlines()[0] == "%% Seeds 11..20" and ds.splitlines()[0] == "%% Seeds 11..20"
        else:
            assert "Seeds" not in ev and "Seeds" not in ds
        body = [ln for ln in ds.splitlines() if not ln.startswith("%") and ln != "tm, rho"]
        out[name] = ([ln for ln in ev.splitlines() if not ln.startswith("%")], body)
    assert out["lo"][0] + out["hi"][0] == out["all"][0]
    merged = tmp_path / "merged.csv"
    merged.write_text("%% seeds 1..10 and 11..20\n" + "\n".join(out["lo"][0] + out["hi"][0]) + "\n")
    (tmp_path / "p.nml").write_text("&settings\n bintype = 'chebyshev'\n nbins = 16\n xmin = 0.0\n xmax = 1.0\n/\n")
    rc, _, err = run(progs["plothisto"], ["p.nml", "merged.csv"], tmp_path)
    assert rc == 0, err
    assert (tmp_path / "replot_1.distrib.csv").read_text().splitlines()[2:] == out["all"][1]
    # the Python driver takes the same key
    res = T.task_tdistrib(T.read_namelists(settings(10, 11)), str(tmp_path / "py"))
    assert [T.fortran_g0(float(v)) for v in res["tallvals"]] == out["hi"][0]
