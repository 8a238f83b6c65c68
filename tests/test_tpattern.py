"""The tpattern task (src/main.f90:735-877) on batched t and r ('incident',
'total') and on the batched deposition matrix ('deposition'): the batch
equals single compute_refl_trans_v1 calls, the averaged probabilities equal
the oracle's, and the C++ program writes the Python driver's rows."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
import recurgreen_gb300 as rg
from recurgreen_gb300 import build
from recurgreen_gb300 import tdistrib as T

pytestmark = pytest.mark.gpu

GUIDES = {
    "dirichlet_m10": dict(boundtype="dirichlet", nxdiso=40, nxfree=2, wol=5.25, exfac=1.0, aratio=1.0, dscat=3.0,
                          ny=32),
    "periodic_m9": dict(boundtype="periodic", nxdiso=30, nxfree=0, wol=4.3, exfac=1.0, aratio=1.0, dscat=2.0),
    "dirichlet_m72": dict(boundtype="dirichlet", nxdiso=10, nxfree=1, wol=36.25, exfac=1.0, aratio=1.0, dscat=6.0,
                          ny=96),
}


@pytest.mark.parametrize("name", sorted(GUIDES))
def test_batch_equals_single_calls(name):
    g = rg.Waveguide(**GUIDES[name])
    seeds = np.array([2, 5, 3], np.int32)
    r, t = g.refl_trans_v1_batch(seeds)
    for k, s in enumerate(seeds):
        r1, t1 = g.compute_refl_trans_v1(int(s))
        np.testing.assert_array_equal(t[k], t1)
        np.testing.assert_array_equal(r[k], r1)


def _oracle_pattern(kw, nseed, imu, probatype):
    o = O.Waveguide(**kw)
    M = o.nmu
    tsum, rsum = np.zeros(M), np.zeros(M)
    for s in range(1, nseed + 1):
        if probatype == "deposition":
            d = o.deposition_upot(o.potential(s), o.nxfree + o.nxdiso // 2 + 1, 1)
            tsum += np.abs(d[:, imu - 1]) ** 2
            continue
        r, t = o.refl_trans_v1_upot(o.potential(s))
        if probatype == "incident":
            tsum += np.abs(t[:, imu - 1]) ** 2
            rsum += np.abs(r[:, imu - 1]) ** 2
        else:
            tsum += (np.abs(t) ** 2).sum(axis=0)
            rsum += (np.abs(r) ** 2).sum(axis=0)
    return tsum / nseed, rsum / nseed


@pytest.mark.parametrize("probatype", ["incident", "total", "deposition"])
@pytest.mark.parametrize("name", ["dirichlet_m10", "periodic_m9"])
def test_pattern_matches_oracle(name, probatype):
    kw = GUIDES[name]
    g = rg.Waveguide(**kw)
    imode = 2
    imu = (imode + g.nmu // 2 - 1) % g.nmu + 1 if kw["boundtype"] == "periodic" else imode
    tp, rp = T.tpattern_probabilities(g, 7, imu, probatype, chunk=3)
    to, ro = _oracle_pattern(kw, 7, imu, probatype)
    assert np.max(np.abs(tp - to)) <= 1e-10 * np.max(np.abs(to))
    if probatype == "deposition":
        assert np.all(rp == 0.0)
        return
    assert np.max(np.abs(rp - ro)) <= 1e-10 * np.max(np.abs(ro))
    if probatype == "total" and kw.get("dabso", 0.0) == 0.0:
        np.testing.assert_allclose(tp + rp, 1.0, rtol=0, atol=1e-10)  # flux per incident propagating channel


NML = """&settings
    task = 'tpattern'
/
&waveguide
    boundtype = 'periodic', wol = 4.3, exfac = 1.0, aratio = 1.0
    dscat = 2.0, dabso = 0.0, nxdiso = 30, nxfree = 0, napera = 1.0, naperb = 1.0
/
&tpattern
    nseed = 9, imode = 2, nthreads = 4, probatype = 'incident'
/
"""


@pytest.mark.parametrize("probatype", ["incident", "deposition"])
def test_cpp_program_writes_python_rows(tmp_path, probatype):
    build.build()
    nml = NML.replace("probatype = 'incident'", f"probatype = '{probatype}'")
    (tmp_path / "s.nml").write_text(nml)
    r = subprocess.run([os.path.join(build.BIN, "recurgreen"), "s.nml"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "out" / "dscat_2." / "dabso_0." / "wol_4.3" / "periodic" / "tpattern" / "result_1.csv"
    lines = out.read_text().splitlines()
    assert lines[4].startswith(f"%% Radiation pattern parameters: probatype='{probatype}', nseed=9, imode=2, time=")
    assert lines[5] == "imu, tprob, rprob"
    py = T.task_tpattern(T.read_namelists(nml), str(tmp_path / "py"))
    pl = open(py).read().splitlines()
    assert pl[1:4] == lines[1:4] and pl[5] == lines[5] and len(pl) == len(lines)
    # same rows up to the libm of |t| (the C++ and numpy hypot may differ by an ulp)
    cpp = np.array([[float(x) for x in l.split(",")] for l in lines[6:]])
    pyv = np.array([[float(x) for x in l.split(",")] for l in pl[6:]])
    np.testing.assert_allclose(cpp, pyv, rtol=1e-15, atol=0)
