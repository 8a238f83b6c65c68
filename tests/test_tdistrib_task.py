"""The tdistrib task driver and plothisto re-binning (src/main.f90:73-328,
src/plot_histogram.f90:7-143): namelist input, Fortran G0.16 output, and the
histogram pipeline checked against the reference's replot fixture."""
import json
import os

import numpy as np
import pytest

from recurgreen_gb300 import tdistrib as T

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _fixture():
    with open(os.path.join(GOLD, "replot_fixture.json")) as f:
        return json.load(f)


def test_g0_16_matches_reference_output():
    r = _fixture()
    for (c, v), line in zip(r["rho"], r["lines"]):
        assert f"{T.fortran_g0(c)}, {T.fortran_g0(v)}" == line
    assert T.fortran_g0(0.5) == "0.5000000000000000"
    assert T.fortran_g0(-2.5e-7) == "-0.2500000000000000E-6"
    assert T.fortran_g0(123456.0) == "123456.0000000000"


NML = """!! settings in the reference's namelist style
&settings
    task = 'tdistrib'   !! comment with a / slash
/
!&waveguide
!    wol = 99.5
!/
&waveguide
    boundtype = 'dirichlet'
    wol = 5.25, exfac = 1.0   !! two on one line
    dscat = 5., dabso = 0.0
    aratio = 1.0
    nxdiso = 200
    nxfree = 0
    napera = 1.0
    naperb = 1.0
/
&tdistrib
    nseed = 40
    nbins = 100
    nthreads = 8
    save_eigvals = .true.
/
&tprofile_group
    tm = 0.998, 0.50, 0.100
/
"""


def test_namelist_reader():
    g = T.read_namelists(NML)
    assert g["settings"]["task"] == "tdistrib"
    w = g["waveguide"]
    assert w["boundtype"] == "dirichlet" and w["wol"] == 5.25 and w["exfac"] == 1.0 and w["nxdiso"] == 200
    assert w["dscat"] == 5.0 and g["tdistrib"]["save_eigvals"] is True
    assert g["tprofile_group"]["tm"] == [0.998, 0.5, 0.1]


def test_read_real_array_semantics(tmp_path):
    p = tmp_path / "data.csv"
    p.write_text("%% header\n0.1\n## comment\n\n-2.5e-3\n.5\nNan\n0.75, -0.1\nblah\n!! x\n17\n")
    v = T.read_real_array(str(p))
    assert np.isnan(v[3])
    np.testing.assert_array_equal(np.delete(v, 3), [0.1, -2.5e-3, 0.5, 0.75, 17.0])


def test_bins():
    b = T.chebyshev_bins(4)
    assert b[0] == 0.0 and b[-1] == 1.0 and abs(b[2] - 0.5) < 1e-16
    np.testing.assert_array_equal(T.linear_bins(4, -1, 1), [-1.0, -0.5, 0.0, 0.5, 1.0])


@pytest.mark.gpu
def test_replot_fixture_on_gpu(tmp_path):
    """plothisto on the reference's test data reproduces test/replot_1.distrib.csv line by line."""
    r = _fixture()
    data = tmp_path / "test_data.csv"
    data.write_text("%% samples\n" + "\n".join("Nan" if s is None else repr(s) for s in r["samples"]) + "\n")
    settings = {"settings": {"bintype": "chebyshev", "nbins": r["nbins"], "xmin": 0.0, "xmax": 1.0}}
    out = T.plot_histo_from_file(settings, str(data))
    lines = [l.rstrip("\n") for l in open(out)]
    assert lines[0] == "%% samples" and lines[1] == "tm, rho"
    assert lines[2:] == r["lines"]


@pytest.mark.gpu
def test_task_tdistrib_end_to_end(tmp_path):
    import oracle as O

    g = T.read_namelists(NML)
    res = T.task_tdistrib(g, str(tmp_path))
    lines = open(res["distrib"]).read().splitlines()
    assert lines[0].startswith("%% Computed on") and lines[4].startswith("%% Nseed=40, Nbins=100")
    assert lines[5] == "tm, rho" and len(lines) == 6 + 100
    wkw = g["waveguide"]
    o = O.Waveguide(**{k: v for k, v in wkw.items()})
    ref = o.tdistrib_batch(np.arange(1, 41, dtype=np.int32))
    assert np.max(np.abs(res["tallvals"] - ref)) <= 1e-9
    rho_o, miss_o = O.prepare_distrib(ref, 100)
    np.testing.assert_allclose(res["rho"], rho_o, rtol=1e-13, atol=0)
    eig = open(res["eigvals"]).read().splitlines()
    assert eig[5] == "%% Transmission eigenvalues (400 values)" and len(eig) == 6 + 400


@pytest.mark.gpu
def test_task_tdistrib_replica_path_matches(tmp_path):
    """The sharded path of task_tdistrib (a process group; here one gloo rank
    on one GPU) writes the same distribution as the single-process path."""
    import torch.distributed as dist

    g = T.read_namelists(NML)
    plain = T.task_tdistrib(g, str(tmp_path / "plain"))
    dist.init_process_group("gloo", store=dist.HashStore(), rank=0, world_size=1)
    try:
        rep = T.task_tdistrib(g, str(tmp_path / "rep"), group=dist.group.WORLD)
    finally:
        dist.destroy_process_group()
    np.testing.assert_array_equal(rep["rho"], plain["rho"])
    np.testing.assert_array_equal(rep["tallvals"], plain["tallvals"])
    assert open(rep["distrib"]).read().splitlines()[5:] == open(plain["distrib"]).read().splitlines()[5:]


def test_seed_range_checked_before_any_device_work():
    """seed0 < 1 and seed ranges past the int32 seeds of the C ABI are rejected
    (no GPU needed: the check comes before the waveguide is built)."""
    s = T.read_namelists(NML)
    for seed0, nseed in ((0, 10), (2 ** 31 - 5, 10)):
        s["tdistrib"]["seed0"], s["tdistrib"]["nseed"] = seed0, nseed
        with pytest.raises(ValueError):
            T.task_tdistrib(s, "/nonexistent")
