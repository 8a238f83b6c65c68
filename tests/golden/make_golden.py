"""Regenerates the golden fixtures of this directory from the reference tree.

Reads, as text, the known-answer data of RecurGreen's own tests and test files
(src/base_utils.test.f90, test/test_data.csv, test/replot_1.distrib.csv) and
writes them as JSON.  Run once where the reference checkout is available:

    python tests/golden/make_golden.py /path/to/RecurGreen

The fixtures are committed; nothing at test time reads the reference tree.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def complex_matrix(src: str, sub: str, var: str, shape):
    """A = reshape([(re, im), ...], shape(A), order=[2, 1]) inside subroutine `sub`."""
    body = src[src.index("subroutine " + sub):]
    body = body[:body.index("end subroutine")]
    m = re.search(var + r"\s*=\s*reshape\(\[(.*?)\],\s*shape", body, re.S)
    pairs = re.findall(r"\(\s*([-0-9.eE]+)_wp\s*,\s*([-0-9.eE]+)_wp\s*\)", m.group(1))
    vals = [[float(a), float(b)] for a, b in pairs]
    assert len(vals) == shape[0] * shape[1]
    return {"shape": list(shape), "order": "row-major", "re_im": vals}


def complex_array_f(src: str, sub: str, var: str, shape):
    """A = reshape([(re, im), ...], shape(A)) inside subroutine `sub`, no
    order= argument: Fortran (column-major) element order."""
    body = src[src.index("subroutine " + sub):]
    body = body[:body.index("end subroutine")]
    body = "\n".join(l for l in body.splitlines() if not l.lstrip().startswith("!"))
    m = re.search(var + r"\s*=\s*reshape\(\[(.*?)\],\s*shape", body, re.S)
    pairs = re.findall(r"\(\s*([-0-9.eE]+)_wp\s*,\s*([-0-9.eE]+)_wp\s*\)", m.group(1))
    vals = [[float(a), float(b)] for a, b in pairs]
    n = 1
    for d in shape:
        n *= d
    assert len(vals) == n
    return {"shape": list(shape), "order": "fortran", "re_im": vals}


def real_vector(src: str, sub: str, var: str):
    body = src[src.index("subroutine " + sub):]
    body = body[:body.index("end subroutine")]
    m = re.search(var + r"\s*=\s*\[(.*?)\]", body, re.S)
    return [float(x.replace("_wp", "")) for x in re.findall(r"[-0-9.eE]+_wp", m.group(1))]


def fortran_list_read(path: str):
    """Values `read(funit, *) buffer` accepts line by line (read_real_array,
    src/base_utils.f90:663-697): the first token of a line if it parses as a
    real (Fortran accepts 'Nan' and leading-dot mantissas), blank lines are
    skipped by list-directed input, anything else is an error and skipped."""
    out = []
    for line in open(path):
        tok = line.strip().replace(",", " ").split()
        if not tok:
            continue
        t = tok[0]
        if t.lower() in ("nan", "+nan", "-nan"):
            out.append(float("nan"))
            continue
        if re.fullmatch(r"[-+]?(\d+\.?\d*|\.\d+)([eEdD][-+]?\d+)?", t):
            out.append(float(t.replace("d", "e").replace("D", "e")))
    return out


def main(ref: str) -> None:
    src = open(os.path.join(ref, "src", "base_utils.test.f90")).read()
    g = {
        "source": "RecurGreen src/base_utils.test.f90",
        "singular_values": {
            "A": complex_matrix(src, "test_singular_values", "A", (4, 3)),
            "S_expc": real_vector(src, "test_singular_values", "S_expc"),
        },
        "diagonalize_ahca": {"A": complex_matrix(src, "test_diagonalize_ahca", "A", (4, 3)),
                             "T_expc": real_vector(src, "test_diagonalize_ahca", "T_expc")},
        "solve_block_tridiag": {
            "amat": complex_array_f(src, "test_solve_block_tridiag", "amat", (3, 2, 2)),
            "imat": complex_array_f(src, "test_solve_block_tridiag", "imat", (3, 2, 1)),
            "bdiag": real_vector(src, "test_solve_block_tridiag", "bdiag"),
        },
        "inverse_complex": {"A": complex_matrix(src, "test_inverse_complex", "A", (4, 4))},
        "norm2_complex": {"A": complex_matrix(src, "test_norm2_complex", "A", (4, 3)), "expected": 2.646045307275178},
        "histogram": {
            "samples": real_vector(src, "test_histogram", "samples"),
            "bins": [-1.0, -0.5, 0.0, 0.5, 1.0],
            "histo_expc": real_vector(src, "test_histogram", "histo_expc"),
        },
        "moving_average": {
            "signal": real_vector(src, "test_moving_average", "signal"),
            "res_expc": real_vector(src, "test_moving_average", "res_expc"),
        },
    }
    with open(os.path.join(HERE, "base_utils_kat.json"), "w") as f:
        json.dump(g, f, indent=1)
    samples = fortran_list_read(os.path.join(ref, "test", "test_data.csv"))
    rows, lines = [], []
    for line in open(os.path.join(ref, "test", "replot_1.distrib.csv")):
        if line.startswith("%") or line.startswith("tm") or not line.strip():
            continue
        a, b = line.split(",")
        rows.append([float(a), float(b)])
        lines.append(line.rstrip("\n"))
    rep = {"source": "RecurGreen test/test_data.csv -> test/replot_1.distrib.csv (plothisto, chebyshev bins on [0, 1])",
           "bintype": "chebyshev", "xmin": 0.0, "xmax": 1.0, "nbins": len(rows),
           "samples": [None if s != s else s for s in samples], "rho": rows, "lines": lines}
    with open(os.path.join(HERE, "replot_fixture.json"), "w") as f:
        json.dump(rep, f, indent=0)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/RecurGreen")
    main(sys.argv[1])
