"""capsp_run, the command-line driver with the reference's main.cu flow: it
reads a Matrix Market file, extracts the unit lower triangle, counts levels,
runs the chosen variant twice and appends the reference's result.csv header and
row.  The structural columns (m, nnzL, nnzL/m, layer, parallelism) must equal
those of the same flow through the host helpers (pinned bit for bit against
the reference elsewhere); the timing columns must show a validated solve."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

import capellinisptrsv_gb300 as cs
from capellinisptrsv_gb300 import build as B

pytestmark = pytest.mark.gpu

HEADER = "filename,m,nnzL,nnzL/m,layer,parallelism,pre_time,solve_time,gflops,bandwith"


def write_mtx(path, n, rows, cols, vals):
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{n} {n} {len(rows)}\n")
        for r, c, v in zip(rows, cols, vals):
            f.write("%d %d %.17g\n" % (r + 1, c + 1, v))


@pytest.fixture(scope="module")
def mtx(tmp_path_factory):
    """A general matrix: the 20k-row workload's lower triangle plus its mirror."""
    m = cs.generate("plain_20k", seed=0)
    rows = np.repeat(np.arange(m.n), np.diff(m.rowptr))
    off = m.colidx != rows
    r = np.concatenate([rows, m.colidx[off]])
    c = np.concatenate([m.colidx, rows[off]])
    v = np.concatenate([m.val, m.val[off]])
    p = tmp_path_factory.mktemp("cli") / "plain20k.mtx"
    write_mtx(p, m.n, r, c, v)
    return p


def expected(path):
    mm, n, nnz, rp, ci, v = cs.read_mtx(str(path))
    nnzL, rpL, ciL, vL = cs.change2tran(mm, rp, ci, v)
    layer, par = cs.matrix_layer(mm, mm, nnzL, rpL, ciL, vL)
    return mm, nnzL, layer, par


@pytest.mark.parametrize("alg,extra", [("wrtfst", []), ("twopart", []), ("mix", []), ("csc", []),
                                       ("wrtfst", ["--f32"])])
def test_cli_result_csv(mtx, tmp_path, alg, extra):
    out = tmp_path / "result.csv"
    r = subprocess.run([str(B.CLI), "--alg", alg, *extra, "--out", str(out), str(mtx)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = out.read_text().splitlines()
    assert len(lines) == 2
    hdr = HEADER + (",warp_occupy,element_occupy" if alg == "mix" else "")
    assert lines[0] == hdr
    f = [x.strip() for x in lines[1].split(",")]
    assert len(f) == len(hdr.split(","))
    m, nnzL, layer, par = expected(mtx)
    assert f[0] == str(mtx)
    assert int(f[1]) == m and int(f[2]) == nnzL and int(f[4]) == layer
    assert f[3] == "%4.2f" % (nnzL / m) and f[5] == "%4.2f" % par
    solve_time, gflops = float(f[7]), float(f[8])
    assert solve_time > 0 and gflops > 0  # the driver validated x against ones
    if alg == "mix":
        assert 0.0 <= float(f[10]) <= 1.0 and 0.0 <= float(f[11]) <= 1.0
