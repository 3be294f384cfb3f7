"""Runtime backup through the C ABI: a file written by either side resumes on both, and the
resumed runs agree (FP64 plain form: relative L2 1e-10 on vorticity and the beam after the
stated steps, the parity bar of the whole step; FP32-compensated form: 1e-5).  A GPU file
read back and written again keeps every record bit for bit (FP64) but the mask, drawn anew,
and the packed spectra, which pass through the device layout and back (relative 1e-15)."""
import numpy as np
import pytest

from conftest import rel, seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C, FSIBE_FP64
from test_backup import read_records

pytestmark = pytest.mark.gpu


def _compare(g, o, tol):
    assert rel(g.vortk(), o.vortk()) < tol
    bg, bo = g.beam(), o.beam()
    assert rel(bg[0], bo[0]) < tol
    sg, so = g.scalars(), o.scalars()
    assert sg.status == 0 and so.status == 0
    assert abs(sg.time - so.time) <= 1e-12 * so.time
    assert rel(np.array(sg.force[:2]), np.array(so.force[:2])) < 100 * tol


@pytest.mark.parametrize("prec,tol", [(FSIBE_FP64, 1e-10), (FSIBE_FP32C, 1e-5)])
@pytest.mark.parametrize("writer", ["gpu", "oracle"])
def test_resume_on_both_sides(oracle, tmp_path, prec, tol, writer):
    import fsibe_2d_gb300 as F
    n, ns = 256, 64
    p = make_params(nx=n, ny=n, ns=ns, precision=prec)
    w = seeded_vorticity(n, seed=11)
    path = tmp_path / "runtime_backup0.in"
    src = F.Run(p) if writer == "gpu" else oracle.OracleRun(p)
    src.init_fields(w)
    src.time_step(8)
    src.MakeRuntimeBackup(path)
    src.close()
    g, o = F.Run(p), oracle.OracleRun(p)
    g.resume(path); o.resume(path)
    _compare(g, o, tol)
    g.time_step(6); o.time_step(6)
    _compare(g, o, tol)
    g.close(); o.close()


def test_gpu_write_read_write(tmp_path):
    import fsibe_2d_gb300 as F
    n = 256
    p = make_params(nx=n, ny=n, ns=64, precision=FSIBE_FP64)
    a, b = tmp_path / "a.in", tmp_path / "b.in"
    g = F.Run(p)
    g.init_fields(seeded_vorticity(n, seed=5))
    g.time_step(7)
    g.MakeRuntimeBackup(a)
    r = F.Run(p)
    r.resume(a)
    r.MakeRuntimeBackup(b)
    ra, rb = read_records(a), read_records(b)
    NN = n * n
    for i in range(len(ra)):
        if i != 2:
            assert ra[i] == rb[i], i
    # n1, dt1; the packed spectra pass through the half-complex layout and back (one rounding
    # of a sum and a difference); workvis, ivideo and u are bit for bit; the mask is drawn anew
    assert ra[2][:12] == rb[2][:12]
    sa = np.frombuffer(ra[2], dtype="<f8", count=4 * NN, offset=12)
    sb = np.frombuffer(rb[2], dtype="<f8", count=4 * NN, offset=12)
    assert rel(sb, sa) < 1e-15
    lo, hi = 12 + 8 * 4 * NN, 12 + 8 * 6 * NN
    assert ra[2][lo:hi] == rb[2][lo:hi]
    assert ra[2][12 + 8 * 9 * NN:] == rb[2][12 + 8 * 9 * NN:]
    g.close(); r.close()
