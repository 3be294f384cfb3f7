"""The per-step files of a GPU run against the oracle's (C1 configuration, first 100 steps):
the records of fsibe_run_records written by fsibe_2d_gb300.outputs in the reference's
formats (beam_data1, u_max, energies, IBES_iter, mouvement1) must read the same, line for line and field
for field: identical, or apart by one unit of the last printed digit, or -- for a value far
below its column's scale, whose printed digits are rounding noise -- within the FP64 parity
bar, 1e-10 of the column's largest magnitude, or at the FP64 rounding level of the file's
largest value (a mean that is zero up to rounding, such as the mean of v)."""
import numpy as np
import pytest

from conftest import seeded_vorticity
from fsibe_2d_gb300 import make_params
from fsibe_2d_gb300 import outputs as O

pytestmark = pytest.mark.gpu


def _value(field):
    """A Fortran ES field as a float (three-digit exponents are written without the E)."""
    if "E" in field or field.lstrip("+-").isdigit():
        return float(field)
    k = max(field.rfind("+"), field.rfind("-"))
    return float(field[:k] + "E" + field[k:])


def _fields_agree(a, b, digits, col_scale, file_scale):
    """Two ES-formatted fields equal, apart by at most one unit of their last digit, within
    1e-10 of their column's scale, or both at the FP64 rounding level of the file's scale."""
    if a == b:
        return True
    va, vb = _value(a), _value(b)
    ulp = 10.0 ** (np.floor(np.log10(max(abs(va), abs(vb), 1e-300))) - digits)
    return abs(va - vb) <= max(1.01 * ulp, 1e-10 * col_scale, 1e-15 * file_scale)


def test_c1_step_files_match_the_oracle(oracle, tmp_path):
    import fsibe_2d_gb300 as F
    n, steps = 256, 100
    p = make_params(nx=n, ny=n, ns=64, Re=100.0, dt=2e-4)
    g, o = F.Run(p), oracle.OracleRun(p)
    w = seeded_vorticity(n, K=8, sigma=1e-3, seed=0)
    g.init_fields(w); o.init_fields(w)
    rg, ro = g.run_records(steps), o.run_records(steps)
    assert np.allclose(rg[:, 35], ro[:, 35])                   # Newton iterations, exactly
    pg = O.write_step_files(str(tmp_path / "gpu"), rg)
    po = O.write_step_files(str(tmp_path / "oracle"), ro)
    digits = {"beam_data1": 8, "u_max": 4, "energies": 8, "IBES_iter": 4, "mouvement1": 8}
    identical = differ = 0
    for a, b in zip(pg, po):
        name = a.rsplit("/", 1)[1]
        la, lb = open(a).read().splitlines(), open(b).read().splitlines()
        assert len(la) == len(lb) == (steps - 1 if name == "IBES_iter" else steps)
        vals = np.abs(np.array([[_value(f) for f in line.split()] for line in lb]))
        scale = vals.max(axis=0)
        file_scale = vals[:, 1:].max()      # column 0 is the time
        for x, y in zip(la, lb):
            if x == y:
                identical += 1
                continue
            differ += 1
            fx, fy = x.split(), y.split()
            assert len(fx) == len(fy)
            for c, (u, v) in enumerate(zip(fx, fy)):
                assert _fields_agree(u, v, digits[name], scale[c], file_scale), (name, c, u, v)
    print(f"step files: {identical} lines identical, {differ} within the last digit")
    g.close(); o.close()
