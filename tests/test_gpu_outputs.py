"""The per-step files of a GPU run against the oracle's (C1 configuration, first 100 steps):
the records of fsibe_run_records written by fsibe_2d_gb300.outputs in the reference's
formats (beam_data1, u_max, energies, IBES_iter) must read the same, line for line and field
for field, except in the last printed digit (FP64 parity is 1e-10, far inside es15.8)."""
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


def _fields_agree(a, b, digits):
    """Two ES-formatted fields equal, or apart by at most one unit of their last digit."""
    if a == b:
        return True
    va, vb = _value(a), _value(b)
    scale = 10.0 ** (np.floor(np.log10(max(abs(va), abs(vb), 1e-300))) - digits)
    return abs(va - vb) <= 1.01 * scale


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
    digits = {"beam_data1": 8, "u_max": 4, "energies": 8, "IBES_iter": 4}
    identical = differ = 0
    for a, b in zip(pg, po):
        name = a.rsplit("/", 1)[1]
        la, lb = open(a).read().splitlines(), open(b).read().splitlines()
        assert len(la) == len(lb) == (steps - 1 if name == "IBES_iter" else steps)
        for x, y in zip(la, lb):
            if x == y:
                identical += 1
                continue
            differ += 1
            fx, fy = x.split(), y.split()
            assert len(fx) == len(fy)
            for u, v in zip(fx, fy):
                assert _fields_agree(u, v, digits[name]), (name, x, y)
    print(f"step files: {identical} lines identical, {differ} within the last digit")
    g.close(); o.close()
