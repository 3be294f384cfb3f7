"""The per-step text files in the reference's Fortran formats (fsibe_2d_gb300.outputs):
ESw.d edits of known values, the line layouts of beam_data, u_max, energies, IBES_iter and
mouvement,
and the files the oracle's records produce (append mode, one line per step)."""
import numpy as np

from fsibe_2d_gb300 import make_params
from fsibe_2d_gb300 import outputs as O
from fsibe_2d_gb300._abi import FSIBE_RECORD_COLS


def test_es_edit_descriptor():
    assert O.es(1.0, 15, 8) == " 1.00000000E+00"
    assert O.es(-0.00123, 15, 8) == "-1.23000000E-03"
    assert O.es(0.0, 12, 4) == "  0.0000E+00"
    assert O.es(123456.0, 11, 4) == " 1.2346E+05"
    assert O.es(2.5e-5, 12, 4) == "  2.5000E-05"
    assert O.es(1e-100, 15, 8) == " 1.00000000-100"     # three-digit exponents drop the E
    assert O.es(-9.99999999999e99, 12, 4) == " -1.0000+100"
    assert O.es(1.0, 5, 4) == "*****"                   # does not fit


def test_line_layouts():
    r = np.arange(1, FSIBE_RECORD_COLS + 1, dtype=float) * 0.5
    assert O.beam_data_line(r[O.BEAM]).count("E") == 21 and len(O.beam_data_line(r[O.BEAM])) == 21 * 16
    assert O.u_max_line(r[O.UMAX]).startswith("  ") and len(O.u_max_line(r[O.UMAX])) == 1 + 5 * 13
    assert len(O.energies_line(r[O.ENERGIES])) == 8 * 16
    assert len(O.mouvement_line(r[O.MOUVEMENT])) == 10 * 16
    assert O.ibes_iter_line([0.25, 3]) == " 2.5000E-01   3"


def test_oracle_records_write_the_reference_files(oracle, tmp_path):
    from conftest import seeded_vorticity
    p = make_params(nx=64, ny=64, ns=16)
    o = oracle.OracleRun(p)
    o.init_fields(seeded_vorticity(64))
    rec = o.run_records(5)
    rows = oracle.OracleRun(p)
    rows.init_fields(seeded_vorticity(64))
    assert np.array_equal(rows.time_step(5), rec[:, :21])       # beam_data: the same rows as fsibe_run
    # the u_max, energies and IBES_iter rows carry the time before the step
    assert np.array_equal(rec[1:, 21], rec[:-1, 0]) and rec[0, 21] == 0.0
    assert np.array_equal(rec[:, 26], rec[:, 21]) and np.array_equal(rec[:, 34], rec[:, 21])
    assert rec[0, 35] == 0 and np.all(rec[1:, 35] >= 3)     # no solve at time 0 (not released)
    paths = O.write_step_files(str(tmp_path), rec[:3])
    O.write_step_files(str(tmp_path), rec[3:])                  # appended
    names = sorted(f.name for f in tmp_path.iterdir())
    assert names == ["IBES_iter", "beam_data1", "energies", "mouvement1", "u_max"]
    # the mouvement row: the time after the step, the fixed angle and leading edge (case 0)
    assert np.array_equal(rec[:, 36], rec[:, 0])
    assert np.all(rec[:, 37] == 0.0) and np.all(rec[:, 40] == p.x0) and np.all(rec[:, 41] == p.y0)
    for path in paths:
        lines = open(path).read().splitlines()
        assert len(lines) == (4 if path.endswith("IBES_iter") else 5)
    first = open(tmp_path / "beam_data1").read().splitlines()[0].split()
    assert np.allclose([float(v) for v in first], rec[0, :21], rtol=1e-8, atol=0)
    o.close(); rows.close()


def test_save_field_format1(tmp_path):
    """FieldExport.f90:612-648: the %format1 header and one value a line, top row first."""
    f = np.arange(4 * 8, dtype=float).reshape(4, 8)      # (ny, nx)
    path = O.write_field(str(tmp_path / "p_0.0000E+00"), f, nsave=2, lx=4.0, ly=2.0, header=["% PARAMS"])
    lines = open(path).read().splitlines()
    assert lines[:8] == ["% PARAMS", "%format1", "00008   % nx", "00004   % ny", " 4.0000E+00   % xl, domain size in x-direction",
                         " 2.0000E+00   % yl, domain size in y-direction",
                         "% The next entry can be used to identify the type of the field: ", "% pressure"]
    vals = [float(v) for v in lines[8:]]
    # rows y = 3, 1 (nsave 2 from the top), columns x = 0, 2, 4, 6
    assert vals == [24.0, 26.0, 28.0, 30.0, 8.0, 10.0, 12.0, 14.0]
    p2 = O.write_field(str(tmp_path / "q"), f, 1, 4.0, 2.0, "precision")
    assert open(p2).read().splitlines()[7] == " 2.400000000E+01"
