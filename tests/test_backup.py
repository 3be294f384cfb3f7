"""Runtime backup (save_fields.f90:109-152, init_fields.f90:44-100) on the oracle: the file's
record layout, a write -> resume -> write round trip, and the refusals of init_fields (wrong
checksum, different ns).  The GPU side of the same files is in test_gpu_backup.py."""
import struct

import numpy as np
import pytest

from conftest import seeded_vorticity
from fsibe_2d_gb300 import make_params


def read_records(path):
    """Fortran sequential unformatted records: int32 length, payload, int32 length."""
    out = []
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        (n,) = struct.unpack_from("<i", data, pos)
        rec = data[pos + 4:pos + 4 + n]
        (m,) = struct.unpack_from("<i", data, pos + 4 + n)
        assert m == n
        out.append(rec)
        pos += n + 8
    return out


def record_sizes(nx, ny, ns):
    NN = nx * ny
    return [8, 8, 4 + 8 + 8 * (6 * NN + 3 * NN) + 4 + 8 * 2 * NN, 4, 12,
            8 * 6 * ns, 8 * 4 * ns, 8 * 11, 8 + 4 + 8 * 4, 4 + 8 + 8 * 6 * ns, 8 * (2 * ns + 2), 8 * NN]


def _oracle_state(oracle, p, steps, path):
    o = oracle.OracleRun(p)
    o.init_fields(seeded_vorticity(p.nx, seed=3))
    o.time_step(steps)
    o.MakeRuntimeBackup(path)
    return o


def test_record_layout(oracle, tmp_path):
    p = make_params(nx=64, ny=64, ns=32)
    path = tmp_path / "runtime_backup0.in"
    o = _oracle_state(oracle, p, 4, path)
    recs = read_records(path)
    assert [len(r) for r in recs] == record_sizes(64, 64, 32)
    (t,) = struct.unpack("<d", recs[0])
    assert t == o.scalars().time
    assert struct.unpack("<d", recs[1])[0] == 123.0
    assert struct.unpack("<i", recs[3])[0] == 32
    NN = 64 * 64
    n1 = struct.unpack_from("<i", recs[2], 0)[0]
    vortk = np.frombuffer(recs[2], dtype="<f8", count=2 * NN, offset=12).reshape(2, 64, 64)
    assert np.array_equal(vortk[1 - n1], o.vortk())
    beam = np.frombuffer(recs[5], dtype="<f8").reshape(6, 32)
    assert np.array_equal(beam[0], o.beam()[0][0])
    o.close()


def test_write_resume_write(oracle, tmp_path):
    """Every record survives a resume except the mask, which init_fields' caller draws anew
    from the beam at the backup's time (time_step.f90:82)."""
    p = make_params(nx=64, ny=64, ns=32)
    a, b = tmp_path / "a.in", tmp_path / "b.in"
    o = _oracle_state(oracle, p, 5, a)
    r = oracle.OracleRun(p)
    r.resume(a)
    r.MakeRuntimeBackup(b)
    ra, rb = read_records(a), read_records(b)
    NN = 64 * 64
    mask_lo, mask_hi = 12 + 8 * 6 * NN, 12 + 8 * 9 * NN
    assert ra[2][:mask_lo] == rb[2][:mask_lo] and ra[2][mask_hi:] == rb[2][mask_hi:]
    for i in range(len(ra)):
        if i != 2:
            assert ra[i] == rb[i], i
    # the resumed run steps on (an AB2 step, a Crank-Nicolson solid step)
    rows = r.time_step(3)
    assert np.all(np.isfinite(rows)) and r.scalars().status == 0
    assert r.scalars().time > o.scalars().time
    o.close(); r.close()


def test_resume_refusals(oracle, tmp_path):
    p = make_params(nx=64, ny=64, ns=32)
    path = tmp_path / "a.in"
    _oracle_state(oracle, p, 2, path).close()
    with pytest.raises(Exception):
        oracle.OracleRun(make_params(nx=64, ny=64, ns=48)).resume(path)
    data = bytearray(path.read_bytes())
    struct.pack_into("<d", data, 8 + 8 + 4, 124.0)  # the checksum record's payload
    bad = tmp_path / "bad.in"
    bad.write_bytes(bytes(data))
    with pytest.raises(Exception):
        oracle.OracleRun(p).resume(bad)
    with pytest.raises(Exception):
        oracle.OracleRun(p).resume(tmp_path / "missing.in")


def test_alternating_files_and_latest(oracle, tmp_path):
    """MakeRuntimeBackup alternates between runtime_backup0.in and runtime_backup1.in;
    inicond = 2 resumes from the later of the two (init_fields.f90:44-92)."""
    from fsibe_2d_gb300 import backup_time
    p = make_params(nx=64, ny=64, ns=32)
    with pytest.raises(FileNotFoundError):
        oracle.OracleRun(p).resume_latest(tmp_path)
    o = oracle.OracleRun(p)
    o.init_fields(seeded_vorticity(64, seed=3))
    o.time_step(2)
    nb = o.make_runtime_backup(tmp_path, 0)
    assert nb == 1
    t0 = o.scalars().time
    o.time_step(2)
    assert o.make_runtime_backup(tmp_path, nb) == 0
    t1 = o.scalars().time
    assert backup_time(tmp_path / "runtime_backup0.in") == t0
    assert backup_time(tmp_path / "runtime_backup1.in") == t1 > t0
    r = oracle.OracleRun(p)
    assert r.resume_latest(tmp_path).endswith("runtime_backup1.in")
    assert r.scalars().time == t1
    assert np.array_equal(r.vortk(), o.vortk())
    # the older file wins once it is rewritten later
    o.time_step(1)
    o.make_runtime_backup(tmp_path, 0)
    assert r.resume_latest(tmp_path).endswith("runtime_backup0.in")
    o.close(); r.close()
