"""The oracle reproduces the committed golden fixtures (tests/golden/make_golden.py)."""
import os

import numpy as np

from conftest import REPO, rel, seeded_vorticity
from fsibe_2d_gb300 import make_params

G = os.path.join(REPO, "tests", "golden")


def test_fft_fixture(oracle):
    d = np.load(os.path.join(G, "fft_64x32.npz"))
    r = oracle.OracleRun(make_params(nx=64, ny=32, ns=16))
    assert rel(r.coftxy(d["f"]), d["fk"]) < 1e-15
    r.close()


def test_fsi_fixture(oracle):
    d = np.load(os.path.join(G, "fsi_64.npz"))
    assert rel(d["vort"], seeded_vorticity(64)) < 1e-15
    r = oracle.OracleRun(make_params(nx=64, ny=64, ns=16))
    r.init_fields(d["vort"])
    rows = r.time_step(20)
    assert (np.abs(rows - d["rows"]) / (np.abs(d["rows"]).max(axis=0) + 1e-300)).max() < 1e-11
    assert rel(r.vortk(), d["vortk"]) < 1e-12
    assert rel(r.beam()[0], d["beam"]) < 1e-12
    r.close()
