"""Regenerates the golden fixtures in this directory from the CPU oracle (oracle/).

    python tests/golden/make_golden.py

fft_64x32.npz   seeded field and its packed coefficients (coftxy)
fsi_64.npz      64^2, ns=16 FSI run: seeded vorticity, 20 beam_data rows, final vortk and beam
c1_256.npz      the plain-form configuration (256^2, ns=64, Re=100, dt=2e-4, EI=0.1, mu=1):
                beam_data rows of the first 100 steps and the final vorticity's norm/samples
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [REPO, os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")]

from conftest import seeded_vorticity  # noqa: E402
from fsibe_2d_gb300 import make_params  # noqa: E402
import pyoracle  # noqa: E402


def main():
    p = make_params(nx=64, ny=32, ns=16)
    r = pyoracle.OracleRun(p)
    f = np.random.default_rng(42).standard_normal((32, 64))
    np.savez_compressed(os.path.join(HERE, "fft_64x32.npz"), f=f, fk=r.coftxy(f))
    r.close()

    p = make_params(nx=64, ny=64, ns=16)
    r = pyoracle.OracleRun(p)
    w = seeded_vorticity(64)
    r.init_fields(w)
    rows = r.time_step(20)
    np.savez_compressed(os.path.join(HERE, "fsi_64.npz"), vort=w, rows=rows, vortk=r.vortk(), beam=r.beam()[0])
    r.close()

    p = make_params(nx=256, ny=256, ns=64)
    r = pyoracle.OracleRun(p)
    w = seeded_vorticity(256)
    r.init_fields(w)
    rows = r.time_step(100)
    v = r.vort()
    np.savez_compressed(os.path.join(HERE, "c1_256.npz"), rows=rows, vort_norm=np.linalg.norm(v),
                        vort_samples=v[::37, ::41])
    r.close()


if __name__ == "__main__":
    main()
