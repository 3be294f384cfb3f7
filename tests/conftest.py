import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def seeded_vorticity(n, K=8, sigma=1e-3, seed=0, ny=None):
    """Seeded N(0, sigma) noise, forward transformed, zeroed where kx^2+ky^2 > K^2 (integer
    mode indices), inverse transformed, no renormalisation (the synthetic inputs of the
    benchmark configurations)."""
    ny = ny or n
    rng = np.random.default_rng(seed)
    w = rng.normal(0.0, sigma, (ny, n))
    wk = np.fft.rfft2(w)
    kx = np.fft.rfftfreq(n, 1.0 / n)
    ky = np.fft.fftfreq(ny, 1.0 / ny)
    wk[(kx[None, :] ** 2 + ky[:, None] ** 2) > K * K] = 0.0
    return np.fft.irfft2(wk, s=(ny, n))


def rel(a, b):
    n = np.linalg.norm(b)
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / (n if n > 0 else 1.0))


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.lib()
    return pyoracle
