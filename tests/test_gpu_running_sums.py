"""The beam kernels' running sums against the serial FP64 loop, bit for bit.

integrate_position.f90:14-44 sums the beam's position and velocity increments node by node; the
positions decide grid-aligned boxes (mask, drag window), so the GPU keeps the serial roundings.
The kernels add the terms as integers on the grid of the running value's binade (the FP64 sum
within a binade), take the FP64 addition when the value leaves it, and check every step with
the FP64 addition (a row failing the check is formed again by the serial loop).  Here:
beam-like rows at several lengths, rows built to hit ties, cancellations, zeros, subnormals,
huge magnitudes and non-finite terms.  Every result must equal the serial loop's bits, and no
row may fail the check."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def serial(terms):
    out = np.empty_like(terms)
    for q in range(terms.shape[0]):
        s = 0.0
        for k in range(terms.shape[1]):
            out[q, k] = s
            s = s + float(terms[q, k])
    return out


def beam_rows(n, seed, angle=0.1, rate=1e-2):
    rng = np.random.default_rng(seed)
    i = np.arange(n)
    th = angle * np.sin(3 * i / n + seed) + rng.uniform(-1e-3, 1e-3, n)
    td = rate * rng.uniform(-1, 1) * np.cos(5 * i / n + seed)
    ds = 1.0 / n
    cn, sn = np.cos(th), np.sin(th)
    return np.stack([cn * ds, sn * ds, -(td * sn * ds), td * cn * ds])


def same_bits(a, b):
    return np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.parametrize("n", [1, 2, 7, 37, 64, 255, 256, 257, 512, 513, 1000, 1024, 2048])
def test_beam_rows_match_the_serial_loop(n):
    import fsibe_2d_gb300 as F
    for seed in range(6):
        t = beam_rows(n, seed)
        got, nser = F.running_sums(t)
        assert same_bits(got, serial(t)), (n, seed)
        assert nser == 0, (n, seed, nser)


def test_hard_rows_match_the_serial_loop():
    import fsibe_2d_gb300 as F
    rng = np.random.default_rng(3)
    n = 600
    rows = {
        "ties": [1.0] + [2.0 ** -53] * 300 + [3 * 2.0 ** -53] * (n - 301),
        "ties2": [0.5] + [(1 + 2 * int(rng.integers(4))) * 2.0 ** -54 for _ in range(n - 1)],
        "down-ties": [1.0] + [-(2.0 ** -54)] * 200 + [-(3 * 2.0 ** -55)] * 200 + [2.0 ** -53] * (n - 401),
        "cancel": [1.0, -1.0] * (n // 2 - 5) + [1e-300] * 10,
        "subnormal": [5e-324] * (n - 10) + [1e-310] * 10,
        "huge": [1e300] * n,
        "mixed": list(rng.uniform(-1, 1, n) * 10.0 ** rng.uniform(-20, 2, n)),
        "alternating": [(-1) ** i * (1 + i * 1e-3) for i in range(n)],
        "zeros": [0.0, -0.0] * (n // 2),
        "powers": [2.0 ** -(i % 60) for i in range(n)],
        "grow": list(np.geomspace(1e-12, 1.0, n)),
        "shrink": list(-np.geomspace(1.0, 1e-12, n) / 2.0),
    }
    names = list(rows)
    for g in range(0, len(names), 4):
        grp = names[g:g + 4]
        t = np.array([rows[k] for k in grp], dtype=np.float64)
        got, nser = F.running_sums(t)
        assert same_bits(got, serial(t)), grp
        assert nser == 0, (grp, nser)


def test_non_finite_terms():
    import fsibe_2d_gb300 as F
    t = beam_rows(300, 1)
    t[1, 100] = math.inf
    t[2, 50] = math.nan
    t[3, 10] = -math.inf
    t[3, 20] = math.inf
    got, nser = F.running_sums(t)
    ref = serial(t)
    assert nser == 0
    for q in range(4):
        fin = np.isfinite(ref[q])
        assert same_bits(got[q][fin], ref[q][fin])
        assert np.array_equal(np.isnan(got[q]), np.isnan(ref[q]))
        assert np.array_equal(np.isinf(got[q]), np.isinf(ref[q]))


def test_lengths_outside_the_range_are_rejected():
    import fsibe_2d_gb300 as F
    with pytest.raises(RuntimeError):
        F.running_sums(np.zeros((4, 0)))
