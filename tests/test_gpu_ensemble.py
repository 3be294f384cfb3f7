"""Ensembles (fsibe_ensemble_*): runs of uneven grid size, beam size and precision advanced
together, one CUDA graph launch per step.  Each run must give exactly what it gives alone:
the ensemble changes only where its kernels are scheduled, not what they compute."""
import numpy as np
import pytest

from conftest import seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C, FSIBE_FP64

pytestmark = pytest.mark.gpu


def _params():
    # uneven sizes (ns = nx/4, as in the batched configuration) and both precision forms
    out = []
    for k, (n, prec, Re) in enumerate([(64, FSIBE_FP64, 150.0), (128, FSIBE_FP32C, 300.0), (128, FSIBE_FP64, 500.0),
                                        (256, FSIBE_FP32C, 800.0), (64, FSIBE_FP32C, 120.0)]):
        out.append(make_params(nx=n, ny=n, ns=n // 4, Re=Re, dt=2e-4, precision=prec,
                               EI=0.05 + 0.1 * k, mu=1.0 + 0.5 * k))
    return out


def test_ensemble_runs_equal_their_single_runs():
    import fsibe_2d_gb300 as F
    ps = _params()
    steps = 12
    ens = F.Ensemble(ps)
    for k, (p, r) in enumerate(zip(ps, ens.runs)):
        r.init_fields(seeded_vorticity(p.nx, seed=10 + k))
    ens.step(steps)
    for k, (p, r) in enumerate(zip(ps, ens.runs)):
        alone = F.Run(p)
        alone.init_fields(seeded_vorticity(p.nx, seed=10 + k))
        for _ in range(steps):
            alone.step()
        assert r.scalars().status == 0
        assert np.array_equal(r.vortk(), alone.vortk()), k
        assert np.array_equal(r.beam()[0], alone.beam()[0]), k
        s1, s2 = r.scalars(), alone.scalars()
        assert s1.time == s2.time and s1.force[0] == s2.force[0], k
        alone.close()
    ens.close()


def test_ensemble_batched_shape_runs():
    """The batched configuration's mix of sizes (scaled down in count): 8 x 256^2, 2 x 512^2,
    1 x 1024^2, FP32-compensated, seeded parameters (Re uniform in [100, 1000], EI
    log-uniform in [0.01, 1], density ratio uniform in [0.5, 5])."""
    import fsibe_2d_gb300 as F
    rng = np.random.default_rng(4)
    ps = []
    for n, count in [(256, 8), (512, 2), (1024, 1)]:
        for _ in range(count):
            ps.append(make_params(nx=n, ny=n, ns=n // 4, precision=FSIBE_FP32C, dt=5e-5,
                                  Re=float(rng.uniform(100, 1000)), EI=float(10 ** rng.uniform(-2, 0)),
                                  mu=float(rng.uniform(0.5, 5))))
    ens = F.Ensemble(ps)
    for k, (p, r) in enumerate(zip(ps, ens.runs)):
        r.init_fields(seeded_vorticity(p.nx, seed=100 + k))
    ens.step(5)
    ms = ens.time_steps(10)
    assert ms > 0
    for r in ens.runs:
        s = r.scalars()
        assert s.status == 0 and np.isfinite(s.force[0])
        assert np.isfinite(r.vort()).all()
    ens.close()
