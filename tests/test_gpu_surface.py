"""BeamSurfaceIntegral (BeamForces.f90:306-509) through the C ABI against the oracle, at the
reference's call point (after GetForces, before the solid step).  Tolerance: each column within
1e-10 of the largest force column (FP64 plain form; summation orders differ: the device sums
the contour points and the grid in blocks), 1e-5 in the FP32-compensated form."""
import numpy as np
import pytest

from conftest import seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C, FSIBE_FP64

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol,angle", [(FSIBE_FP64, 1e-10, 0.0), (FSIBE_FP64, 1e-10, 20.0), (FSIBE_FP32C, 1e-5, 0.0)])
def test_surface_integral_matches_oracle(oracle, prec, tol, angle):
    import fsibe_2d_gb300 as F
    n, ns = 256, 64
    p = make_params(nx=n, ny=n, ns=ns, precision=prec, angle_beam=angle)
    w = seeded_vorticity(n, seed=9)
    g, o = F.Run(p), oracle.OracleRun(p)
    for r in (g, o):
        r.init_fields(w)
        r.time_step(5)
    outs = []
    for r in (g, o):
        t = r.scalars().time
        r.create_mask(t); r.EvolveFluidAB2(); r.GetForces(t)
        outs.append(r.BeamSurfaceIntegral(t))
    og, oo = outs
    assert og[0] == oo[0]
    scale = np.abs(oo[1:]).max()
    assert np.all(np.isfinite(og)) and scale > 0
    assert np.abs(og[1:] - oo[1:]).max() <= tol * scale, (og, oo)
    g.close(); o.close()
