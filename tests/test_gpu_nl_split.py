"""The fused step forms cal_nlk's right-hand side in two launches: the advection part
(no mask) beside the mask kernels, then the penalization part on the rows of the mask's box
alone (outside the box the mask, and with it the penalization, is zero).  The routine-by-routine
path (create_mask, EvolveFluidAB2, GetForces, SolidSolverWrapper, advance) forms the whole
right-hand side in one launch.  Both give the same state: the split changes no arithmetic,
only which rows carry an exactly-zero penalization term.

The fused step also forms the viscous stresses only on the rows that the forces' stencils can
reach (k_stress_x with the beam's y range); the routine-by-routine path forms them on every
row, so equal forces show that the range covers every stencil."""
import numpy as np
import pytest

from conftest import rel, seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C, FSIBE_FP64

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,angle", [(FSIBE_FP64, 0.0), (FSIBE_FP32C, 0.0), (FSIBE_FP64, 30.0)])
def test_split_nonlinear_term_matches_whole(prec, angle):
    import fsibe_2d_gb300 as F
    n, ns = 256, 64
    p = make_params(nx=n, ny=n, ns=ns, precision=prec, angle_beam=angle)
    w = seeded_vorticity(n, seed=7)
    a, b = F.Run(p), F.Run(p)
    a.init_fields(w); b.init_fields(w)
    a.time_step(5); b.time_step(5)
    for _ in range(6):
        a.step()
        t = b.scalars().time
        b.create_mask(t)
        b.EvolveFluidAB2()
        b.GetForces(t)
        b.SolidSolverWrapper(t)
        b.advance()
    assert rel(a.vortk(), b.vortk()) == 0.0
    ba, bb = a.beam(), b.beam()
    for i in range(len(ba)):
        assert np.array_equal(ba[i], bb[i]), i
    sa, sb = a.scalars(), b.scalars()
    assert sa.status == 0 and sb.status == 0
    assert sa.force[0] == sb.force[0] and sa.force[1] == sb.force[1]
    a.close(); b.close()
