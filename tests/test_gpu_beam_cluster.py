"""The two forms of the beam's Newton kernel: the thread-block cluster form (16 or 8 CTAs,
the default on a device that places the cluster) and the single-CTA form
(FSIBE_BEAM_CLUSTER=0).  Both run FP64 Newton with an FP32-preconditioned FP64 iterative
refinement to 2^-30 of the correction; they differ only in the preconditioner's application
(inverse rows against triangular solves), so they agree to refinement rounding, far inside
the 1e-10 bar that both meet against the oracle."""
import numpy as np
import pytest

from conftest import rel, seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C

pytestmark = pytest.mark.gpu


def _run(p, w, steps, monkeypatch, cluster):
    import fsibe_2d_gb300 as F
    if cluster is None:
        monkeypatch.delenv("FSIBE_BEAM_CLUSTER", raising=False)
    else:
        monkeypatch.setenv("FSIBE_BEAM_CLUSTER", str(cluster))
    r = F.Run(p)
    monkeypatch.delenv("FSIBE_BEAM_CLUSTER", raising=False)
    r.init_fields(w)
    rows = r.time_step(steps)
    return r, rows


@pytest.mark.parametrize("n,ns,steps,prec", [(128, 32, 40, 0), (256, 64, 60, 0), (256, 64, 40, FSIBE_FP32C)])
def test_cluster_form_matches_single_cta_form(monkeypatch, n, ns, steps, prec):
    p = make_params(nx=n, ny=n, ns=ns, precision=prec)
    w = seeded_vorticity(n)
    a, ra = _run(p, w, steps, monkeypatch, None)
    s, rs = _run(p, w, steps, monkeypatch, 0)
    assert a.beam_cluster() in (8, 16), "the cluster form does not run on this device"
    assert s.beam_cluster() == 0
    ba, bs = a.beam(), s.beam()
    assert rel(ba[0], bs[0]) < 1e-12
    assert rel(a.vortk(), s.vortk()) < 1e-12
    scale = np.abs(rs).max(axis=0) + 1e-30
    assert (np.abs(ra - rs) / scale).max() < 1e-10
    sa, ss = a.scalars(), s.scalars()
    assert sa.status == 0 and ss.status == 0 and sa.newton_iters == ss.newton_iters
    a.close(); s.close()


@pytest.mark.parametrize("n,ns,steps", [(512, 512, 12), (1024, 1024, 12)])
def test_large_beam_cluster_form_matches_single_cta_form(monkeypatch, n, ns, steps):
    """ns >= 512: the factor and M^-1 exceed a CTA's shared memory; the cluster form keeps them
    in global memory (L2-resident) and must agree with the single-CTA form as at small ns."""
    p = make_params(nx=n, ny=n, ns=ns, Re=500.0, dt=5e-5)
    w = seeded_vorticity(n, seed=1)
    a, ra = _run(p, w, steps, monkeypatch, None)
    s, rs = _run(p, w, steps, monkeypatch, 0)
    assert a.beam_cluster() in (8, 16) and s.beam_cluster() == 0
    assert rel(a.beam()[0], s.beam()[0]) < 1e-12
    assert rel(a.vortk(), s.vortk()) < 1e-12
    # the rows: both forms stop Newton at the 1e-10 tolerance, and at ns = 1024 the rates
    # (theta_dot, the tip velocity: differences over dt) carry that to 2e-10 of their column
    scale = np.abs(rs).max(axis=0) + 1e-12
    assert (np.abs(ra - rs) / scale).max() < 1e-9
    sa, ss = a.scalars(), s.scalars()
    assert sa.status == 0 and ss.status == 0 and sa.newton_iters == ss.newton_iters
    a.close(); s.close()


def test_cluster_sizes_agree(monkeypatch):
    """16 and 8 CTAs split the rows differently; the results agree to refinement rounding."""
    n, ns, steps = 256, 64, 30
    p = make_params(nx=n, ny=n, ns=ns)
    w = seeded_vorticity(n, seed=5)
    a, ra = _run(p, w, steps, monkeypatch, 16)
    b, rb = _run(p, w, steps, monkeypatch, 8)
    assert b.beam_cluster() == 8
    assert rel(a.beam()[0], b.beam()[0]) < 1e-12
    a.close(); b.close()


def test_cluster_form_new_state_refactors(oracle, monkeypatch):
    """An uploaded beam state invalidates the stored inverse; the next steps rebuild it and
    track the oracle from the same state."""
    n, ns = 128, 32
    p = make_params(nx=n, ny=n, ns=ns)
    import fsibe_2d_gb300 as F
    monkeypatch.delenv("FSIBE_BEAM_CLUSTER", raising=False)
    g = F.Run(p)
    o = oracle.OracleRun(p)
    w = seeded_vorticity(n, seed=3)
    g.init_fields(w); o.init_fields(w)
    g.time_step(6); o.time_step(6)
    b, po, pn, to, tn = o.beam()
    b = b.copy(); b[4] += 2e-3 * np.sin(np.linspace(0, 3, ns)); b[4][0] = 0.0
    o.set_beam(b, po, pn, to, tn); g.set_beam(b, po, pn, to, tn)
    g.time_step(10); o.time_step(10)
    assert rel(g.beam()[0], o.beam()[0]) < 1e-10
    assert g.scalars().status == 0
    g.close(); o.close()
