"""The fused step launches the next step's advection part of cal_nlk beside its own pressure,
forces and beam (the advection part reads only the fluid state the step has just formed).  The
pipelined run must equal, bit for bit, the run that forms each step's advection part at its
start (FSIBE_ADV_PIPE=0), with the CUDA graph and without, and after the host changes the state
between steps (the next step then forms its own).  (By default the pipeline runs from 2048^2
on; FSIBE_ADV_PIPE=1 forces it here.)"""
import numpy as np
import pytest

from conftest import seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C, FSIBE_FP64

pytestmark = pytest.mark.gpu


def _make(monkeypatch, pipe, p, w, graph):
    import fsibe_2d_gb300 as F
    monkeypatch.setenv("FSIBE_ADV_PIPE", "1" if pipe else "0")
    r = F.Run(p)
    monkeypatch.delenv("FSIBE_ADV_PIPE", raising=False)
    r.init_fields(w)
    r.use_graph(graph)
    return r


@pytest.mark.parametrize("prec,graph", [(FSIBE_FP32C, True), (FSIBE_FP64, True), (FSIBE_FP32C, False)])
def test_pipelined_advection_is_bitwise_the_same(monkeypatch, prec, graph):
    n = 256
    p = make_params(nx=n, ny=n, ns=64, precision=prec)
    w = seeded_vorticity(n, seed=12)
    a, b = _make(monkeypatch, True, p, w, graph), _make(monkeypatch, False, p, w, graph)
    ra, rb = a.time_step(20), b.time_step(20)
    assert np.array_equal(ra, rb)
    # the host changes the state (its own vorticity back): the next step forms its own part
    va = a.vortk(); a.set_vortk(va); b.set_vortk(b.vortk())
    ra, rb = a.time_step(10), b.time_step(10)
    assert np.array_equal(ra, rb)
    assert np.array_equal(a.vortk(), b.vortk()) and np.array_equal(a.u(), b.u())
    assert a.scalars().status == 0
    a.close(); b.close()
