"""The paired FP32 form of k_press_x (two adjacent butterflies a thread, 16-byte exchanges;
FSIBE_PX_PAIRED=1 forces it, 0 forbids it) against the oracle and against the one-butterfly
form: the same step within the FP32-compensated tolerance."""
import numpy as np
import pytest

from conftest import rel, seeded_vorticity
from fsibe_2d_gb300 import make_params, FSIBE_FP32C

pytestmark = pytest.mark.gpu


def _run(monkeypatch, paired, p, w, steps):
    import fsibe_2d_gb300 as F
    monkeypatch.setenv("FSIBE_PX_PAIRED", "1" if paired else "0")
    r = F.Run(p)
    monkeypatch.delenv("FSIBE_PX_PAIRED", raising=False)
    assert (r.tile_config()[1][1] == 16) == paired      # the paired kernel's marker
    r.init_fields(w)
    rows = r.time_step(steps)
    return r, rows


@pytest.mark.parametrize("n,ns,steps", [(64, 16, 30), (256, 64, 60), (1024, 256, 40), (512, 128, 30)])
def test_paired_press_x_matches_the_oracle(oracle, monkeypatch, n, ns, steps):
    kw = dict(nx=n, ny=n, ns=ns, Re=500.0, dt=5e-5) if n >= 512 else dict(nx=n, ny=n, ns=ns)
    w = seeded_vorticity(n, seed=4)
    g, rg = _run(monkeypatch, True, make_params(precision=FSIBE_FP32C, **kw), w, steps)
    h, rh = _run(monkeypatch, False, make_params(precision=FSIBE_FP32C, **kw), w, steps)
    o = oracle.OracleRun(make_params(**kw))
    o.init_fields(w)
    ro = o.time_step(steps)
    err = {"vorticity": rel(g.vort(), o.vort()), "u": rel(g.u(), o.u()), "press": rel(g.press(), o.press()),
           "drag": rel(rg[:, 10], ro[:, 10]), "deflection": rel(g.beam()[0][1], o.beam()[0][1])}
    print(f"{n}^2 paired press_x against the oracle:", err,
          "one-butterfly form:", rel(h.vort(), o.vort()), rel(h.press(), o.press()))
    assert max(err.values()) < 1e-5, err
    assert rel(g.vort(), h.vort()) < 1e-5
    g.close(); h.close(); o.close()


@pytest.mark.parametrize("n", [256, 1024])
def test_press_y_engines_match_the_oracle(oracle, monkeypatch, n):
    """k_press_y's two FP32 engines (FSIBE_PY_ENG=0 paired, 1 one butterfly a thread)."""
    import fsibe_2d_gb300 as F
    kw = dict(nx=n, ny=n, ns=n // 4, Re=500.0, dt=5e-5)
    w = seeded_vorticity(n, seed=6)
    o = oracle.OracleRun(make_params(**kw))
    o.init_fields(w)
    o.time_step(20)
    errs = []
    for eng in ("0", "1"):
        monkeypatch.setenv("FSIBE_PY_ENG", eng)
        g = F.Run(make_params(precision=FSIBE_FP32C, **kw))
        monkeypatch.delenv("FSIBE_PY_ENG", raising=False)
        assert g.press_y_engine() == int(eng)
        g.init_fields(w)
        g.time_step(20)
        errs.append(rel(g.press(), o.press()))
        assert rel(g.vort(), o.vort()) < 1e-5
        g.close()
    print(f"{n}^2 press_y engines against the oracle (pressure):", errs)
    assert max(errs) < 1e-5
    o.close()
