"""Bounded device-side waits: a grid-barrier wait that gives up is reported
as CB_ERR_TIMEOUT and leaves the handle (and the GPU context) usable.

The waits are made to run out on purpose with cb_set_wait_limit(-1): a CTA
that is not the last to arrive at a grid barrier records the timeout at
once and its kernel returns early. Nothing here faults or hangs a GPU.
"""
import numpy as np
import pytest

import cubens
import oracle
from cubens import models

pytestmark = pytest.mark.gpu

TIMEOUT = 8  # CB_ERR_TIMEOUT


def _panel(n=8):
    c = models.MsalControls(joint=n // 2 * (n + 1) + n // 2 + 1, direction=3, dk=-0.2, toldisp=1e-5,
                            tolforc=1.0, tolener=1.0, itemax=100)
    return models.cylindrical_panel(n, controls=c).text


@pytest.mark.parametrize("precision", [cubens.FP64, cubens.MIXED])
def test_factor_and_solve_waits_time_out_then_recover(precision):
    text = _panel()
    m = cubens.Model(text, precision=precision)
    m.set_wait_limit(-1)
    with pytest.raises(cubens.CubensError) as e:
        m.begin()                                  # factor + solves: grid barriers give up
    assert e.value.code == TIMEOUT
    assert "timed out" in str(e.value)
    # the same handle with the default bound, and a fresh handle, run normally
    m.set_wait_limit(0)
    r = m.run(3)
    fresh = cubens.Model(text, precision=precision).run(3)
    o = oracle.OracleModel(text).msal(3)
    for g in (r, fresh):
        assert list(g["its"]) == list(o["its"])
        assert np.max(np.abs(g["lam"] - o["lam"]) / np.abs(o["lam"])) < 1e-5


def test_newmark_direct_solve_wait_times_out():
    f = models.frame_building(2, 2, 3, steps=4, dt=0.005, seed=3)
    m = cubens.Model(f.text)
    m.set_wait_limit(-1)
    m.newmark_begin()
    with pytest.raises(cubens.CubensError) as e:
        m.newmark_step()
    assert e.value.code == TIMEOUT
