"""Checkpoint and restart of the nonlinear Newmark driver (checkPoint and
restartStep, misc.c:494-716): a run restarted from a checkpoint continues
exactly as the uninterrupted run, bit for bit, for the band LDL^T (FP64)
and the FGMRES solver; the loader refuses files of another model, another
format or a truncated one, and leaves the handle unchanged."""
import numpy as np
import pytest

import cubens
from cubens import models

pytestmark = pytest.mark.gpu


def _steps(m, n):
    out = []
    for _ in range(n):
        r = m.newmark_step()
        assert not r.done
        out.append((r.lam, r.iterations, m.displacements()[0].copy()))
    return out


@pytest.mark.parametrize("solver", [cubens.SOLVER_BAND, cubens.SOLVER_FGMRES])
def test_restart_continues_bit_for_bit(tmp_path, solver):
    spec = models.frame_building(3, 2, 4, steps=12, dt=0.005, seed=7)
    kw = dict(precision=cubens.FP64, solver=solver)
    full = cubens.Model(spec.text, **kw)
    full.newmark_begin()
    ref = _steps(full, 8)

    first = cubens.Model(spec.text, **kw)
    first.newmark_begin()
    _steps(first, 4)
    ck = tmp_path / "state.ckpt"
    first.checkpoint_save(ck)
    first.close()

    second = cubens.Model(spec.text, **kw)
    second.newmark_begin()
    second.checkpoint_load(ck)
    rest = _steps(second, 4)
    for (lam, its, d), (lam_r, its_r, d_r) in zip(rest, ref[4:]):
        assert lam == lam_r and its == its_r
        assert np.array_equal(d, d_r)
    u, v, a = second.newmark_state()
    u_r, v_r, a_r = full.newmark_state()
    assert np.array_equal(u, u_r) and np.array_equal(v, v_r) and np.array_equal(a, a_r)


def test_loader_refuses_other_files(tmp_path):
    spec = models.frame_building(3, 2, 4, steps=12, dt=0.005, seed=7)
    other = models.frame_building(2, 2, 4, steps=12, dt=0.005, seed=7)
    a = cubens.Model(spec.text, precision=cubens.FP64)
    a.newmark_begin()
    _steps(a, 2)
    ck = tmp_path / "a.ckpt"
    a.checkpoint_save(ck)

    b = cubens.Model(other.text, precision=cubens.FP64)
    with pytest.raises(cubens.CubensError) as e:  # before newmark_begin
        b.checkpoint_load(ck)
    assert e.value.code == 7
    b.newmark_begin()
    with pytest.raises(cubens.CubensError) as e:  # another model's sizes
        b.checkpoint_load(ck)
    assert e.value.code == 1

    c = cubens.Model(spec.text, precision=cubens.FP64)
    c.newmark_begin()
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(b"not a checkpoint" * 8)
    with pytest.raises(cubens.CubensError) as e:
        c.checkpoint_load(bad)
    assert e.value.code == 2
    cut = tmp_path / "cut.ckpt"
    cut.write_bytes(ck.read_bytes()[:-100])
    with pytest.raises(cubens.CubensError) as e:
        c.checkpoint_load(cut)
    assert e.value.code == 2
    # the refused loads left c at rest: it runs as a fresh handle does
    fresh = cubens.Model(spec.text, precision=cubens.FP64)
    fresh.newmark_begin()
    r1, r2 = _steps(c, 2), _steps(fresh, 2)
    assert all(np.array_equal(x[2], y[2]) for x, y in zip(r1, r2))


def test_checkpoint_needs_newmark(tmp_path):
    text = models.cylindrical_panel(8).text
    m = cubens.Model(text, precision=cubens.FP64)
    with pytest.raises(cubens.CubensError) as e:
        m.checkpoint_save(tmp_path / "x.ckpt")
    assert e.value.code == 4
