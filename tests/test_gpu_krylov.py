"""FGMRES(m) with nodal block-Jacobi for the nonlinear Newmark driver.

The Krylov solve is checked by what it feeds: whole Newmark runs against the
reference's own runs (golden fixtures) and against the oracle on a larger
frame. Every solve goes to a relative residual of 1e-12, so the full Newton
iteration counts equal the direct solve's and the displacement histories
agree to 1e-6 relative (the FP64 path's tolerance); the mixed mode keeps the
FP64 matrix and stores the preconditioner in FP32, which changes the Krylov
iteration counts, not the solution's tolerance.
"""
import numpy as np
import pytest

import cubens
import oracle
from cubens import models

pytestmark = pytest.mark.gpu


def _hist_err(d, ref):
    return np.max(np.abs(d - ref)) / np.max(np.abs(ref))


def _fgmres(text, **kw):
    return cubens.Model(text, solver=cubens.SOLVER_FGMRES, **kw)


@pytest.mark.parametrize("name", ["frame_newmark_fixed", "frame_newmark_member"])
def test_fgmres_newmark_matches_reference(golden_dir, name):
    z = np.load(golden_dir / f"run_{name}.npz")
    steps = len(z["lam"])
    m = _fgmres(str(z["model_def"]))
    assert m.info["solver"] == cubens.SOLVER_FGMRES and m.info["nnz"] > 0 and m.info["node_blocks"] > 0
    r = m.run_newmark(steps)
    np.testing.assert_array_equal(r["its"], z["iterations"])
    assert _hist_err(r["d"], z["d"]) < 1e-6
    s = m.krylov_stats()
    assert s["solves"] >= int(np.sum(z["iterations"]))
    assert s["unconverged"] == 0
    assert s["last_residual"] <= 1e-12


def test_fgmres_larger_frame_matches_oracle():
    spec = models.frame_building(4, 3, 6, steps=24, dt=0.005, seed=11)
    ref = oracle.OracleModel(spec.text).newmark(25)
    assert ref["rc"] == 25, ref["error"]
    for prec in (cubens.FP64, cubens.MIXED):
        m = _fgmres(spec.text, precision=prec)
        r = m.run_newmark(25)
        np.testing.assert_array_equal(r["its"], ref["its"])
        assert _hist_err(r["d"], ref["d"]) < 1e-6, prec
        s = m.krylov_stats()
        assert s["unconverged"] == 0 and s["iterations"] > s["solves"]


def test_fgmres_restarts_and_iteration_limit():
    """A short restart length forces several restart cycles per solve (the
    true residual is recomputed at each); a tiny step limit ends solves
    unconverged, which the counters report."""
    spec = models.frame_building(3, 2, 4, steps=6, dt=0.005, seed=5)
    ref = oracle.OracleModel(spec.text).newmark(6)
    m = _fgmres(spec.text, restart=4)
    r = m.run_newmark(6)
    np.testing.assert_array_equal(r["its"], ref["its"])
    assert _hist_err(r["d"], ref["d"]) < 1e-6
    s = m.krylov_stats()
    assert s["unconverged"] == 0 and s["iterations"] > 4 * s["solves"]
    m2 = _fgmres(spec.text, restart=4, maxit=2, rtol=1e-12)
    m2.newmark_begin()
    try:
        m2.newmark_step()
    except cubens.CubensError as e:  # Newton may fail to converge on such solves
        assert e.code == 6
    assert m2.krylov_stats()["unconverged"] > 0


def test_fgmres_is_bit_reproducible(golden_dir):
    z = np.load(golden_dir / "run_frame_newmark_member.npz")
    a = _fgmres(str(z["model_def"])).run_newmark(8)
    b = _fgmres(str(z["model_def"])).run_newmark(8)
    assert np.array_equal(a["d"], b["d"])


def test_fgmres_spmv_profile_and_band_entry_points(golden_dir):
    z = np.load(golden_dir / "run_frame_newmark_fixed.npz")
    m = _fgmres(str(z["model_def"]))
    m.newmark_begin()
    m.newmark_step()
    ms, nbytes, flops = m.profile_kernel(cubens.K_SPMV, reps=5)
    assert ms > 0 and nbytes > 12 * m.info["nnz"] and flops == 2 * m.info["nnz"]
    with pytest.raises(cubens.CubensError) as e:
        m.profile_kernel(cubens.K_BAND_LDLT, reps=1)
    assert e.value.code == 4
    with pytest.raises(cubens.CubensError) as e:
        m.factor_solve(np.ones(m.neq))
    assert e.value.code == 4
