"""The arc-length driver (ALGFLAG 3) on FGMRES with nodal block-Jacobi.

The reference's arc-length loop reads two things from its factorisation: the
sign of det (the predictor's direction, main.c's skyfact call) and the pivots
ssd (psi = min |ssd / ssd_o| against psi_thresh picks the constraint). An
iterative solver has no factor, so the Krylov path substitutes:
  det   K is taken as indefinite when q . K^-1 q <= 0 (the sign of the
        current stiffness parameter; it flips where the load path passes a
        limit point, the crossing skyfact's det reports)
  ssd   the LDL^T pivots of the joints' diagonal blocks of K
Every solve runs to a relative residual of 1e-12, so on the reference's own
runs the path keeps the iteration counts and agrees to 1e-6 relative (the
FP64 path's tolerance).
"""
import numpy as np
import pytest

import cubens
import oracle
from cubens import models

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(1e-300, np.max(np.abs(b)))


def _fgmres(text, **kw):
    return cubens.Model(text, solver=cubens.SOLVER_FGMRES, **kw)


def _check_path(r, z, steps, tol):
    np.testing.assert_array_equal(r["its"], z["iterations"][:steps])
    assert _rel(r["lam"], z["lam"][:steps]) < tol
    for k in range(steps):
        err = np.linalg.norm(r["d"][k] - z["d"][k]) / np.linalg.norm(z["d"][k])
        assert err < tol, (k, err)


# (fixture, increments, FGMRES restart length). The DKT panel's tangent is
# ill-conditioned for nodal block-Jacobi (bending: the scaled condition
# number grows as n^4), so its solves take over a thousand Arnoldi steps and
# the longest restart (64) keeps every one within the iteration limit. The frame run
# approaches a limit point: at its 14th increment the reference's psi (the
# smallest ratio of the factor's pivots to the first ones) falls below
# psi_thresh 0.1 and the constraint drops its load term, while the ratio of
# the joint blocks' pivots stays above it. From there the two runs follow the
# same equilibrium curve with different increments, so the frame is checked
# over its first 13.
CASES = [("truss_c1", 50, 50), ("panel16_imp", 8, 64), ("frame_msal", 13, 50)]


@pytest.mark.parametrize("name,steps,restart", CASES)
def test_krylov_msal_matches_reference(golden_dir, name, steps, restart):
    z = np.load(golden_dir / f"run_{name}.npz")
    m = _fgmres(str(z["model_def"]), restart=restart)
    assert m.info["solver"] == cubens.SOLVER_FGMRES
    _check_path(m.run(steps), z, steps, 1e-6)
    s = m.krylov_stats()
    assert s["unconverged"] == 0 and s["last_residual"] <= 1e-12


def test_krylov_msal_mixed_matches_reference(golden_dir):
    """FP32 preconditioner with nested FP32 FGMRES inside the FP64 one: the
    solves still reach 1e-12, the path stays within the mixed tolerance."""
    z = np.load(golden_dir / "run_truss_c1.npz")
    m = _fgmres(str(z["model_def"]), precision=cubens.MIXED)
    _check_path(m.run(50), z, 50, 1e-5)
    assert m.krylov_stats()["unconverged"] == 0


def test_krylov_msal_is_bit_reproducible(golden_dir):
    z = np.load(golden_dir / "run_truss_c1.npz")
    a = _fgmres(str(z["model_def"])).run(20)
    b = _fgmres(str(z["model_def"])).run(20)
    assert np.array_equal(a["d"], b["d"]) and np.array_equal(a["lam"], b["lam"])
