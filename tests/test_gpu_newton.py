"""Static Newton-Raphson (ALGFLAG 1) and modified Newton-Raphson (ALGFLAG 2)
load control on the GPU against the reference's own runs (golden fixtures
made by the reference binary): the same converged load levels and iteration
counts, displacement histories to 1e-6 relative (FP64), and the same ending
(lpf past lpfmax, or the reference's subdivision failure)."""
import numpy as np
import pytest

import cubens

pytestmark = pytest.mark.gpu

CASES = ["truss_nr", "truss_mnr", "panel8_nr", "panel8_mnr"]


def _hist_err(d, ref):
    return np.max(np.abs(d - ref)) / np.max(np.abs(ref))


@pytest.mark.parametrize("name", CASES)
def test_newton_raphson_matches_reference(golden_dir, name):
    z = np.load(golden_dir / f"run_{name}.npz")
    m = cubens.Model(str(z["model_def"]), precision=cubens.FP64)
    assert m.info["algflag"] == (1 if name.endswith("_nr") else 2)
    r = m.run_newton(len(z["lam"]))
    np.testing.assert_array_equal(r["its"], z["iterations"])
    np.testing.assert_allclose(r["lam"], z["lam"], rtol=1e-14)
    assert _hist_err(r["d"], z["d"]) < 1e-6
    tail = str(z["results_tail"])
    if "Solution successful" in tail:
        assert m.newton_step().done
    else:
        with pytest.raises(cubens.CubensError) as e:
            m.newton_step()
        assert e.value.code == 6


@pytest.mark.parametrize("name", ["truss_mnr", "truss_nr"])
def test_newton_raphson_mixed_precision_tracks_reference(golden_dir, name):
    """FP32 tangent and factor, FP64 residual: the same load levels, the
    displacement history to the mixed tolerance."""
    z = np.load(golden_dir / f"run_{name}.npz")
    r = cubens.Model(str(z["model_def"]), precision=cubens.MIXED).run_newton(len(z["lam"]))
    np.testing.assert_allclose(r["lam"], z["lam"], rtol=1e-14)
    assert _hist_err(r["d"], z["d"]) < 1e-5


def test_newton_call_order(golden_dir):
    z = np.load(golden_dir / "run_truss_nr.npz")
    m = cubens.Model(str(z["model_def"]))
    with pytest.raises(cubens.CubensError) as e:
        m.newton_step()
    assert e.value.code == 7
    with pytest.raises(cubens.CubensError) as e:
        m.begin()  # an MSAL call on a Newton-Raphson model
    assert e.value.code == 7


def test_frame_newton_raphson_is_self_consistent():
    """Frames: the reference's own static loop gives NaN displacements on
    these buildings (a non-positive pivot reported, then a solve on the
    partly factored matrix), so the GPU path is checked on its own: every
    converged increment in equilibrium, and full and modified Newton-Raphson
    at the same load levels agree."""
    from cubens import models
    N = models.NewtonControls
    runs = []
    for alg in (1, 2):
        spec = models.frame_building(2, 2, 3, msal=N(alg=alg, lpfmax=4e6, lpf=5e5, dlpf=5e5, dlpfmax=2e6,
                                                     dlpfmin=3e4, itemax=60, toldisp=1e-10, tolener=1e-12))
        runs.append(cubens.Model(spec.text).run_newton(20))
    nr, mnr = runs
    assert len(nr["lam"]) >= 3
    np.testing.assert_allclose(mnr["lam"], nr["lam"], rtol=1e-14)
    assert np.all(nr["res"] < 1e-9) and np.all(mnr["res"] < 1e-9)
    assert _hist_err(mnr["d"], nr["d"]) < 1e-7
    assert np.all(nr["its"] <= mnr["its"])
