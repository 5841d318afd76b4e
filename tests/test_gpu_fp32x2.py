"""The double-word (FP32x2) band LDL^T against the reference and the FP64 path.

CB_FP32X2 keeps the band as pairs of floats (about 48 significant bits) and
factors and solves it on the FP32 pipe. It carries the conditioning of the
large DKT panels that an FP32 factor cannot, so it is held to the plain FP64
path's tolerances: agreement with the FP64 factor to 1e-10 on one solve, the
reference's iteration counts and 1e-6 on load-displacement paths.
"""
import numpy as np
import pytest

import cubens
import oracle
from cubens import models

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(1e-300, np.max(np.abs(b)))


def test_fp32x2_factor_solve_matches_reference_and_fp64(golden_dir):
    z = np.load(golden_dir / "elem_shell_panel8.npz")
    text = str(z["model_def"])
    q = oracle.OracleModel(text).q
    out = {}
    for prec in (cubens.FP64, cubens.FP32X2):
        m = cubens.Model(text, precision=prec)
        maxa, ss = m.eval_tangent(z["x_after"], z["c_i"], z["area_i"])
        np.testing.assert_array_equal(maxa, z["maxa"])
        assert _rel(ss, z["ss"]) < 1e-12          # the tangent is assembled in FP64 before the split
        v, ssd, det = m.factor_solve(q)
        assert det == int(z["det"])
        assert _rel(ssd, z["ssd"]) < 1e-9
        assert _rel(v, z["ldlt_solution"]) < 1e-8
        out[prec] = (v, ssd)
    assert _rel(out[cubens.FP32X2][0], out[cubens.FP64][0]) < 1e-10
    assert _rel(out[cubens.FP32X2][1], out[cubens.FP64][1]) < 1e-10


@pytest.mark.parametrize("name", ["truss_c1", "panel8", "panel16_imp"])
def test_fp32x2_msal_path_matches_reference(golden_dir, name):
    z = np.load(golden_dir / f"run_{name}.npz")
    steps = len(z["lam"])
    r = cubens.Model(str(z["model_def"]), precision=cubens.FP32X2).run(steps)
    np.testing.assert_array_equal(r["its"], z["iterations"])
    assert _rel(r["lam"], z["lam"]) < 1e-6
    for k in range(steps):
        assert np.linalg.norm(r["d"][k] - z["d"][k]) / np.linalg.norm(z["d"][k]) < 1e-6, k


@pytest.mark.parametrize("n,toldisp", [(32, 1e-4), (64, 1e-5)])
def test_fp32x2_wide_band_panel_matches_oracle(n, toldisp):
    """Bands of 203 and 395 equations: many trailing tiles per panel, the
    look-ahead of the next diagonal block and the multi-CTA solve."""
    c = models.MsalControls(joint=n // 2 * (n + 1) + n // 2 + 1, direction=3, dk=-0.2, toldisp=toldisp,
                            tolforc=1.0, tolener=1.0, itemax=100)
    text = models.cylindrical_panel(n, seed=3, imperfection=0.05, controls=c).text
    steps = 4
    o = oracle.OracleModel(text).msal(steps)
    assert o["rc"] == steps, o["error"]
    g = cubens.Model(text, precision=cubens.FP32X2).run(steps)
    np.testing.assert_array_equal(g["its"], o["its"])
    assert _rel(g["lam"], o["lam"]) < 1e-6
    for k in range(steps):
        assert np.linalg.norm(g["d"][k] - o["d"][k]) / np.linalg.norm(o["d"][k]) < 1e-6, k


def test_fp32x2_newton_raphson_matches_reference(golden_dir):
    z = np.load(golden_dir / "run_panel8_nr.npz")
    r = cubens.Model(str(z["model_def"]), precision=cubens.FP32X2).run_newton(len(z["lam"]))
    np.testing.assert_array_equal(r["its"], z["iterations"])
    assert _rel(r["lam"], z["lam"]) < 1e-6
    assert _rel(r["d"][-1], z["d"][-1]) < 1e-6


def test_fp32x2_is_bit_reproducible(golden_dir):
    z = np.load(golden_dir / "run_panel8.npz")
    a = cubens.Model(str(z["model_def"]), precision=cubens.FP32X2).run(5)
    b = cubens.Model(str(z["model_def"]), precision=cubens.FP32X2).run(5)
    assert np.array_equal(a["d"], b["d"]) and np.array_equal(a["lam"], b["lam"])


def test_fp32x2_refused_for_newmark():
    f = models.frame_building(2, 2, 3, steps=4, dt=0.005, seed=3)
    with pytest.raises(cubens.CubensError) as e:
        cubens.Model(f.text, precision=cubens.FP32X2)
    assert e.value.code == 4


def _bench_controls(n):
    # the controls of the 1.58M-equation benchmark panel (bench.large_text)
    c = models.MsalControls(joint=n // 2 * (n + 1) + n // 2 + 1, direction=3, dk=-0.05, toldisp=1e-5,
                            tolforc=1.0, tolener=1.0, itemax=100)
    return models.cylindrical_panel(n, seed=5, imperfection=0.05, controls=c).text


def test_fp32x2_benchmark_window_matches_oracle():
    """The benchmark's controls and imperfection on a 64 x 64 mesh, over as
    many increments as the benchmark takes (first increment, 3 warm-up and 5
    timed): the oracle's iteration counts, lambda and d to 1e-6 at every one."""
    text = _bench_controls(64)
    steps = 1 + 3 + 5
    o = oracle.OracleModel(text).msal(steps)
    assert o["rc"] == steps, o["error"]
    g = cubens.Model(text, precision=cubens.FP32X2).run(steps)
    np.testing.assert_array_equal(g["its"], o["its"])
    assert _rel(g["lam"], o["lam"]) < 1e-6
    for k in range(steps):
        assert np.linalg.norm(g["d"][k] - o["d"][k]) / np.linalg.norm(o["d"][k]) < 1e-6, k


def test_fp32x2_large_panel_matches_fp64_gpu():
    """The benchmark panel itself (512 x 512, 1,575,936 equations): the
    FP32x2 band against the FP64 band on the first two increments (an FP64
    increment takes about half a minute)."""
    text = _bench_controls(512)
    out = []
    for prec in (cubens.FP64, cubens.FP32X2):
        m = cubens.Model(text, precision=prec, band_solve=1)
        assert m.neq == 1575936
        out.append(m.run(2))
        m.close()
    f64, x2 = out
    np.testing.assert_array_equal(x2["its"], f64["its"])
    assert _rel(x2["lam"], f64["lam"]) < 1e-6
    for k in range(2):
        assert np.linalg.norm(x2["d"][k] - f64["d"][k]) / np.linalg.norm(f64["d"][k]) < 1e-6, k
