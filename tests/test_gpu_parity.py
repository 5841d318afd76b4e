"""GPU path against the reference: element routines against golden vectors,
whole MSAL paths against the reference's own runs, larger cases against the
oracle. Every call goes through the C ABI (libcubens_gb300.so via ctypes).

Tolerances: 1e-12 relative for element-level FP64 quantities; 1e-6 relative
on load-displacement paths of the plain FP64 path and 1e-5 on the mixed
(FP32 tangent) path, as the specification states.
"""
import numpy as np
import pytest

import cubens
import oracle
from cubens import models

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(1e-300, np.max(np.abs(b)))


def test_shell_forces_match_reference(golden_dir):
    z = np.load(golden_dir / "elem_shell_panel8.npz")
    m = cubens.Model(str(z["model_def"]))
    c_i, a_i, ef_i, _, f = m.eval_forces(z["x_after"], z["dd"], z["c_ip"], z["ef_ip"])
    assert _rel(c_i, z["c_i"]) < 1e-13
    assert _rel(a_i, z["area_i"]) < 1e-13
    assert _rel(ef_i, z["ef_i"]) < 1e-12
    assert _rel(f, z["f"]) < 1e-12


def test_shell_tangent_factor_solve_match_reference(golden_dir):
    z = np.load(golden_dir / "elem_shell_panel8.npz")
    m = cubens.Model(str(z["model_def"]))
    maxa, ss = m.eval_tangent(z["x_after"], z["c_i"], z["area_i"])
    np.testing.assert_array_equal(maxa, z["maxa"])
    assert _rel(ss, z["ss"]) < 1e-12
    v, ssd, det = m.factor_solve(oracle.OracleModel(str(z["model_def"])).q)
    assert det == int(z["det"])
    assert _rel(ssd, z["ssd"]) < 1e-9
    assert _rel(v, z["ldlt_solution"]) < 1e-8


def test_truss_forces_and_tangent_match_reference(golden_dir):
    z = np.load(golden_dir / "elem_truss_c1.npz")
    m = cubens.Model(str(z["model_def"]))
    _, _, _, ef_tr, f = m.eval_forces(z["x_after"], z["dd"])
    assert _rel(ef_tr, z["ef_i"]) < 1e-12
    assert _rel(f, z["f"]) < 1e-12
    maxa, ss = m.eval_tangent(z["x_after"], ef_tr=z["ef_i"])
    np.testing.assert_array_equal(maxa, z["maxa"])
    assert _rel(ss, z["ss"]) < 1e-12


@pytest.mark.parametrize("name", ["truss_c1", "panel8", "panel16_imp"])
def test_msal_path_matches_reference(golden_dir, name):
    z = np.load(golden_dir / f"run_{name}.npz")
    steps = len(z["lam"])
    m = cubens.Model(str(z["model_def"]), precision=cubens.FP64)
    r = m.run(steps)
    np.testing.assert_array_equal(r["its"], z["iterations"])
    assert _rel(r["lam"], z["lam"]) < 1e-6
    for k in range(steps):
        err = np.linalg.norm(r["d"][k] - z["d"][k]) / np.linalg.norm(z["d"][k])
        assert err < 1e-6, (k, err)


def test_msal_is_bit_reproducible(golden_dir):
    z = np.load(golden_dir / "run_panel8.npz")
    a = cubens.Model(str(z["model_def"])).run(6)
    b = cubens.Model(str(z["model_def"])).run(6)
    assert np.array_equal(a["d"], b["d"]) and np.array_equal(a["lam"], b["lam"])


def test_msal_without_graphs_matches_graphs(golden_dir):
    z = np.load(golden_dir / "run_panel8.npz")
    a = cubens.Model(str(z["model_def"]), use_graphs=False).run(4)
    b = cubens.Model(str(z["model_def"]), use_graphs=True).run(4)
    assert np.array_equal(a["d"], b["d"])


def _panel(n, seed=None, imp=0.0, toldisp=1e-5):
    c = cubens.models.MsalControls(joint=n // 2 * (n + 1) + n // 2 + 1, direction=3, dk=-0.2,
                                   toldisp=toldisp, tolforc=1.0, tolener=1.0, itemax=100)
    return cubens.models.cylindrical_panel(n, seed=seed, imperfection=imp, controls=c)


def test_msal_panel32_matches_oracle():
    m = _panel(32, seed=3, imp=0.05, toldisp=1e-4)
    steps = 6
    o = oracle.OracleModel(m.text).msal(steps)
    assert o["rc"] == steps, o["error"]
    g = cubens.Model(m.text).run(steps)
    np.testing.assert_array_equal(g["its"], o["its"])
    assert _rel(g["lam"], o["lam"]) < 1e-6
    assert _rel(g["d"][-1], o["d"][-1]) < 1e-6


def _curve_err(g, o):
    """Largest |lambda - lambda_ref(d_k)| / |lambda_ref| of the run g against
    the oracle curve o, at matched control displacement."""
    k = int(np.argmax(np.abs(o["d"][0])))  # the control DOF carries the largest displacement
    dk_o, lam_o = o["d"][:, k], o["lam"]
    order = np.argsort(dk_o)
    errs = [abs(lam - np.interp(dk, dk_o[order], lam_o[order])) / abs(np.interp(dk, dk_o[order], lam_o[order]))
            for dk, lam in zip(g["d"][:, k], g["lam"]) if dk_o.min() <= dk <= dk_o.max()]
    return max(errs)


def test_mixed_precision_path_tracks_fp64_curve():
    """FP32 tangent and factor on the 16 x 16 panel: the oracle's curve
    lambda(d_k) within 1e-5 and the displacements within 1e-5 at every
    increment (measured: 5e-10 and 2e-7, the same iteration counts)."""
    m = _panel(16)
    steps = 8
    o = oracle.OracleModel(m.text).msal(steps)
    g = cubens.Model(m.text, precision=cubens.MIXED).run(steps)
    assert abs(g["lam"][0] - o["lam"][0]) / abs(o["lam"][0]) < 1e-5
    assert _curve_err(g, o) < 1e-5
    for k in range(steps):
        assert np.linalg.norm(g["d"][k] - o["d"][k]) / np.linalg.norm(o["d"][k]) < 1e-5, k
    assert np.all(g["res"] < 1e-2)


def test_status_codes_and_errors():
    with pytest.raises(cubens.CubensError) as e:
        cubens.Model("2\n1\n0\n1\n2\n1,0,0,0,0\n")
    assert e.value.code in (2, 4)


def test_benchmark_panel64_matches_oracle():
    """The benchmark workload itself (64x64 panel, NEQ 24,960): the FP64 path
    against the oracle for the first increment and four arc-length steps,
    and the mixed path's curve against it (1e-5 on lambda at the same
    control displacement is the mixed path's tolerance)."""
    import bench
    text, _ = bench.panel_text(64)
    steps = 5
    o = oracle.OracleModel(text).msal(steps)
    assert o["rc"] == steps, o["error"]
    g = cubens.Model(text, precision=cubens.FP64).run(steps)
    np.testing.assert_array_equal(g["its"], o["its"])
    assert _rel(g["lam"], o["lam"]) < 1e-6
    for k in range(steps):
        assert np.linalg.norm(g["d"][k] - o["d"][k]) / np.linalg.norm(o["d"][k]) < 1e-6
    mx = cubens.Model(text, precision=cubens.MIXED).run(steps)
    np.testing.assert_array_equal(mx["its"], o["its"])
    assert _rel(mx["lam"], o["lam"]) < 1e-5


def test_mixed_panel64_curve_within_1e5_over_14_increments():
    """The FP32 factor on the 64 x 64 panel keeps the oracle's curve within
    1e-5 (at matched control displacement) for the first 14 increments;
    past them, near the limit point, it departs by up to 2e-4 (measured over
    26 increments), which is why the large-panel benchmark factors in FP32x2
    (tests/test_gpu_fp32x2.py holds that path to 1e-6)."""
    import bench
    text, _ = bench.panel_text(64)
    steps = 14
    o = oracle.OracleModel(text).msal(steps)
    assert o["rc"] == steps, o["error"]
    mx = cubens.Model(text, precision=cubens.MIXED).run(steps)
    assert _curve_err(mx, o) < 1e-5


def test_cluster_factor_matches_grid_factor_and_oracle():
    """The FP32 band LDL^T as one thread-block cluster (the window of the band
    in distributed shared memory) and as the cooperative grid kernel: the
    oracle's iteration counts on the benchmark panel, curves within the mixed
    tolerance, the cluster run reproducible bit for bit, and one factor+solve
    of a small panel against the FP64 factor."""
    import bench
    text, _ = bench.panel_text(64)
    steps = 5
    o = oracle.OracleModel(text).msal(steps)
    cl = cubens.Model(text, precision=cubens.MIXED, factor_kernel=1)
    assert cl.info["factor_cluster"] in (8, 16)
    a = cl.run(steps)
    gr = cubens.Model(text, precision=cubens.MIXED)
    assert gr.info["factor_cluster"] == 0
    b = gr.run(steps)
    for r in (a, b):
        np.testing.assert_array_equal(r["its"], o["its"])
        assert _rel(r["lam"], o["lam"]) < 1e-5
    a2 = cubens.Model(text, precision=cubens.MIXED, factor_kernel=1).run(steps)
    assert np.array_equal(a["d"], a2["d"])


def test_cluster_factor_solve_against_reference(golden_dir):
    """One FP32 factor+solve of the reference's own tangent (skyfact/skysolve
    golden vectors) by the cluster kernel and by the grid kernel: the same
    determinant flag, pivots and solution to FP32 accuracy (norm-wise: the
    drilling pivots, 1e-4 of the others, lose relative digits in FP32 in
    both kernels)."""
    z = np.load(golden_dir / "elem_shell_panel8.npz")
    q = oracle.OracleModel(str(z["model_def"])).q
    out, errs = [], []
    for fk in (1, 0):
        m = cubens.Model(str(z["model_def"]), precision=cubens.MIXED, factor_kernel=fk)
        assert (m.info["factor_cluster"] > 0) == (fk == 1)
        m.eval_tangent(z["x_after"], z["c_i"], z["area_i"])
        v, ssd, det = m.factor_solve(q)
        assert det == int(z["det"])
        errs.append((np.linalg.norm(ssd - z["ssd"]) / np.linalg.norm(z["ssd"]),
                     np.linalg.norm(v - z["ldlt_solution"]) / np.linalg.norm(z["ldlt_solution"])))
        out.append(v)
    for e_ssd, e_v in errs:
        assert e_ssd < 2e-4 and e_v < 1e-3, errs
    assert np.linalg.norm(out[0] - out[1]) / np.linalg.norm(out[1]) < 1e-3, errs
