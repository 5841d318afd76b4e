"""The CPU oracle against golden vectors produced by the reference's own code.

The fixtures under tests/golden/ were written by tests/golden/make_golden.py
from the reference compiled unmodified (oracle/_ref). These tests pin the
oracle restatement before it is trusted as the checker of the GPU path.
"""
import numpy as np
import pytest

import oracle


def _model(z):
    return oracle.OracleModel(str(z["model_def"]))


@pytest.mark.parametrize("name", ["truss_c1", "panel8", "panel16_imp", "frame_msal"])
def test_msal_path_matches_reference(golden_dir, name):
    z = np.load(golden_dir / f"run_{name}.npz")
    o = _model(z)
    assert o.neq == int(z["neq"])
    steps = len(z["lam"])
    r = o.msal(steps)
    assert r["rc"] == steps, r["error"]
    # the same iteration counts step by step, and the same path
    np.testing.assert_array_equal(r["its"], z["iterations"])
    np.testing.assert_allclose(r["lam"], z["lam"], rtol=1e-10)
    for k in range(steps):
        err = np.linalg.norm(r["d"][k] - z["d"][k]) / np.linalg.norm(z["d"][k])
        assert err < 1e-9, (k, err)


def test_shell_forces_match_reference(golden_dir):
    z = np.load(golden_dir / "elem_shell_panel8.npz")
    o = _model(z)
    c_i, a_i, ef_i, f = o.shell_forces(z["x_after"], z["dd"], z["c_ip"], z["ef_ip"])
    np.testing.assert_allclose(c_i, z["c_i"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(a_i, z["area_i"], rtol=1e-14)
    scale = np.abs(z["ef_i"]).max()
    np.testing.assert_allclose(ef_i, z["ef_i"], rtol=0, atol=1e-12 * scale)
    np.testing.assert_allclose(f, z["f"], rtol=0, atol=1e-12 * np.abs(z["f"]).max())


def test_shell_tangent_and_ldlt_match_reference(golden_dir):
    z = np.load(golden_dir / "elem_shell_panel8.npz")
    o = _model(z)
    E = o.ne_sh
    maxa, ss = o.tangent(z["x_after"], z["c_i"], z["area_i"], np.zeros(0), np.zeros(0), np.zeros(0))
    np.testing.assert_array_equal(maxa, z["maxa"])
    np.testing.assert_allclose(ss, z["ss"], rtol=0, atol=1e-12 * np.abs(z["ss"]).max())
    v, ssd, det, _ = o.skyline_solve(ss, o.q, fact=0)
    assert det == int(z["det"])
    np.testing.assert_allclose(ssd, z["ssd"], rtol=1e-9)
    np.testing.assert_allclose(v, z["ldlt_solution"], rtol=1e-8, atol=1e-12 * np.abs(v).max())
    assert E == 128


def test_truss_forces_and_tangent_match_reference(golden_dir):
    z = np.load(golden_dir / "elem_truss_c1.npz")
    o = _model(z)
    L, dr, ef, f = o.truss_forces(z["x_after"])
    np.testing.assert_allclose(L, z["length_i"], rtol=1e-15)
    np.testing.assert_allclose(dr, z["dir_i"], atol=1e-15)
    np.testing.assert_allclose(ef, z["ef_i"], rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(f, z["f"], rtol=0, atol=1e-12 * np.abs(z["f"]).max())
    maxa, ss = o.tangent(z["x_after"], np.zeros(0), np.zeros(0), L, dr, ef)
    np.testing.assert_array_equal(maxa, z["maxa"])
    np.testing.assert_allclose(ss, z["ss"], rtol=0, atol=1e-12 * np.abs(z["ss"]).max())


@pytest.mark.parametrize("name", ["frame_newmark_fixed", "frame_newmark_member"])
def test_newmark_path_matches_reference(golden_dir, name):
    """Nonlinear Newmark time loop (ALGFLAG 5) on a 2x2-bay, 3-storey frame,
    warping fixed (6 DOF per joint) and one warping DOF per member end."""
    z = np.load(golden_dir / f"run_{name}.npz")
    o = _model(z)
    assert o.neq == int(z["neq"])
    steps = len(z["lam"])
    r = o.newmark(steps)
    assert r["rc"] == steps, r["error"]
    np.testing.assert_array_equal(r["its"], z["iterations"])
    np.testing.assert_array_equal(r["time"], z["lam"])
    np.testing.assert_array_equal(r["d"], z["d"])
    assert np.all(r["res"] < 1e-6)


def test_frame_forces_tangent_mass_match_reference(golden_dir):
    z = np.load(golden_dir / "elem_frame_2x2x3.npz")
    o = _model(z)
    c_i, len_i, ef_i, f = o.frame_forces(z["x_after"], z["dd"], z["c_ip"], z["ef_ip"], z["len_ip"],
                                         z["lref"])
    np.testing.assert_allclose(c_i, z["c_i"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(len_i, z["len_i"], rtol=1e-15)
    np.testing.assert_allclose(ef_i, z["ef_i"], rtol=0, atol=1e-12 * np.abs(z["ef_i"]).max())
    np.testing.assert_allclose(f, z["f"], rtol=0, atol=1e-12 * np.abs(z["f"]).max())
    maxa, ss = o.tangent_fr(z["c_i"], z["ef_i"], z["len_i"], z["lref"])
    np.testing.assert_array_equal(maxa, z["maxa"])
    np.testing.assert_allclose(ss, z["ss"], rtol=0, atol=1e-12 * np.abs(z["ss"]).max())
    sm = o.frame_mass(z["x_after"])
    np.testing.assert_array_equal(sm, z["sm"])


@pytest.mark.parametrize("name", ["frame_linear_fixed", "frame_linear_member", "panel8_linear"])
def test_linear_newmark_path_matches_reference(golden_dir, name):
    """Linear Newmark (ANAFLAG 1, ALGFLAG 4) with HHT-type dissipation: frames
    with initial conditions, and the DKT panel with its lumped shell mass. The
    oracle's displacements per time step equal the reference's bit for bit."""
    z = np.load(golden_dir / f"run_{name}.npz")
    steps = len(z["time"])
    o = oracle.OracleModel(str(z["model_def"])).linear_newmark(steps)
    assert o["rc"] == steps
    np.testing.assert_array_equal(o["time"], z["time"])
    np.testing.assert_array_equal(o["d"], z["d"])
