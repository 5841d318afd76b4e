"""GPU frame elements and the nonlinear Newmark driver against the reference.

Element routines against the golden vectors of the reference's own forces_fr,
stiff_fr and mass_fr; whole MSAL and Newmark runs against the reference's
runs; a larger frame against the oracle. Every call goes through the C ABI.

Tolerances: 1e-12 relative for element-level FP64 quantities; 1e-6 relative
on displacement histories of the FP64 path and 1e-5 on the mixed (FP32
tangent and factor) path.
"""
import numpy as np
import pytest

import cubens
import oracle
from cubens import models

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(1e-300, np.max(np.abs(b)))


def _hist_err(d, ref):
    """max over steps of |d_k - ref_k| / max_k |ref_k| (displacement histories
    start from rest, so early steps are compared at the run's scale)."""
    return np.max(np.abs(d - ref)) / np.max(np.abs(ref))


def test_frame_forces_tangent_mass_match_reference(golden_dir):
    z = np.load(golden_dir / "elem_frame_2x2x3.npz")
    m = cubens.Model(str(z["model_def"]))
    assert m.ne_fr == 63
    c_i, len_i, ef_i, f = m.eval_frame_forces(z["x_after"], z["dd"], z["c_ip"], z["ef_ip"], z["len_ip"],
                                              z["lref"])
    assert _rel(c_i, z["c_i"]) < 1e-13
    assert _rel(len_i, z["len_i"]) < 1e-14
    assert _rel(ef_i, z["ef_i"]) < 1e-12
    assert _rel(f, z["f"]) < 1e-12
    maxa, ss = m.eval_frame_tangent(z["c_i"], z["ef_i"], z["len_i"], z["lref"])
    np.testing.assert_array_equal(maxa, z["maxa"])
    assert _rel(ss, z["ss"]) < 1e-12
    sm, L = m.eval_frame_mass(z["x_after"])
    assert _rel(sm, z["sm"]) < 1e-14
    assert _rel(L, z["mass_len"]) < 1e-14


def test_frame_msal_path_matches_reference(golden_dir):
    """The first 16 increments, up to the limit point. Past it the reference's
    own path zig-zags (lambda alternates between two branches) and every
    increment multiplies a perturbation by about 3, so a last-bit difference
    (FMA contraction on the GPU) reaches 1e-8 by increment 25 and changes
    the iteration counts after it; the oracle reproduces all 40 increments
    bit for bit."""
    z = np.load(golden_dir / "run_frame_msal.npz")
    steps = 16
    r = cubens.Model(str(z["model_def"])).run(steps)
    np.testing.assert_array_equal(r["its"], z["iterations"][:steps])
    assert _rel(r["lam"], z["lam"][:steps]) < 1e-6
    for k in range(steps):
        err = np.linalg.norm(r["d"][k] - z["d"][k]) / np.linalg.norm(z["d"][k])
        assert err < 1e-6, (k, err)


@pytest.mark.parametrize("name", ["frame_newmark_fixed", "frame_newmark_member"])
def test_newmark_path_matches_reference(golden_dir, name):
    z = np.load(golden_dir / f"run_{name}.npz")
    steps = len(z["lam"])
    m = cubens.Model(str(z["model_def"]), precision=cubens.FP64)
    assert m.info["algflag"] == 5 and m.info["nsteps"] == steps
    r = m.run_newmark(steps)
    np.testing.assert_array_equal(r["its"], z["iterations"])
    np.testing.assert_allclose(r["time"], z["lam"], rtol=0, atol=1e-15)
    assert _hist_err(r["d"], z["d"]) < 1e-6
    assert np.all(r["res"] < 1e-6)
    # one more call reports the end of the record
    assert m.newmark_step().done


def test_newmark_mixed_precision_tracks_fp64(golden_dir):
    z = np.load(golden_dir / "run_frame_newmark_fixed.npz")
    steps = len(z["lam"])
    r = cubens.Model(str(z["model_def"]), precision=cubens.MIXED).run_newmark(steps)
    assert len(r["time"]) == steps
    assert _hist_err(r["d"], z["d"]) < 1e-5


def test_newmark_larger_frame_matches_oracle():
    spec = models.frame_building(4, 3, 6, steps=24, dt=0.005, seed=11)
    o = oracle.OracleModel(spec.text)
    ref = o.newmark(25)
    assert ref["rc"] == 25, ref["error"]
    m = cubens.Model(spec.text)
    r = m.run_newmark(25)
    np.testing.assert_array_equal(r["its"], ref["its"])
    assert _hist_err(r["d"], ref["d"]) < 1e-6
    u, v, a = m.newmark_state()
    np.testing.assert_array_equal(u, r["d"][-1])
    assert np.all(np.isfinite(v)) and np.all(np.isfinite(a))


def test_newmark_is_bit_reproducible(golden_dir):
    z = np.load(golden_dir / "run_frame_newmark_member.npz")
    a = cubens.Model(str(z["model_def"])).run_newmark(8)
    b = cubens.Model(str(z["model_def"])).run_newmark(8)
    assert np.array_equal(a["d"], b["d"])


def test_newmark_call_order_and_model_kind(golden_dir):
    z = np.load(golden_dir / "run_frame_newmark_fixed.npz")
    m = cubens.Model(str(z["model_def"]))
    with pytest.raises(cubens.CubensError) as e:
        m.newmark_step()
    assert e.value.code == 7
    with pytest.raises(cubens.CubensError) as e:
        m.begin()  # an MSAL call on a Newmark model
    assert e.value.code == 7
    zs = np.load(golden_dir / "run_panel8.npz")
    with pytest.raises(cubens.CubensError) as e:
        cubens.Model(str(zs["model_def"])).newmark_begin()
    assert e.value.code == 7


def test_batched_msal_matches_single_runs():
    """cb_batch_msal runs independent panels of different sizes concurrently;
    every handle's path equals its run alone (and the oracle's)."""
    specs = []
    for i, n in enumerate((8, 16, 24, 8, 16)):
        c = models.MsalControls(joint=n // 2 * (n + 1) + n // 2 + 1, direction=3, dk=-0.2, toldisp=1e-4,
                                tolforc=1.0, tolener=1.0, itemax=100)
        specs.append(models.cylindrical_panel(n, seed=100 + i, imperfection=0.1, controls=c))
    steps = 4
    batch = [cubens.Model(s.text, precision=cubens.MIXED) for s in specs]
    rc, res = cubens.batch_msal(batch, steps, threads=3)
    assert rc == 0
    for s, r in zip(specs, res):
        alone = cubens.Model(s.text, precision=cubens.MIXED).run(steps, with_d=False)
        np.testing.assert_array_equal(r["its"], alone["its"])
        np.testing.assert_array_equal(r["lam"], alone["lam"])
    o = oracle.OracleModel(specs[2].text).msal(steps)
    np.testing.assert_array_equal(res[2]["its"], o["its"])
    assert np.max(np.abs(res[2]["lam"] - o["lam"]) / np.abs(o["lam"])) < 1e-5
