"""Linear Newmark (ANAFLAG 1, ALGFLAG 4) on the GPU against the reference's
own runs: the stiffness of the initial state and the lumped mass, the
effective stiffness factored once in FP64, then per time step one solve and
the kinematics (main.c:3143-3302, solve.c:139-222 and 246-467). The runs use
numopt 1 (HHT-type dissipation, so the K u_m term of the effective load is
active): frames with initial conditions, warping fixed and one warping DOF
per member end, and the DKT panel with its lumped shell mass (mass_sh,
shell.c:1505-1592) under a pulse at its centre. The path is linear and FP64, so the displacement history agrees to
1e-10 relative (the band LDL^T and the reference's skyline LDL^T sum in
different orders)."""
import numpy as np
import pytest

import cubens

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["frame_linear_fixed", "frame_linear_member", "panel8_linear"])
def test_linear_newmark_matches_reference(golden_dir, name, tmp_path):
    z = np.load(golden_dir / f"run_{name}.npz")
    steps = len(z["time"])
    m = cubens.Model(str(z["model_def"]))
    assert m.info["algflag"] == 4 and m.info["nsteps"] == steps
    m.results_open(tmp_path)
    r = m.run_newmark(steps)
    np.testing.assert_allclose(r["time"], z["time"], rtol=0, atol=1e-15)
    err = np.max(np.abs(r["d"] - z["d"])) / np.max(np.abs(z["d"]))
    assert err < 1e-10, err
    assert m.newmark_step().done          # the end of the record
    m.results_close()
    assert (tmp_path / "results1.txt").read_text().endswith("\nSolution successful!!\n")
