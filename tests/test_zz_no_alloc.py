"""cb_solve_noalloc: the solve for callers that cannot allocate GPU memory.

Callers running under CUDA-graph capture, inside another allocator's pool or
in a fixed-footprint loop cannot call cudaMalloc; cb_solve_noalloc runs the
same solve with its work vectors in a static device array. This file is
collected last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

import cubens
import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [cubens.FP64, cubens.MIXED])
def test_noalloc_solve_matches_factor_solve(golden_dir, precision):
    torch = pytest.importorskip("torch")
    z = np.load(golden_dir / "elem_shell_panel8.npz")
    text = str(z["model_def"])
    m = cubens.Model(text, precision=precision)
    m.eval_tangent(z["x_after"], z["c_i"], z["area_i"])
    q = oracle.OracleModel(text).q
    v_ref, _, _ = m.factor_solve(q)          # existing entry point (factor + solve)
    rhs = torch.tensor(q, dtype=torch.float64, device="cuda")
    lib = cubens.load()
    for call in range(2):                     # two calls in a row share the static scratch
        x = torch.full_like(rhs, float("nan"))
        torch.cuda.synchronize()
        rc = lib.cb_solve_noalloc(m.h, C.c_void_p(rhs.data_ptr()), C.c_void_p(x.data_ptr()))
        assert rc == 0, lib.cb_last_error(m.h)
        v = x.cpu().numpy()
        err = np.max(np.abs(v - v_ref)) / np.max(np.abs(v_ref))
        assert err <= 1e-12, (call, err)
