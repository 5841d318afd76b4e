"""cb_solve_noalloc: the solve for callers that cannot allocate GPU memory.

A host application whose own allocator or fixed pool already holds the GPU's
memory, or a loop whose footprint must not change after start-up, cannot
call cudaMalloc where it needs a solve; cb_solve_noalloc runs the same solve
with its work vectors in a static device array. These tests compare it with
the allocating entry point (cb_factor_solve) through the C ABI, on two calls
in a row, for the block solve (arc-length models) and the direct
substitution (Newmark models); they also check its size limit and that a
grid-barrier wait that gives up is reported. This file is collected last so
that a run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import cubens
import oracle
from cubens import models

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the two entry points run the same kernels on the same factor


def _noalloc(lib, m, rhs, torch):
    x = torch.full_like(rhs, float("nan"))
    torch.cuda.synchronize()
    rc = lib.cb_solve_noalloc(m.h, C.c_void_p(rhs.data_ptr()), C.c_void_p(x.data_ptr()))
    return rc, x.cpu().numpy()


def _check_two_calls(lib, m, rhs_np, v_ref, torch):
    rhs = torch.tensor(rhs_np, dtype=torch.float64, device="cuda")
    for call in range(2):                     # two calls in a row share the static scratch
        rc, v = _noalloc(lib, m, rhs, torch)
        assert rc == 0, lib.cb_last_error(m.h)
        err = np.max(np.abs(v - v_ref)) / np.max(np.abs(v_ref))
        assert err <= TOL, (call, err)


@pytest.mark.parametrize("precision", [cubens.FP64, cubens.MIXED])
def test_noalloc_solve_matches_factor_solve(golden_dir, precision):
    torch = pytest.importorskip("torch")
    z = np.load(golden_dir / "elem_shell_panel8.npz")
    text = str(z["model_def"])
    m = cubens.Model(text, precision=precision)
    m.eval_tangent(z["x_after"], z["c_i"], z["area_i"])
    q = oracle.OracleModel(text).q
    v_ref, _, _ = m.factor_solve(q)          # existing entry point (factor + solve)
    _check_two_calls(cubens.load(), m, q, v_ref, torch)


def test_noalloc_direct_substitution_matches_factor_solve(golden_dir):
    """A Newmark model's factor serves one solve: no solve blocks, the
    substitution runs on the band itself."""
    torch = pytest.importorskip("torch")
    text = str(np.load(golden_dir / "run_frame_newmark_fixed.npz")["model_def"])
    m = cubens.Model(text)
    o = oracle.OracleModel(text)
    c0, L0 = o.frame_initial()
    m.eval_frame_tangent(c0, np.zeros(14 * m.ne_fr), L0, L0)
    rhs = np.random.default_rng(7).standard_normal(m.neq)
    v_ref, _, _ = m.factor_solve(rhs)
    _check_two_calls(cubens.load(), m, rhs, v_ref, torch)


def test_noalloc_reports_a_timed_out_wait_and_recovers(golden_dir):
    torch = pytest.importorskip("torch")
    z = np.load(golden_dir / "elem_shell_panel8.npz")
    text = str(z["model_def"])
    m = cubens.Model(text)
    m.eval_tangent(z["x_after"], z["c_i"], z["area_i"])
    q = oracle.OracleModel(text).q
    v_ref, _, _ = m.factor_solve(q)
    lib = cubens.load()
    rhs = torch.tensor(q, dtype=torch.float64, device="cuda")
    m.set_wait_limit(-1)                      # a CTA that is not last gives up at once
    rc, _ = _noalloc(lib, m, rhs, torch)
    assert rc == 8, rc                        # CB_ERR_TIMEOUT
    assert b"timed out" in lib.cb_last_error(m.h)
    m.set_wait_limit(0)                       # the default bound again
    _check_two_calls(lib, m, q, v_ref, torch)


def test_noalloc_rejects_models_beyond_its_limit():
    """541,800 equations with an FP64 factor: more than the 524,288 padded
    equations whose three FP64 work vectors the static array holds."""
    torch = pytest.importorskip("torch")
    spec = models.cylindrical_panel(300)
    m = cubens.Model(spec.text, precision=cubens.FP64, band_solve=1)
    assert m.neq > 524288
    lib = cubens.load()
    rhs = torch.zeros(m.neq, dtype=torch.float64, device="cuda")
    rc, _ = _noalloc(lib, m, rhs, torch)
    assert rc == 9, rc                        # CB_ERR_LIMIT
    assert b"524288" in lib.cb_last_error(m.h)
