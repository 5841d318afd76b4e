"""The learned preconditioner on the GPU.

The network's forward output, loss, parameter gradient and Adam step against
the CPU definition (oracle/mpnn_ref.py, float64); then the network inside
FGMRES in the Newmark driver: trained online on the first time steps, used
afterwards with block-Jacobi as the fallback. FGMRES solves to the same 1e-12
relative residual with either preconditioner, so the Newmark path keeps the
oracle's iteration counts and a 1e-6 relative displacement history; what the
network changes is the Krylov work, which the last test reports.

Tolerances: the dense products run on BF16 tensor cores (operands rounded
to bfloat16, FP32 accumulation) and the CPU definition rounds the same
operands the same way (mpnn_ref.bf16), so what remains is the float32
arithmetic and the accumulation order, plus operands within an ulp of a
bfloat16 rounding tie that the two sides round apart: the output is compared
at 1e-3 of the network's own contribution, the gradient per parameter block
at 5e-3 (relative norm), the Adam step at 1e-6 absolute (learning rate
1e-3). Against the unrounded float64 network the output agrees to a few
1e-2 of its contribution (bfloat16 has 8 significant bits).
"""
import numpy as np
import pytest

import cubens
import mpnn_ref as M
import oracle
from cubens import models

pytestmark = pytest.mark.gpu


def _learned(spec, **kw):
    m = cubens.Model(spec.text, solver=cubens.SOLVER_FGMRES, precond=cubens.PRECOND_LEARNED, **kw)
    jc, _ = m.topology()
    pairs = [(a - 1, b - 1) for a, b in spec.params["members"]]
    return m, M.Graph.from_jcode(jc.reshape(-1, 7), pairs, m.neq)


def test_network_forward_gradient_and_adam_match_the_cpu_definition():
    spec = models.frame_building(2, 2, 2, steps=4, dt=0.005, seed=3)
    m, g = _learned(spec)
    th = M.init_params(11)
    M.unpack(th)["Wd"][:] *= 50  # a decoder large enough to matter
    m.set_mpnn_params(th)
    rng = np.random.default_rng(7)
    r, p, t = rng.standard_normal((3, m.neq))
    z, loss = m.mpnn_eval(r, p, t)
    _, grad = m.mpnn_params()
    t64 = th.astype(np.float64)
    zr, _ = M.forward(t64, g, r, p, bf=True)
    Lr, gr = M.loss_and_grad(t64, g, r, t, p, bf=True)
    assert np.max(np.abs(z - zr)) <= 1e-3 * np.max(np.abs(zr - p))
    assert abs(loss - Lr) <= 1e-4 * Lr
    z64, _ = M.forward(t64, g, r, p)  # the unrounded network
    assert np.max(np.abs(z - z64)) <= 5e-2 * np.max(np.abs(z64 - p))
    o = 0
    for name, shape in M.layout():
        k = int(np.prod(shape))
        ref = gr[o:o + k]
        err = np.linalg.norm(grad[o:o + k] - ref) / max(np.linalg.norm(ref), 1e-30)
        assert err < 5e-3, (name, err)
        o += k
    # one Adam step from the same parameters uses the same gradient
    m.set_mpnn_params(th)
    m.mpnn_eval(r, p, t, train=True)
    th1, _ = m.mpnn_params()
    ref1, _, _ = M.adam(t64, grad.astype(np.float64), np.zeros_like(t64), np.zeros_like(t64), 1, 1e-3)
    assert np.max(np.abs(th1 - ref1)) < 1e-6


def _newmark(spec, steps, learned, train=None):
    if learned:
        m, _ = _learned(spec)
        m.set_learning(train_steps=train, adam_per_solve=8, lr=1e-3, stall_factor=2.0)
    else:
        m = cubens.Model(spec.text, solver=cubens.SOLVER_FGMRES)
    r = m.run_newmark(steps)
    return m, r


def test_learned_preconditioner_keeps_the_newmark_path():
    spec = models.frame_building(4, 3, 6, steps=30, dt=0.005, seed=11)
    ref = oracle.OracleModel(spec.text).newmark(30)
    assert ref["rc"] == 30, ref["error"]
    m, r = _newmark(spec, 30, True, train=12)
    np.testing.assert_array_equal(r["its"], ref["its"])
    assert np.max(np.abs(r["d"] - ref["d"])) / np.max(np.abs(ref["d"])) < 1e-6
    s = m.krylov_stats()
    assert s["train_steps"] > 0 and s["learned_solves"] > 0 and np.isfinite(s["train_loss"])
    assert s["unconverged"] == 0
    # training and application are deterministic
    m2, r2 = _newmark(spec, 30, True, train=12)
    assert np.array_equal(r["d"], r2["d"])
    assert m2.krylov_stats()["iterations"] == s["iterations"]


def test_what_the_network_gains_over_block_jacobi(record_property):
    """Krylov steps per solve after training, learned vs block-Jacobi (the
    same solves to the same tolerance); recorded, and the learned run must
    stay within its stall budget (fallbacks are counted, not hidden)."""
    spec = models.frame_building(4, 3, 6, steps=40, dt=0.005, seed=11)
    bj, _ = _newmark(spec, 40, False)
    ln, _ = _newmark(spec, 40, True, train=20)
    sb, sl = bj.krylov_stats(), ln.krylov_stats()
    record_property("bj_iterations_per_solve", sb["iterations"] / sb["solves"])
    record_property("learned_stats", sl)
    assert sl["learned_solves"] > 0
    assert sl["fallbacks"] <= sl["learned_solves"]
