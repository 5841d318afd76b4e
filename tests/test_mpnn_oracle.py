"""The learned preconditioner's CPU definition (oracle/mpnn_ref.py) checked
on its own: analytic gradients against central finite differences, the
block-Jacobi limit (zero decoder), positive homogeneity, and Adam."""
import numpy as np

import mpnn_ref as M


def _graph(seed=0, nj=14, neq=None):
    rng = np.random.default_rng(seed)
    node_eq = np.arange(nj * 6).reshape(nj, 6)
    node_eq[rng.random((nj, 6)) < 0.15] = -1          # fixed DOFs
    free = node_eq >= 0
    node_eq[free] = np.arange(free.sum())
    pairs = [(i, (i + 1) % nj) for i in range(nj)] + [(i, (i + 5) % nj) for i in range(0, nj, 2)]
    return M.Graph.from_jcode(np.concatenate([node_eq + 1, np.zeros((nj, 1), int)], 1), pairs, free.sum())


def test_gradient_matches_finite_differences():
    g = _graph()
    rng = np.random.default_rng(1)
    theta = (rng.standard_normal(M.n_params()) * 0.2).astype(np.float64)
    b, t, p = (rng.standard_normal(g.neq) for _ in range(3))
    L, grad = M.loss_and_grad(theta, g, b, t, p)
    assert np.isfinite(L)
    idx = rng.choice(M.n_params(), 60, replace=False)
    # every parameter block is probed at least once
    starts = np.cumsum([0] + [int(np.prod(s)) for _, s in M.layout()])[:-1]
    idx = np.unique(np.concatenate([idx, starts]))
    eps = 1e-6
    for k in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[k] += eps
        tm[k] -= eps
        fd = (M.loss_and_grad(tp, g, b, t, p)[0] - M.loss_and_grad(tm, g, b, t, p)[0]) / (2 * eps)
        assert abs(fd - grad[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, grad[k])


def test_zero_decoder_is_block_jacobi_and_scaling():
    g = _graph(2)
    rng = np.random.default_rng(3)
    theta = M.init_params(5).astype(np.float64)
    P = M.unpack(theta)
    P["Wd"][:] = 0
    r, p = rng.standard_normal(g.neq), rng.standard_normal(g.neq)
    z, _ = M.forward(theta, g, r, p)
    np.testing.assert_array_equal(z, p)
    theta = M.init_params(5).astype(np.float64)
    z1, _ = M.forward(theta, g, r, p)
    z2, _ = M.forward(theta, g, 3.5 * r, 3.5 * p)
    np.testing.assert_allclose(z2, 3.5 * z1, rtol=1e-12, atol=1e-12)


def test_adam_step():
    th = np.array([1.0, -2.0])
    g = np.array([0.5, -0.25])
    t1, m, v = M.adam(th, g, np.zeros(2), np.zeros(2), 1, 1e-2)
    # first step moves each parameter by lr against the gradient's sign
    np.testing.assert_allclose(t1, th - 1e-2 * np.sign(g), rtol=1e-6)
    t2, _, _ = M.adam(t1, g, m, v, 2, 1e-2)
    assert np.all(np.abs(t2 - t1) > 0)
