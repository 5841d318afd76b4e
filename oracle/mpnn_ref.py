"""CPU restatement of the learned preconditioner's network (test
infrastructure: only the tests and the benchmark's CPU legs use it).

The reference has no learned part; this file is the definition the GPU
kernels are checked against (forward outputs, parameter gradients, the Adam
update), in float64 so it also serves finite-difference checks.

Network (a mesh message-passing network on the joint graph):
  inputs   per joint i, 12 features: the residual r and its block-Jacobi
           image p = B^-1 r at the joint's six equations (0 where a DOF is
           fixed), scaled by their root-mean-square over the equations
  encoder  h = relu(W0 x + b0)                                  12 -> 64
  3 layers m_ij = relu(A h_i + B h_j + c)       (edges i-j of the joint graph)
           a_i  = mean_j m_ij                    (0 for a joint without edges)
           h_i <- h_i + relu(U h_i + V a_i + d)
  decoder  y = Wd h + bd                                         64 -> 6
  output   z = p + rms(p) * y at the joint's equations
so P(alpha r) = alpha P(r) for alpha > 0, and with y = 0 the preconditioner
is block-Jacobi itself. The loss of a pair (b, t = K^-1 b) is
|P(b) - t|^2 / |t|^2.

Parameters are one flat float32 vector (row-major out x in matrices):
  W0[64x12] b0[64] | per layer A B [64x64] c[64] U V [64x64] d[64] | Wd[6x64] bd[6]
"""
from __future__ import annotations

import numpy as np

H = 64
F_IN = 12
F_OUT = 6
LAYERS = 3


def layout():
    """(name, shape) of each parameter block, in storage order."""
    out = [("W0", (H, F_IN)), ("b0", (H,))]
    for l in range(LAYERS):
        out += [(f"A{l}", (H, H)), (f"B{l}", (H, H)), (f"c{l}", (H,)), (f"U{l}", (H, H)), (f"V{l}", (H, H)),
                (f"d{l}", (H,))]
    out += [("Wd", (F_OUT, H)), ("bd", (F_OUT,))]
    return out


def n_params() -> int:
    return int(sum(np.prod(s) for _, s in layout()))


def unpack(theta):
    p, o = {}, 0
    for name, shape in layout():
        k = int(np.prod(shape))
        p[name] = theta[o:o + k].reshape(shape)
        o += k
    return p


def init_params(seed: int) -> np.ndarray:
    """He-scaled normal weights from a seeded generator, zero biases, a small
    decoder (the network starts close to block-Jacobi)."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in layout():
        if len(shape) == 1:
            parts.append(np.zeros(shape))
        else:
            fan_in = shape[1]
            scale = np.sqrt(2.0 / fan_in) * (0.01 if name == "Wd" else (0.5 if name[0] in "ABUV" else 1.0))
            parts.append(rng.standard_normal(shape) * scale)
    return np.concatenate([q.ravel() for q in parts]).astype(np.float32)


class Graph:
    """Joint graph of a model: node_eq[NJ, 6] (0-based equations, -1 fixed)
    and the sorted neighbour lists adj_ptr / adj (both directions)."""

    def __init__(self, node_eq, adj_ptr, adj, neq):
        self.node_eq = np.asarray(node_eq, dtype=np.int64)
        self.adj_ptr = np.asarray(adj_ptr, dtype=np.int64)
        self.adj = np.asarray(adj, dtype=np.int64)
        self.neq = int(neq)
        self.n = self.node_eq.shape[0]
        self.deg = np.diff(self.adj_ptr)
        self.src = np.repeat(np.arange(self.n), self.deg)  # edge i -> adj[e]

    @staticmethod
    def from_jcode(jcode, conn_pairs, neq):
        """jcode: (NJ, 7) 1-based equations; conn_pairs: iterable of joint
        pairs that share an element."""
        jc = np.asarray(jcode).reshape(-1, 7)
        node_eq = jc[:, :6] - 1
        nj = jc.shape[0]
        nbr = [set() for _ in range(nj)]
        for a, b in conn_pairs:
            if a != b:
                nbr[a].add(b)
                nbr[b].add(a)
        ptr = np.zeros(nj + 1, dtype=np.int64)
        adj = []
        for i in range(nj):
            s = sorted(nbr[i])
            adj += s
            ptr[i + 1] = len(adj)
        return Graph(node_eq, ptr, np.array(adj, dtype=np.int64), neq)


def _gather(g: Graph, v):
    out = np.zeros((g.n, 6))
    m = g.node_eq >= 0
    out[m] = v[g.node_eq[m]]
    return out


def _rms(v):
    return float(np.sqrt(np.mean(v * v)))


def bf16(x):
    """x rounded as the GPU rounds a float32 operand of its BF16 tensor-core
    products: to float32 first, then to the nearest bfloat16 (ties to even)."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _ident(x):
    return x


def forward(theta, g: Graph, r, p, bf=False):
    """Returns z and the saved activations. With bf, the operands of the
    dense products (not the decoder's) are rounded as the GPU's BF16
    tensor-core layers round them."""
    q = bf16 if bf else _ident
    P = unpack(theta.astype(np.float64))
    sr, sp = _rms(r), _rms(p)
    if sr == 0 or sp == 0:
        return p.copy(), None
    x = np.concatenate([_gather(g, r) / sr, _gather(g, p) / sp], axis=1)
    S = q(x) @ q(P["W0"]).T + P["b0"]
    h = np.maximum(S, 0)
    cache = dict(x=x, S=S, sp=sp, layers=[])
    for l in range(LAYERS):
        Pn = q(h) @ q(P[f"A{l}"]).T
        Qn = q(h) @ q(P[f"B{l}"]).T
        pre = Pn[g.src] + Qn[g.adj] + P[f"c{l}"]
        msg = np.maximum(pre, 0)
        a = np.zeros_like(h)
        np.add.at(a, g.src, msg)
        deg = np.maximum(g.deg, 1)[:, None]
        a = a / deg
        T = q(h) @ q(P[f"U{l}"]).T + q(a) @ q(P[f"V{l}"]).T + P[f"d{l}"]
        cache["layers"].append(dict(h=h, pre=pre, a=a, T=T))
        h = h + np.maximum(T, 0)
    y = h @ P["Wd"].T + P["bd"]
    cache["h_last"] = h
    z = p.copy()
    m = g.node_eq >= 0
    z[g.node_eq[m]] += sp * y[m]
    return z, cache


def loss_and_grad(theta, g: Graph, b, t, p, bf=False):
    """Loss |P(b) - t|^2 / |t|^2 and its gradient (float64); with bf the
    operands of every product the GPU forms on its BF16 tensor cores (dense
    layers forward and backward, weight and bias gradients) are rounded as
    it rounds them."""
    q = bf16 if bf else _ident
    P = unpack(theta.astype(np.float64))
    z, c = forward(theta, g, b, p, bf=bf)
    tt = float(t @ t)
    e = z - t
    L = float(e @ e) / tt
    grads = {k: np.zeros_like(v) for k, v in P.items()}
    if c is None:
        return L, np.zeros(n_params())
    dz = 2 * e / tt
    dy = c["sp"] * _gather(g, dz)
    h = c["h_last"]
    grads["Wd"] = q(dy).T @ q(h)
    grads["bd"] = q(dy).sum(0)
    dh = q(dy) @ q(P["Wd"])
    deg = np.maximum(g.deg, 1)[:, None]
    for l in reversed(range(LAYERS)):
        L_ = c["layers"][l]
        hin, a, T, pre = L_["h"], L_["a"], L_["T"], L_["pre"]
        dT = dh * (T > 0)
        grads[f"U{l}"] = q(dT).T @ q(hin)
        grads[f"V{l}"] = q(dT).T @ q(a)
        grads[f"d{l}"] = q(dT).sum(0)
        da = q(dT) @ q(P[f"V{l}"])
        dh_in = dh + q(dT) @ q(P[f"U{l}"])
        gm = (da / deg)[g.src] * (pre > 0)
        dPn = np.zeros_like(hin)
        np.add.at(dPn, g.src, gm)
        dQn = np.zeros_like(hin)
        np.add.at(dQn, g.adj, gm)
        grads[f"c{l}"] = q(dPn).sum(0) if bf else gm.sum(0)
        grads[f"A{l}"] = q(dPn).T @ q(hin)
        grads[f"B{l}"] = q(dQn).T @ q(hin)
        dh_in += q(dPn) @ q(P[f"A{l}"]) + q(dQn) @ q(P[f"B{l}"])
        dh = dh_in
    dS = dh * (c["S"] > 0)
    grads["W0"] = q(dS).T @ q(c["x"])
    grads["b0"] = q(dS).sum(0)
    flat = np.concatenate([grads[name].ravel() for name, _ in layout()])
    return L, flat


def adam(theta, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (step counts from 1); returns new theta, m, v (float64)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return theta - lr * mh / (np.sqrt(vh) + eps), m, v
