"""NumPy restatement of the learned-start network (blqh_gb300/csrc/mlp.cu).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the CUDA
forward and backward passes -- never by the product package. The reference has
no such network (its Lanczos start is random, Vec::init_random,
matrix.cpp:54-75), so this oracle is pinned by finite differences of its own
loss (tests/test_mlp_oracle.py) instead of by reference outputs.

It rounds to BF16 at the same points as the CUDA kernels (inputs, weight
copies, each layer's tanh activation, each back-propagated pre-activation
gradient) and accumulates in float64 where the kernels accumulate in FP32, so
the two agree to BF16 rounding of the stored tensors.
"""
from __future__ import annotations

import numpy as np


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    x = np.ascontiguousarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    return ((u + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


def layout(n_bits, width):
    k0 = (n_bits + 2 + 31) // 32 * 32
    sizes = [("Wt0", (width, k0)), ("b0", (width,)), ("Wt1", (width, width)), ("b1", (width,)),
             ("Wt2", (width, width)), ("b2", (width,)), ("w3", (width,)), ("b3", (1,))]
    out, o = {}, 0
    for name, shp in sizes:
        n = int(np.prod(shp))
        out[name] = (o, shp)
        o += n
    return out, o, k0


def unpack(w, n_bits, width):
    lay, n, _ = layout(n_bits, width)
    assert w.size == n
    return {k: np.asarray(w[o:o + int(np.prod(s))], np.float64).reshape(s) for k, (o, s) in lay.items()}


def features(ids, n_bits, d, dsas, k0):
    ids = np.asarray(ids, np.uint64)
    x = np.zeros((len(ids), k0), np.float32)
    for b in range(n_bits):
        x[:, b] = np.where((ids >> np.uint64(b)) & np.uint64(1), 1.0, -1.0)
    x[:, n_bits] = np.float32(d / 3.0)
    x[:, n_bits + 1] = np.float32(dsas * 10.0)
    return bf16(x).astype(np.float64)


def forward(P, x):
    a = [x]
    for l in range(3):
        z = a[-1] @ bf16(P[f"Wt{l}"]).astype(np.float64).T + P[f"b{l}"]
        a.append(bf16(np.tanh(z)).astype(np.float64))
    out = a[3] @ P["w3"] + P["b3"][0]
    return out, a


def loss_grad(w, n_bits, width, ids, conds, targets):
    """Mean over points of 1 - <p,t>^2 / (<p,p><t,t>) and its gradient (flat, float64)."""
    lay, n, k0 = layout(n_bits, width)
    P = unpack(np.asarray(w, np.float32), n_bits, width)
    xs = np.concatenate([features(ids, n_bits, d, s, k0) for d, s in conds])
    out, a = forward(P, xs)
    dim = len(ids)
    npts = len(conds)
    t = np.asarray(targets, np.float64).reshape(npts, dim)
    t = t.astype(np.float32).astype(np.float64)
    g = np.zeros_like(out)
    L = 0.0
    for p in range(npts):
        o, tt = out[p * dim:(p + 1) * dim], t[p]
        s, PP, T = o @ tt, o @ o, tt @ tt
        L += 1 - s * s / (PP * T)
        g[p * dim:(p + 1) * dim] = (-(2 * s / (PP * T)) * tt + (2 * s * s / (PP * PP * T)) * o) / npts
    L /= npts
    grads = {}
    grads["w3"] = a[3].T @ g
    grads["b3"] = np.array([g.sum()])
    dz = bf16((g[:, None] * P["w3"][None, :]) * (1 - a[3] ** 2)).astype(np.float64)
    for l in (2, 1, 0):
        grads[f"Wt{l}"] = dz.T @ a[l]
        grads[f"b{l}"] = dz.sum(0)
        if l > 0:
            dz = bf16((dz @ bf16(P[f"Wt{l}"]).astype(np.float64)) * (1 - a[l] ** 2)).astype(np.float64)
    flat = np.zeros(n)
    for k, (o, s) in lay.items():
        flat[o:o + int(np.prod(s))] = grads[k].ravel()
    return L, flat


def loss_exact(w, n_bits, width, ids, conds, targets):
    """The same loss without any BF16 rounding (float64 throughout): the function
    whose finite differences pin loss_grad's formulas."""
    lay, n, k0 = layout(n_bits, width)
    P = unpack(np.asarray(w, np.float64), n_bits, width)
    L = 0.0
    for (d, s), tt in zip(conds, np.asarray(targets, np.float64).reshape(len(conds), -1)):
        ids = np.asarray(ids, np.uint64)
        x = np.zeros((len(ids), k0))
        for b in range(n_bits):
            x[:, b] = np.where((ids >> np.uint64(b)) & np.uint64(1), 1.0, -1.0)
        x[:, n_bits] = d / 3.0
        x[:, n_bits + 1] = s * 10.0
        a = x
        for l in range(3):
            a = np.tanh(a @ P[f"Wt{l}"].T + P[f"b{l}"])
        o = a @ P["w3"] + P["b3"][0]
        L += 1 - (o @ tt) ** 2 / ((o @ o) * (tt @ tt))
    return L / len(conds)


def grad_exact(w, n_bits, width, ids, conds, targets):
    """Analytic gradient of loss_exact (float64, no rounding)."""
    lay, n, k0 = layout(n_bits, width)
    P = unpack(np.asarray(w, np.float64), n_bits, width)
    ids = np.asarray(ids, np.uint64)
    dim = len(ids)
    xs = []
    for d, s in conds:
        x = np.zeros((dim, k0))
        for b in range(n_bits):
            x[:, b] = np.where((ids >> np.uint64(b)) & np.uint64(1), 1.0, -1.0)
        x[:, n_bits] = d / 3.0
        x[:, n_bits + 1] = s * 10.0
        xs.append(x)
    a = [np.concatenate(xs)]
    for l in range(3):
        a.append(np.tanh(a[-1] @ P[f"Wt{l}"].T + P[f"b{l}"]))
    out = a[3] @ P["w3"] + P["b3"][0]
    npts = len(conds)
    t = np.asarray(targets, np.float64).reshape(npts, dim)
    g = np.zeros_like(out)
    for p in range(npts):
        o, tt = out[p * dim:(p + 1) * dim], t[p]
        s, PP, T = o @ tt, o @ o, tt @ tt
        g[p * dim:(p + 1) * dim] = (-(2 * s / (PP * T)) * tt + (2 * s * s / (PP * PP * T)) * o) / npts
    grads = {"w3": a[3].T @ g, "b3": np.array([g.sum()])}
    dz = (g[:, None] * P["w3"][None, :]) * (1 - a[3] ** 2)
    for l in (2, 1, 0):
        grads[f"Wt{l}"] = dz.T @ a[l]
        grads[f"b{l}"] = dz.sum(0)
        if l > 0:
            dz = (dz @ P[f"Wt{l}"]) * (1 - a[l] ** 2)
    flat = np.zeros(n)
    for k, (o, s) in lay.items():
        flat[o:o + int(np.prod(s))] = grads[k].ravel()
    return flat
