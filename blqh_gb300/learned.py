"""Learned Lanczos start vectors along a parameter sweep (config of the learned part:
Nphi = 14, 7 + 7, (J, K) = (0, 0), trained at d/l in {0, 0.25, ..., 3.0},
evaluated at the held-out midpoints).

Everything here runs through the library: ground states for training come from
the GPU Lanczos (blqh_ground_state), the network trains with its own CUDA
forward/backward kernels (blqh_mlp_train), and the evaluation runs the GPU
Lanczos from the learned start and from the reference's random start
(std::mt19937 stream, Vec::init_random, matrix.cpp:54-75) on the same sector.
The random start stays the fallback: the learned start is used only when its
overlap with the ground state of the nearest trained point is at least 0.5.
"""
from __future__ import annotations

import numpy as np

from . import VAL_FP64, Basis, Hamiltonian, Lanczos, MLP, ground_state


def training_states(nphi, nel, nup, J, K, ds, delta_sas=0.0, precision=VAL_FP64, ctx=None):
    """Ground states (host, normalized, largest component positive) and energies at each d."""
    psis, es = [], []
    for d in ds:
        r = ground_state(nphi, nel, nup, J, K, d, delta_sas, precision=precision, max_steps=500, tol=1e-13,
                         want_psi=True, ctx=ctx)
        psi = np.asarray(r["psi"], np.float64)
        psi = psi / np.linalg.norm(psi)
        if psi[np.argmax(np.abs(psi))] < 0:
            psi = -psi
        psis.append(psi)
        es.append(r["energy"])
    return np.array(psis), np.array(es)


def iterations_to(alpha, beta, e_exact, tol=1e-9):
    """Smallest m whose m x m Lanczos tridiagonal has its lowest eigenvalue within tol of e_exact."""
    from scipy.linalg import eigvalsh_tridiagonal

    for m in range(1, len(alpha) + 1):
        if m == 1:
            lo = alpha[0]
        else:
            lo = eigvalsh_tridiagonal(alpha[:m], beta[1:m], select="i", select_range=(0, 0))[0]
        if abs(lo - e_exact) < tol:
            return m
    return None


def lanczos_from(H, start, max_steps=400, rng_seed=1):
    """GPU Lanczos (full reorthogonalization) from `start` (None: the reference's
    mt19937 stream); runs to convergence and returns (coefficients, steps, psi)."""
    L = Lanczos(H, max_steps=max_steps, reorth=True, tol=1e-14, check_every=5, seed=rng_seed, rng=0, start=start)
    L.iterate()
    a, b = L.coeffs()
    psi = L.ritz_vector()
    L.close()
    return a, b, psi


def evaluate(mlp, basis, H, d, e_exact, psi_exact, train_ds, train_psis, delta_sas=0.0, tol=1e-9):
    """Learned versus random start at one parameter point."""
    pred = mlp.predict(basis, d, delta_sas)
    near = train_psis[int(np.argmin(np.abs(np.asarray(train_ds) - d)))]
    guard = abs(float(pred @ near))
    use = guard >= 0.5
    a_r, b_r, _ = lanczos_from(H, None)
    it_random = iterations_to(a_r, b_r, e_exact, tol)
    it_learned = it_random
    if use:
        a_l, b_l, _ = lanczos_from(H, pred)
        it_learned = iterations_to(a_l, b_l, e_exact, tol)
    return {"d": d, "overlap_exact": abs(float(pred @ psi_exact)), "overlap_nearest_trained": guard,
            "used_learned": bool(use), "iterations_random": it_random, "iterations_learned": it_learned}


def time_to_egs(nphi, nel, nup, J, K, d, precision, start=None, ctx=None, repeat=2):
    """Wall time of one blqh_ground_state call (basis, CSR, Lanczos to tol 1e-12, Rayleigh
    quotient; best of `repeat`) and its result; start None = the reference's mt19937 start."""
    import time

    best, r = 1e30, None
    for _ in range(repeat):
        t0 = time.perf_counter()
        r = ground_state(nphi, nel, nup, J, K, d, precision=precision, max_steps=500, tol=1e-12, check_every=5,
                         start=start, ctx=ctx)
        best = min(best, time.perf_counter() - t0)
    return best, r


def train_flops(rows, k0, width):
    """Tensor-core flops of one training step (forward, weight and input gradients)."""
    W = width
    return 2.0 * rows * (2 * k0 * W + 6 * W * W + W)


def run(nphi=14, nel=14, nup=7, J=0, K=0, train_ds=None, test_ds=None, steps=600, lr=2e-3, width=256, seed=1,
        ctx=None, timing=False):
    """Train on train_ds, evaluate at test_ds; returns a dict of per-point results.

    timing: also time, at every test point, the plain FP64 path from the random
    start against the mixed-precision path from the learned start (the network's
    inference included), both through blqh_ground_state."""
    import time
    train_ds = list(np.arange(0.0, 3.0001, 0.25)) if train_ds is None else list(train_ds)
    test_ds = list(np.arange(0.125, 3.0, 0.25)) if test_ds is None else list(test_ds)
    basis = Basis(nphi, nel, nup, J, K, ctx=ctx)
    psis, _ = training_states(nphi, nel, nup, J, K, train_ds, ctx=ctx)
    mlp = MLP(2 * nphi, width, seed, ctx=ctx)
    conds = [(d, 0.0) for d in train_ds]
    t0 = time.perf_counter()
    losses = mlp.train(basis, conds, psis, steps=steps, lr=lr)
    t_train = time.perf_counter() - t0
    out = []
    for d in test_ds:
        tpsi, te = training_states(nphi, nel, nup, J, K, [d], ctx=ctx)
        H = Hamiltonian(basis, d)
        p = evaluate(mlp, basis, H, d, te[0], tpsi[0], train_ds, psis)
        H.close()
        if timing:
            from . import VAL_FP32

            t64, r64 = time_to_egs(nphi, nel, nup, J, K, d, VAL_FP64, ctx=ctx)
            t1 = time.perf_counter()
            pred = mlp.predict(basis, d) if p["used_learned"] else None
            t_pred = time.perf_counter() - t1
            t32, r32 = time_to_egs(nphi, nel, nup, J, K, d, VAL_FP32, start=pred, ctx=ctx)
            p.update({"fp64_random_s": t64, "mixed_learned_s": t32 + t_pred, "predict_s": t_pred,
                      "E_fp64": r64["energy"], "E_mixed_learned": r32["energy"],
                      "abs_dE": abs(r64["energy"] - r32["energy"]), "steps_fp64_random": r64["steps"],
                      "steps_mixed_learned": r32["steps"]})
        out.append(p)
    return {"loss_first": float(losses[0]), "loss_last": float(losses[-1]), "train_s": t_train, "steps": steps,
            "points": out, "dim": basis.dim}
