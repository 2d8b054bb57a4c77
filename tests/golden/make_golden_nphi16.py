"""Generates the Nphi=16, Ne=16 (8+8) fixtures in tests/golden/n16/ from the CPU oracle.

The oracle (oracle/blqh_oracle.cpp, a restatement of BLQH_without_spin pinned
bit-exactly to the reference's own outputs up to Nphi=14 by
tests/test_oracle_golden.py) builds the whole sector at the headline
configuration: d/l = 1, Delta_SAS = 0.05, Delta_V = 0, square torus. Per sector
the fixture holds

  * the basis: dimension and SHA-256 digests of `id` (uint64) and `period` (int16);
  * the whole CSR structure: nnz, SHA-256 of row_ptr (int64) and of col (int32),
    and value checksums (sum v, sum |v|, sum v * (col mod 7 + 1));
  * 2000 rows chosen by a seeded stride over the whole row range, in full
    (row index, row length, columns, values);
  * the reference's own method for E_gs (lanczos_hamiltonian.cpp:453-606):
    lambda = 200 steps of the plain three-term recurrence from the std::mt19937
    seed-1 start vector, eigenvalues of the tridiagonal (alpha, beta);
  * an independent FP64 Lanczos with full reorthogonalization over the same
    CSR (numpy), run to a residual below 1e-10: its lowest eigenvalue, the
    ground state's amplitudes at 16384 stride-sampled indices and the residual;
  * wall times of each stage on this machine.

usage: python tests/golden/make_golden_nphi16.py [J K ...]   (default: 0 0  0 1)
Memory: about 20 GB per sector. Time: about 40 minutes per sector on 8 cores.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

NPHI, NEL, NEL_UP = 16, 16, 8
D, DSAS, DV = 1.0, 0.05, 0.0
N_ROWS = 2000
N_AMP = 16384
SEED = 1


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def stride_sample(n: int, k: int, seed: int) -> np.ndarray:
    """k indices spread over [0, n): a seeded offset in [0, n // k), then every n // k."""
    step = n // k
    off = int(np.random.default_rng(seed).integers(step))
    return off + step * np.arange(k, dtype=np.int64)


def reorth_lanczos(spmv, dim, tol=1e-10, max_steps=400):
    """Textbook Lanczos with full (twice-repeated classical) Gram-Schmidt, FP64 complex.

    Returns (E0, psi, residual, steps): psi is the normalized ground Ritz vector and
    residual = ||H psi - E0 psi||."""
    from scipy.linalg import eigh_tridiagonal

    rng = np.random.default_rng(2024)
    v = rng.standard_normal(dim) + 1j * rng.standard_normal(dim)
    v /= np.linalg.norm(v)
    V = np.zeros((max_steps + 1, dim), np.complex128)
    V[0] = v
    a, b = [], []
    for j in range(max_steps):
        w = spmv(V[j])
        a.append(float(np.vdot(V[j], w).real))
        for _ in range(2):
            c = np.conj(V[: j + 1] @ np.conj(w))  # c_i = <v_i, w>
            w -= c @ V[: j + 1]
        bj = float(np.linalg.norm(w))
        m = j + 1
        e, y = eigh_tridiagonal(np.array(a), np.array(b), select="i", select_range=(0, 0))
        if bj * abs(y[-1, 0]) < tol or m == max_steps or bj == 0:
            psi = y[:, 0] @ V[:m]
            psi /= np.linalg.norm(psi)
            r = float(np.linalg.norm(spmv(psi) - e[0] * psi))
            return float(e[0]), psi, r, m
        b.append(bj)
        V[j + 1] = w / bj


def run(J: int, K: int) -> None:
    from scipy.linalg import eigh_tridiagonal

    from oracle import oracle as O

    name = f"n16_j{J}_k{K}_d1"
    t = {}
    t0 = time.time()
    B = O.Basis(NPHI, NEL, NEL_UP, J, K)
    t["basis"] = time.time() - t0
    dim = B.dim
    print(f"{name}: dim {dim}, basis {t['basis']:.1f} s", flush=True)

    t0 = time.time()
    H = O.Hamil(B, D, DSAS, DV)
    t["build"] = time.time() - t0
    nnz = H.nnz
    print(f"{name}: nnz {nnz}, build {t['build']:.1f} s", flush=True)
    rp, col, val = H.row_ptr, H.col, H.val
    is_complex = bool(np.max(np.abs(val.imag)) > 1e-13)

    col32 = col.astype(np.int32)
    w = (col32 % 7 + 1).astype(np.float64)
    checks = np.array([val.sum(), np.abs(val).sum(), (val * w).sum()], np.complex128)

    rows = stride_sample(dim, N_ROWS, seed=16 * J + K)
    lens = (rp[rows + 1] - rp[rows]).astype(np.int32)
    sel = np.concatenate([np.arange(rp[r], rp[r + 1]) for r in rows])
    row_col = col32[sel]
    row_val = val[sel]

    # the reference's method: lambda = 200 plain steps from the seed-1 mt19937 start vector
    t0 = time.time()
    alpha, beta = H.lanczos(200, SEED)
    t["lanczos200"] = time.time() - t0
    ev = eigh_tridiagonal(alpha, beta[1:200], eigvals_only=True)
    print(f"{name}: lambda=200 E0 {ev[0]:.15f}, {t['lanczos200']:.1f} s", flush=True)

    # independent check: full reorthogonalization to a small residual, ground-state amplitudes
    t0 = time.time()
    E0, psi, resid, steps = reorth_lanczos(H.spmv, dim)
    t["reorth_lanczos"] = time.time() - t0
    print(f"{name}: reorth E0 {E0:.15f} ({steps} steps, residual {resid:.2e}), {t['reorth_lanczos']:.1f} s",
          flush=True)
    amp_idx = stride_sample(dim, N_AMP, seed=1000 + 16 * J + K)
    amp = psi[amp_idx]

    out = dict(
        spec=np.array([NPHI, NEL, NEL_UP, J, K, 200, SEED], np.int64),
        params=np.array([D, DSAS, DV], np.float64),
        dim=np.array([dim], np.int64),
        id_sha=np.array(sha(B.id.astype(np.uint64))),
        period_sha=np.array(sha(B.period.astype(np.int16))),
        nnz=np.array([nnz], np.int64),
        row_ptr_sha=np.array(sha(rp.astype(np.int64))),
        col_sha=np.array(sha(col32)),
        val_checks=checks,
        is_complex=np.array([is_complex]),
        rows=rows,
        row_ids=B.id[rows],
        row_len=lens,
        row_col=row_col,
        row_val=row_val if is_complex else row_val.real.copy(),
        alpha=alpha,
        beta=beta,
        eigenvalues=ev,
        E_reorth=np.array([E0]),
        reorth_steps=np.array([steps]),
        reorth_residual=np.array([resid]),
        amp_idx=amp_idx,
        amp=amp,
        meta=np.array(json.dumps({"wall_s": t, "threads": os.cpu_count(), "machine": "x86_64 build container"})),
    )
    os.makedirs(os.path.join(HERE, "n16"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "n16", name + ".npz"), **out)
    print(f"{name}: written", flush=True)


def main(argv):
    pairs = [int(a) for a in argv] or [0, 0, 0, 1]
    for J, K in zip(pairs[::2], pairs[1::2]):
        run(J, K)


if __name__ == "__main__":
    main(sys.argv[1:])
