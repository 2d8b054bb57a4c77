"""Generates the Nphi=14, Ne=14 (7+7) sweep fixtures in tests/golden/c2/ from the reference itself.

Runs oracle/_ref/ref_probe (the reference's BLQH_without_spin sources compiled
out-of-tree by oracle/build_ref.sh) on a seeded subset of the sweep over every
(J, K) sector at d/l in {0.5, 1.0, 1.5}, Delta_SAS = Delta_V = 0, square torus,
lambda = 200, start vector std::mt19937 seed 1: for each K in [0, 14) one J drawn
by a seeded generator, times the three layer distances (42 points). Each
fixture is compact (no per-state arrays): basis digests, the CSR digest in the
format of make_golden.py (SHA-256 of row_ptr and col as int64), value
checksums, the Lanczos coefficients, the tridiagonal's eigenvalues, the
reference's printed Rayleigh quotient and the probe's stage times.

usage: python tests/golden/make_golden_c2.py [name ...]
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PROBE = os.path.join(ROOT, "oracle", "_ref", "ref_probe")
OUT = os.path.join(HERE, "c2")

NPHI, NEL, NEL_UP, LAMBDA, SEED = 14, 14, 7, 200, 1
DS = (0.5, 1.0, 1.5)


def cases():
    rng = np.random.default_rng(14)
    js = rng.integers(0, NPHI, size=NPHI)
    out = {}
    for K in range(NPHI):
        for d in DS:
            out[f"n14_j{int(js[K])}_k{K}_d{str(d).replace('.', '')}"] = (int(js[K]), K, d)
    return out


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run_case(name, J, K, d):
    with tempfile.TemporaryDirectory() as tmp:
        cmd = [PROBE, str(NPHI), str(NEL), str(NEL_UP), str(J), str(K), repr(d), "0.0", "0.0", str(LAMBDA),
               str(SEED), str(os.cpu_count() or 1), tmp, "0"]
        subprocess.run(cmd, check=True)
        meta = {}
        with open(os.path.join(tmp, "meta.txt")) as f:
            for line in f:
                k, v = line.split()
                meta[k] = float(v)

        def rd(n, dt):
            return np.fromfile(os.path.join(tmp, n + ".bin"), dt)

        ids, period = rd("id", np.uint64), rd("period", np.int16)
        row_ptr, col, val = rd("row_ptr", np.int64), rd("col", np.int64), rd("val", np.complex128)
        h = hashlib.sha256()
        h.update(row_ptr.tobytes())
        h.update(col.tobytes())
        w = (col % 7 + 1).astype(np.float64)
        out = dict(
            spec=np.array([NPHI, NEL, NEL_UP, J, K, LAMBDA, SEED], np.int64),
            params=np.array([d, 0.0, 0.0], np.float64),
            dim=np.array([len(ids)], np.int64),
            id_sha=np.array(sha(ids)),
            period_sha=np.array(sha(period)),
            first_ids=ids[:64],
            nnz=np.array([len(col)], np.int64),
            csr_digest=np.array(h.hexdigest()),
            val_checks=np.array([val.sum(), np.abs(val).sum(), (val * w).sum()], np.complex128),
            alpha=rd("alpha", np.float64),
            beta=rd("beta", np.float64),
            eigenvalues=rd("eigenvalues", np.float64),
            E_rq=np.array([meta["E_rq"]]),
            Ec=np.array([meta["Ec"]]),
            meta=np.array(json.dumps(meta)),
        )
    os.makedirs(OUT, exist_ok=True)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **out)
    print(f"{name}: dim={len(ids)} nnz={len(col)} E0={out['eigenvalues'][0]:.12f} "
          f"build={meta['t_build']:.1f}s", flush=True)


def main(argv):
    if not os.path.exists(PROBE):
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    all_cases = cases()
    for n in argv or list(all_cases):
        if not argv and os.path.exists(os.path.join(OUT, n + ".npz")):
            continue
        run_case(n, *all_cases[n])


if __name__ == "__main__":
    main(sys.argv[1:])
