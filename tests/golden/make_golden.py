"""Generates the golden fixtures in tests/golden/ from the reference itself.

Runs oracle/_ref/ref_probe (the reference's own sources compiled out-of-tree
by oracle/build_ref.sh) on a fixed list of sectors and stores what it prints
as compressed .npz files. Only this script reads the reference; the fixtures
are committed so that tests need neither the reference nor its build.

usage: python tests/golden/make_golden.py [case-name ...]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PROBE = os.path.join(ROOT, "oracle", "_ref", "ref_probe")

# name: (nphi, nel, nel_up, J, K, d, dsas, dv, lambda, seed, dense, full_csr)
CASES = {
    # README.md:58-76 and 85-103 (the reference's published transcripts)
    "readme_d0": (8, 8, 4, 4, 4, 0.0, 0.0, 0.0, 200, 1, 1, 1),
    "readme_d3": (8, 8, 4, 4, 4, 3.0, 0.0, 0.0, 200, 1, 1, 1),
    # complex sector, bias on, tunnelling requested (a no-op with a fixed split)
    "n8_j0_k1_d1": (8, 8, 4, 0, 1, 1.0, 0.0, 0.0, 200, 1, 1, 1),
    "n8_j0_k0_bias": (8, 8, 4, 0, 0, 1.0, 0.05, 0.1, 200, 1, 1, 1),
    "n8_j2_k3_d05": (8, 8, 4, 2, 3, 0.5, 0.0, 0.0, 200, 1, 1, 1),
    "n8_j4_k0_uneven": (8, 8, 3, 4, 0, 1.0, 0.0, 0.0, 200, 1, 1, 1),
    "n10_j5_k5_d1": (10, 10, 5, 5, 5, 1.0, 0.0, 0.0, 200, 1, 1, 1),
    "n10_j0_k3_d15": (10, 10, 5, 0, 3, 1.5, 0.0, 0.0, 200, 1, 0, 1),
    # free layer split (nel_up < 0): tunnelling acts
    "n6_all_j0_k0_sas": (6, 6, -1, 0, 0, 1.0, 0.1, 0.0, 200, 1, 1, 1),
    "n6_all_j3_k2_sas": (6, 6, -1, 3, 2, 1.0, 0.1, 0.05, 200, 1, 1, 1),
    # larger sectors: basis + energies + CSR digest only
    "n12_j0_k0_d1": (12, 12, 6, 0, 0, 1.0, 0.0, 0.0, 200, 1, 0, 0),
    "n12_j3_k5_d1": (12, 12, 6, 3, 5, 1.0, 0.0, 0.0, 200, 1, 0, 0),
    "n14_j0_k0_d1": (14, 14, 7, 0, 0, 1.0, 0.0, 0.0, 200, 1, 0, 0),
}
# every (J, K) sector of Nphi = 6, Ne = 6 (3 + 3): short orbits and null orbits included
for _J in range(6):
    for _K in range(6):
        CASES[f"n6_j{_J}_k{_K}"] = (6, 6, 3, _J, _K, 1.0, 0.0, 0.0, 200, 1, 1, 1)


def csr_digest(row_ptr, col, val):
    """Order-sensitive digest of the column structure and rounded values."""
    import hashlib

    h = hashlib.sha256()
    h.update(np.asarray(row_ptr, np.int64).tobytes())
    h.update(np.asarray(col, np.int64).tobytes())
    return h.hexdigest()


def run_case(name, spec):
    nphi, nel, nel_up, J, K, d, dsas, dv, lam, seed, dense, full = spec
    with tempfile.TemporaryDirectory() as tmp:
        cmd = [PROBE, str(nphi), str(nel), str(nel_up), str(J), str(K), repr(d), repr(dsas), repr(dv), str(lam),
               str(seed), str(os.cpu_count() or 1), tmp, str(dense)]
        subprocess.run(cmd, check=True)
        meta = {}
        with open(os.path.join(tmp, "meta.txt")) as f:
            for line in f:
                k, v = line.split()
                meta[k] = float(v)

        def rd(n, dt):
            p = os.path.join(tmp, n + ".bin")
            return np.fromfile(p, dt) if os.path.exists(p) else np.zeros(0, dt)

        out = dict(
            spec=np.array([nphi, nel, nel_up, J, K, lam, seed], np.int64),
            params=np.array([d, dsas, dv], np.float64),
            id=rd("id", np.uint64),
            period=rd("period", np.int16),
        )
        if len(out["id"]):
            row_ptr, col, val = rd("row_ptr", np.int64), rd("col", np.int64), rd("val", np.complex128)
            out.update(
                alpha=rd("alpha", np.float64),
                beta=rd("beta", np.float64),
                eigenvalues=rd("eigenvalues", np.float64),
                E_rq=np.array([meta["E_rq"]]),
                Ec=np.array([meta["Ec"]]),
                V=rd("V", np.float64),
                nnz=np.array([len(col)], np.int64),
                csr_digest=np.array(csr_digest(row_ptr, col, val)),
                diag=np.array([val[row_ptr[i]:row_ptr[i + 1]][col[row_ptr[i]:row_ptr[i + 1]] == i].sum()
                               for i in range(len(row_ptr) - 1)], np.complex128),
            )
            if full:
                out.update(row_ptr=row_ptr, col=col.astype(np.int32), val=val, psir0=rd("psir0", np.complex128))
            if dense:
                out.update(dense_eigenvalues=rd("dense_eigenvalues", np.float64),
                           E_dense_printed=np.array([meta["E_dense_printed"]]))
        out["meta"] = np.array(json.dumps(meta))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(f"{name}: dim={len(out['id'])} nnz={int(meta.get('nnz', 0))}", flush=True)


def main(argv):
    if not os.path.exists(PROBE):
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    names = argv or list(CASES)
    for n in names:
        run_case(n, CASES[n])


if __name__ == "__main__":
    main(sys.argv[1:])
