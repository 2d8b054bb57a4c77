"""Generates the spinful golden fixtures in tests/golden/spin/ from the reference itself.

Runs oracle/_ref/ref_probe_spin (BLQH_with_spin's own sources compiled out of
tree by oracle/build_ref.sh) on a fixed list of sectors and stores what it
prints as compressed .npz files. Only this script reads the reference.

usage: python tests/golden/make_golden_spin.py [case-name ...]   (s8_j0_k0 s8_j1_k3: the large sectors)
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "spin")
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
PROBE = os.path.join(ROOT, "oracle", "_ref", "ref_probe_spin")

# name: (nphi, nel, nel_up, nel_su, J, K, d, dsas, dv, dz, lambda, seed, dense)
CASES = {}
# the batched configuration's spinful part: Nphi = 6, Ne = 6 (3 + 3 layers, 3 + 3 spins),
# Zeeman 0.02, bias 0.01, every (J, K)
for _J in range(6):
    for _K in range(6):
        CASES[f"s6_j{_J}_k{_K}"] = (6, 6, 3, 3, _J, _K, 1.0, 0.05, 0.01, 0.02, 200, 1, 1)
# other spin polarizations and layer splits
CASES["s6_su4_j0_k0"] = (6, 6, 3, 4, 0, 0, 0.5, 0.0, 0.01, 0.02, 200, 1, 1)
CASES["s6_up2_j1_k3"] = (6, 6, 2, 3, 1, 3, 1.5, 0.0, 0.0, 0.0, 200, 1, 1)
CASES["s6_nosu_j0_k0"] = (6, 6, 3, -1, 0, 0, 1.0, 0.0, 0.01, 0.02, 200, 1, 1)
# free layer split: tunnelling and spin-flip tunnelling act
CASES["s4_all_j0_k0"] = (4, 4, -1, 2, 0, 0, 1.0, 0.1, 0.02, 0.02, 200, 1, 1)
CASES["s4_all_j1_k1"] = (4, 4, -1, 2, 1, 1, 1.0, 0.1, 0.02, 0.02, 200, 1, 1)
CASES["s5_all_j0_k2"] = (5, 4, -1, -1, 0, 2, 1.0, 0.1, 0.0, 0.05, 200, 1, 1)


# sectors above the size a dense shared-memory row could hold: stored compactly in
# tests/golden/spin_large/ (digests of the basis and of the whole CSR, value
# checksums, 256 stride-sampled rows in full, the Lanczos results and observables)
LARGE = {
    "s8_j0_k0": (8, 8, 4, 4, 0, 0, 1.0, 0.05, 0.01, 0.02, 200, 1, 0),
    "s8_j1_k3": (8, 8, 4, 4, 1, 3, 1.0, 0.05, 0.01, 0.02, 200, 1, 0),
}


def run_large(name, spec):
    import hashlib

    nphi, nel, nel_up, nel_su, J, K, d, dsas, dv, dz, lam, seed, dense = spec
    with tempfile.TemporaryDirectory() as tmp:
        cmd = [PROBE, str(nphi), str(nel), str(nel_up), str(nel_su), str(J), str(K), repr(d), repr(dsas), repr(dv),
               repr(dz), str(lam), str(seed), tmp, "0"]
        subprocess.run(cmd, check=True)
        meta = {}
        with open(os.path.join(tmp, "meta.txt")) as f:
            for line in f:
                k, v = line.split()
                meta[k] = float(v)

        def rd(n, dt):
            return np.fromfile(os.path.join(tmp, n + ".bin"), dt)

        ids, period = rd("id", np.uint64), rd("period", np.int16)
        rp, col, val = rd("row_ptr", np.int64), rd("col", np.int64), rd("val", np.complex128)
        h = hashlib.sha256()
        h.update(rp.tobytes())
        h.update(col.tobytes())
        w = (col % 7 + 1).astype(np.float64)
        rows = np.linspace(0, len(ids) - 1, 256).astype(np.int64)
        sel = np.concatenate([np.arange(rp[r], rp[r + 1]) for r in rows])
        out = dict(spec=np.array([nphi, nel, nel_up, nel_su, J, K, lam, seed], np.int64),
                   params=np.array([d, dsas, dv, dz], np.float64), dim=np.array([len(ids)], np.int64),
                   id_sha=np.array(hashlib.sha256(ids.tobytes()).hexdigest()),
                   period_sha=np.array(hashlib.sha256(period.tobytes()).hexdigest()),
                   nnz=np.array([len(col)], np.int64), csr_digest=np.array(h.hexdigest()),
                   val_checks=np.array([val.sum(), np.abs(val).sum(), (val * w).sum()], np.complex128),
                   rows=rows, row_len=np.diff(rp)[rows], row_col=col[sel].astype(np.int32), row_val=val[sel],
                   alpha=rd("alpha", np.float64), beta=rd("beta", np.float64),
                   eigenvalues=rd("eigenvalues", np.float64), E_rq=np.array([meta["E_rq"]]),
                   obs=rd("obs", np.float64), meta=np.array(json.dumps(meta)))
    os.makedirs(os.path.join(os.path.dirname(HERE), "spin_large"), exist_ok=True)
    np.savez_compressed(os.path.join(os.path.dirname(HERE), "spin_large", name + ".npz"), **out)
    print(f"{name}: dim={len(ids)} nnz={len(col)} E0={out['eigenvalues'][0]:.12f}", flush=True)


def run_case(name, spec):
    nphi, nel, nel_up, nel_su, J, K, d, dsas, dv, dz, lam, seed, dense = spec
    with tempfile.TemporaryDirectory() as tmp:
        cmd = [PROBE, str(nphi), str(nel), str(nel_up), str(nel_su), str(J), str(K), repr(d), repr(dsas), repr(dv),
               repr(dz), str(lam), str(seed), tmp, str(dense)]
        subprocess.run(cmd, check=True)
        meta = {}
        with open(os.path.join(tmp, "meta.txt")) as f:
            for line in f:
                k, v = line.split()
                meta[k] = float(v)

        def rd(n, dt):
            p = os.path.join(tmp, n + ".bin")
            return np.fromfile(p, dt) if os.path.exists(p) else np.zeros(0, dt)

        out = dict(spec=np.array([nphi, nel, nel_up, nel_su, J, K, lam, seed], np.int64),
                   params=np.array([d, dsas, dv, dz], np.float64), id=rd("id", np.uint64),
                   period=rd("period", np.int16))
        if len(out["id"]):
            out.update(row_ptr=rd("row_ptr", np.int64), col=rd("col", np.int64).astype(np.int32),
                       val=rd("val", np.complex128), alpha=rd("alpha", np.float64), beta=rd("beta", np.float64),
                       eigenvalues=rd("eigenvalues", np.float64), E_rq=np.array([meta["E_rq"]]),
                       Ec=np.array([meta["Ec"]]), psir0=rd("psir0", np.complex128),
                       obs=rd("obs", np.float64))
            if dense:
                out.update(dense_eigenvalues=rd("dense_eigenvalues", np.float64),
                           E_dense_printed=np.array([meta["E_dense_printed"]]))
        out["meta"] = np.array(json.dumps(meta))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(f"{name}: dim={len(out['id'])} nnz={int(meta.get('nnz', 0))}", flush=True)


def main(argv):
    if not os.path.exists(PROBE):
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    for n in argv or list(CASES) + list(LARGE):
        if n in LARGE:
            run_large(n, LARGE[n])
        else:
            run_case(n, CASES[n])


if __name__ == "__main__":
    main(sys.argv[1:])
