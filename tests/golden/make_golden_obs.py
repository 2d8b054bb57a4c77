"""Generates tests/golden/obs/: the reference's own ground-state observables
(pseudospin_Sz, pseudospin_Sx, occupatation_number; BLQH_without_spin/
lanczos_hamiltonian.cpp:658-736) on a few sectors, by oracle/_ref/ref_probe
(the reference compiled from its sources by oracle/build_ref.sh).

usage: python tests/golden/make_golden_obs.py
"""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "obs")
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
PROBE = os.path.join(ROOT, "oracle", "_ref", "ref_probe")

# name: (nphi, nel, nel_up, J, K, d, dsas, dv)
CASES = {
    "readme_d0": (8, 8, 4, 4, 4, 0.0, 0.0, 0.0),
    "n8_j0_k1_d1": (8, 8, 4, 0, 1, 1.0, 0.0, 0.0),
    "n6_all_j0_k0_sas": (6, 6, -1, 0, 0, 1.0, 0.1, 0.0),
    "n6_all_j3_k2_sas": (6, 6, -1, 3, 2, 1.0, 0.1, 0.05),
    "n8_all_j0_k0_sas": (8, 8, -1, 0, 0, 0.5, 0.05, 0.0),
    "n8_all_j2_k4_sas": (8, 8, -1, 2, 4, 1.5, 0.2, 0.02),
}


def main():
    if not os.path.exists(PROBE):
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    for name, (nphi, nel, nup, J, K, d, dsas, dv) in CASES.items():
        with tempfile.TemporaryDirectory() as tmp:
            subprocess.run([PROBE, str(nphi), str(nel), str(nup), str(J), str(K), repr(d), repr(dsas), repr(dv),
                            "200", "1", str(os.cpu_count() or 1), tmp, "0", "1.0", "1"], check=True)
            o = np.fromfile(os.path.join(tmp, "obs.bin"), np.float64)
            ev = np.fromfile(os.path.join(tmp, "eigenvalues.bin"), np.float64)
            np.savez_compressed(os.path.join(HERE, name + ".npz"),
                                spec=np.array([nphi, nel, nup, J, K], np.int64), params=np.array([d, dsas, dv]),
                                Sz=o[0:1], Sx=o[1:2], occupation=o[2:].reshape(2, nphi), eigenvalues=ev[:1])
            print(name, "Sz", o[0], "Sx", o[1], flush=True)


if __name__ == "__main__":
    main()
