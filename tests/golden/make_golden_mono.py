"""Turns the reference's recorded monolayer outputs into fixtures.

Reads Monolayer/check/ek_nphi_18_nel_6 (10 lowest eigenvalues of every
(J, K) sector of nphi = 18, nel = 6 on the square torus, dense ED, printed to 6
significant digits; line index = 6 J + K) and Monolayer/check/gs_energy_nel{4,5,6}
(ground energy per electron of the full space, no momentum filter, against
filling nu = nel / nphi, torus aspect ratio lx / ly = nel / 4) from a reference
checkout and writes tests/golden/mono/check.npz. The numbers are copied as
printed; nothing is recomputed here.

Usage: python tests/golden/make_golden_mono.py <reference root>
"""
import os
import sys

import numpy as np


def main(root):
    chk = os.path.join(root, "Monolayer", "check")
    ek = np.loadtxt(os.path.join(chk, "ek_nphi_18_nel_6"))
    out = {"ek_nphi18_nel6": ek}
    for nel in (4, 5, 6):
        out[f"gs_nel{nel}"] = np.loadtxt(os.path.join(chk, f"gs_energy_nel{nel}"))
    here = os.path.dirname(os.path.abspath(__file__))
    np.savez_compressed(os.path.join(here, "mono", "check.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("BLQH_REFERENCE", "/root/reference"))
