"""The monolayer C++ drop-in classes (blqh_gb300/dropin_mono): the reference's
Monolayer main.cpp must compile and link against them unmodified, their host
methods must match the oracle, and a program using them the way that main()
does must reproduce the reference's recorded monolayer spectrum on the GPU
(Monolayer/check/ek_nphi_18_nel_6)."""
import math
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

DROPIN = os.path.join(ROOT, "blqh_gb300", "dropin_mono")
LIBDIR = os.path.join(ROOT, "blqh_gb300")
REF = os.path.join(os.environ.get("BLQH_REFERENCE", "/root/reference"), "Monolayer")


def _ensure_built():
    from blqh_gb300 import build

    build.build()


def _compile(sources, out, extra=()):
    cmd = ["g++", "-O2", "-std=c++11", "-I", DROPIN, "-I", os.path.join(ROOT, "include"), *sources, "-o", out,
           "-L", LIBDIR, "-lblqh_dropin_mono", "-lblqh_gpu", f"-Wl,-rpath,{LIBDIR}", *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference checkout not present")
def test_reference_monolayer_main_compiles_against_dropin():
    """main.cpp and init.cpp of Monolayer, unmodified, built against the drop-in headers."""
    _ensure_built()
    with tempfile.TemporaryDirectory() as tmp:
        for f in ("main.cpp", "init.cpp", "init.h"):
            shutil.copy(os.path.join(REF, f), tmp)
        _compile([os.path.join(tmp, "main.cpp"), os.path.join(tmp, "init.cpp")], os.path.join(tmp, "mlqh"), ("-w",))
        assert os.path.exists(os.path.join(tmp, "mlqh"))


def test_mono_driver_compiles():
    _ensure_built()
    with tempfile.TemporaryDirectory() as tmp:
        _compile([os.path.join(ROOT, "tests", "dropin_mono_driver.cpp")], os.path.join(tmp, "drv"))


def test_mono_basis_host_methods_match_oracle(oracle):
    """translate / inv_translate / get_sign of the drop-in basis (host code, no GPU)."""
    src = r'''
#include <cstdio>
#include "basis.h"
int main() {
  basis b(12, 4, 0, 0);
  b.C = b.common_divisor(4, 12);
  unsigned long cs[4] = {0x00fUL, 0x123UL, 0xa05UL, 0x881UL};
  for (unsigned long c : cs)
    for (int k = 0; k < 4; k++) {
      int s1 = 0, s2 = 0, n1 = 0, n2 = 0;
      unsigned long t = b.translate(c, k, s1, n1), u = b.inv_translate(c, k, s2, n2);
      printf("%lu %d %lu %d %lu %d\n", c, k, t, s1, u, s2);
    }
  printf("sign %d %d\n", b.get_sign(0x0f0, 4, 7, 1, 10), b.get_sign(0x0f0, 5, 6, 9, 2));
  return 0;
}
'''
    _ensure_built()
    with tempfile.TemporaryDirectory() as tmp:
        p = os.path.join(tmp, "t.cpp")
        with open(p, "w") as f:
            f.write(src)
        _compile([p], os.path.join(tmp, "t"))
        out = subprocess.run([os.path.join(tmp, "t")], capture_output=True, text=True, check=True).stdout.split("\n")
    ob = oracle.MonoBasis(12, 4, 0, 0)
    rows = [l.split() for l in out if l and not l.startswith("sign")]
    assert len(rows) == 16
    for c, k, t, s1, u, s2 in rows:
        c, k = int(c), int(k)
        if k == 0:
            continue
        assert (int(t), int(s1)) == ob.translate(c, k)
        assert (int(u), int(s2)) == ob.translate(c, k, inverse=True)
    sign = [l for l in out if l.startswith("sign")][0].split()[1:]

    def get_sign(c, n, m, nt, mt):
        b = c ^ ((1 << n) | (1 << m))
        ns = sum((b >> k) & 1 for k in range(min(n, nt) + 1, max(n, nt)))
        ns += sum((b >> k) & 1 for k in range(min(m, mt) + 1, max(m, mt)))
        ns += (nt > mt and m > n) or (mt > nt and m < n)
        return -1 if ns % 2 else 1

    assert [int(x) for x in sign] == [get_sign(0x0f0, 4, 7, 1, 10), get_sign(0x0f0, 5, 6, 9, 2)]


@pytest.mark.gpu
@pytest.mark.parametrize("J,K", [(0, 0), (3, 3), (1, 2), (5, 5)])
def test_mono_dropin_matches_reference_spectrum(J, K):
    ek = dict(np.load(os.path.join(GOLDEN, "mono", "check.npz")))["ek_nphi18_nel6"]
    row = ek[6 * J + K]
    _ensure_built()
    with tempfile.TemporaryDirectory() as tmp:
        drv = os.path.join(tmp, "drv")
        _compile([os.path.join(ROOT, "tests", "dropin_mono_driver.cpp")], drv)
        ck = os.path.join(tmp, "ck.txt")
        out = subprocess.run([drv, "18", "6", str(J), str(K), "1.0", ck], capture_output=True, text=True,
                             check=True).stdout
    vals = {}
    levels = []
    for line in out.splitlines():
        k, v = line.split()
        if k == "level":
            levels.append(float(v))
        else:
            vals[k] = float(v)
    half = 0.5e-5 + 1e-12
    assert vals["C"] == 6
    assert abs(vals["eig0"] - row[1]) <= half
    assert abs(vals["E_lanczos"] - vals["eig0"]) < 1e-10
    assert abs(vals["E_dense"] - vals["eig0"]) < 1e-10
    assert abs(vals["read_eig0"] - vals["eig0"]) < 1e-7 * abs(vals["eig0"])
    assert vals["herm"] < 1e-15
    # the distinct levels of the sector, in order, against the reference's dense list (a level the
    # Krylov space holds more than once is counted once on both sides)
    def distinct(v):
        out = [v[0]]
        for x in v[1:]:
            if abs(x - out[-1]) > 2e-5:
                out.append(x)
        return out

    mine, ref = distinct(levels), distinct(list(row[1:]))
    assert len(mine) >= 5
    for a, b in zip(mine, ref):
        assert abs(a - b) <= half, (mine, ref)
    lx = ly = math.sqrt(2.0 * math.pi * 18)
    from oracle import oracle as O

    assert abs(vals["E_cl"] - O.mono_classical_energy(18, lx, ly)) < 1e-14
    assert abs(vals["V01"] - O.mono_coulomb_table(18, lx, ly)[0, 1]) < 1e-14
