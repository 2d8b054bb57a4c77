"""The spinful C++ drop-in classes (blqh_gb300/dropin_spin): the reference's
BLQH_with_spin main.cpp must compile and link against them unmodified, and a
program using them the way that main() does must reproduce the reference's
spinful fixtures on the GPU."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT

DROPIN = os.path.join(ROOT, "blqh_gb300", "dropin_spin")
LIBDIR = os.path.join(ROOT, "blqh_gb300")
REF = os.path.join(os.environ.get("BLQH_REFERENCE", "/root/reference"), "BLQH_with_spin")
SPIN = os.path.join(ROOT, "tests", "golden", "spin")


def _ensure_built():
    from blqh_gb300 import build

    build.build()


def _compile(sources, out, extra=()):
    cmd = ["g++", "-O2", "-std=c++11", "-I", DROPIN, "-I", os.path.join(ROOT, "include"), *sources, "-o", out,
           "-L", LIBDIR, "-lblqh_dropin_spin", "-lblqh_gpu", f"-Wl,-rpath,{LIBDIR}", *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference checkout not present")
def test_reference_spin_main_compiles_against_dropin():
    """main.cpp and init.cpp of BLQH_with_spin, unmodified, built against the
    spinful drop-in headers (copied away from the reference headers)."""
    _ensure_built()
    with tempfile.TemporaryDirectory() as tmp:
        for f in ("main.cpp", "init.cpp", "init.h"):
            shutil.copy(os.path.join(REF, f), tmp)
        _compile([os.path.join(tmp, "main.cpp"), os.path.join(tmp, "init.cpp")], os.path.join(tmp, "blqh"),
                 ("-w",))
        assert os.path.exists(os.path.join(tmp, "blqh"))


def test_spin_driver_compiles():
    _ensure_built()
    with tempfile.TemporaryDirectory() as tmp:
        _compile([os.path.join(ROOT, "tests", "dropin_spin_driver.cpp")], os.path.join(tmp, "drv"))


def test_spin_basis_host_methods_match_oracle():
    """translate / inv_translate of the drop-in basis (host code) against the
    oracle's restatement, through a small C++ program that needs no GPU."""
    from oracle import spin_ref as S

    src = r'''
#include <cstdio>
#include "basis.h"
int main() {
  basis b(6, 6, 3, 0, 0);
  b.nphi = 6;
  b.popcount_table.assign(1 << 6, 0);
  for (int i = 0; i < 64; i++) b.popcount_table[i] = __builtin_popcount(i);
  unsigned long cs[4] = {0x0f3a5cUL, 0x123456UL, 0xabcdefUL, 0x00ffffUL};
  for (unsigned long c : cs)
    for (int k = 0; k < 6; k++) {
      int s1 = 0, s2 = 0;
      unsigned long t = b.translate(c, k, s1), u = b.inv_translate(c, k, s2);
      printf("%lu %d %lu %d %lu %d\n", c, k, t, s1, u, s2);
    }
  return 0;
}
'''
    _ensure_built()
    with tempfile.TemporaryDirectory() as tmp:
        p = os.path.join(tmp, "t.cpp")
        with open(p, "w") as f:
            f.write(src)
        exe = os.path.join(tmp, "t")
        _compile([p], exe)
        env = dict(os.environ)
        r = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=60)
        assert r.returncode == 0, r.stderr
    for line in r.stdout.split("\n"):
        if not line.strip():
            continue
        c, k, t, s1, u, s2 = map(int, line.split())
        assert (t, s1) == S.translate(c, k, 6)
        assert (u, s2) == S.translate(c, k, 6, inverse=True)


CASES = ["s6_j0_k0", "s6_j2_k3", "s6_su4_j0_k0", "s6_up2_j1_k3", "s4_all_j0_k0", "s4_all_j1_k1", "s5_all_j0_k2"]


def _pseudospin_sz(ids, psi, nphi, nel):
    m = (1 << nphi) - 1
    up = sum((bin(int(c) & m).count("1") + bin((int(c) >> nphi) & m).count("1")) * abs(a) ** 2
             for c, a in zip(ids, psi))
    return (2.0 * up / np.sum(np.abs(psi) ** 2) - nel) / (2.0 * nel)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_spin_driver_reproduces_fixture(name):
    g = np.load(os.path.join(SPIN, name + ".npz"), allow_pickle=True)
    nphi, nel, nel_up, nel_su, J, K, _, _ = (int(x) for x in g["spec"])
    d, dsas, dv, dz = (float(x) for x in g["params"])
    _ensure_built()
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "drv")
        _compile([os.path.join(ROOT, "tests", "dropin_spin_driver.cpp")], exe)
        args = [nphi, nel, nel_up, nel_su, J, K, repr(d), repr(dsas), repr(dv), repr(dz)]
        r = subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr
    out = dict(line.split() for line in r.stdout.strip().splitlines())
    assert int(out["nHilbert"]) == len(g["id"])
    assert int(out["id0"]) == int(g["id"][0]) and int(out["idlast"]) == int(g["id"][-1])
    e0 = float(g["dense_eigenvalues"][0])
    for k in ("E_dense", "E_lanczos", "eig0"):
        assert abs(float(out[k]) - e0) <= 1e-10, (k, out[k], e0)
    ev = g["dense_eigenvalues"]
    if ev[1] - ev[0] > 1e-6:  # non-degenerate: the ground state is fixed up to a phase
        want = _pseudospin_sz(g["id"], g["psir0"], nphi, nel)
        assert abs(float(out["pseudospin_Sz"]) - want) <= 1e-8
        # the reference's own observables (its methods on its psir_0, fixture "obs")
        obs = g["obs"]
        names = ["Sz", "pseudospin_Sz", "upper_Sz", "down_Sz", "Sx", "spinflip"]
        names += [f"occ_{a}_{j}" for a in range(2) for j in range(nphi)]
        for k, name in enumerate(names):
            assert abs(float(out[name]) - obs[k]) <= 1e-8, (name, out[name], obs[k])
