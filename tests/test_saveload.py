"""The Lanczos checkpoint text (lhamil::save_to_file / read_from_file,
BLQH_without_spin/lanczos_hamiltonian.cpp:738-819) in the drop-in classes and the
Python mirror: byte-identical to what the reference's own writer produces for
the same data, and each side reads the other's file. psi_n0 (first components of
the tridiagonal's eigenvectors) against numpy."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT

REF_PROBE = os.path.join(ROOT, "oracle", "_ref", "ref_saveload")
PROBE_SRC = os.path.join(ROOT, "oracle", "ref_saveload.cpp")


def _data(n=37, seed=4):
    rng = np.random.default_rng(seed)
    return dict(nHilbert=5926, n=n, seed=12345, eigenvalues=np.sort(rng.standard_normal(n) * 3 - 7),
                norm=np.abs(rng.standard_normal(n + 1)) * 10 ** rng.uniform(-6, 0, n + 1),
                overlap=rng.standard_normal(n) - 5, psi_0=rng.standard_normal(n) / 7,
                psi_n0=rng.standard_normal(n) * 1e-3)


def _write_input(path, d):
    with open(path, "w") as f:
        f.write(f"{d['nHilbert']} {d['n']} {d['seed']}\n")
        for k in ("eigenvalues", "norm", "overlap", "psi_0", "psi_n0"):
            f.write(" ".join(repr(float(x)) for x in d[k]) + "\n")


def _parse_dump(txt):
    lines = txt.strip().splitlines()
    head = [int(x) for x in lines[0].split()]
    return head, [np.array([float(x) for x in l.split()]) for l in lines[1:]]


@pytest.fixture(scope="module")
def dropin_probe():
    from blqh_gb300 import build

    build.build()
    d = tempfile.mkdtemp()
    exe = os.path.join(d, "dropin_saveload")
    inc = os.path.join(ROOT, "blqh_gb300", "dropin")
    lib = os.path.join(ROOT, "blqh_gb300")
    r = subprocess.run(["g++", "-O2", "-std=c++11", "-I", inc, "-I", os.path.join(ROOT, "include"), PROBE_SRC,
                        "-o", exe, "-L", lib, "-lblqh_dropin", "-lblqh_gpu", f"-Wl,-rpath,{lib}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def test_python_writer_reader_roundtrip(tmp_path):
    import blqh_gb300 as B

    d = _data()
    p = tmp_path / "ckpt.txt"
    B.save_lanczos_text(p, d["nHilbert"], d["n"], d["seed"], d["eigenvalues"], d["norm"], d["overlap"], d["psi_0"],
                        d["psi_n0"])
    r = B.read_lanczos_text(p)
    assert (r["nHilbert"], r["lambda"], r["seed"]) == (d["nHilbert"], d["n"], d["seed"])
    for k in ("eigenvalues", "norm", "overlap", "psi_0", "psi_n0"):
        assert np.allclose(r[k], d[k], rtol=1e-7, atol=0)


def test_dropin_writer_matches_python_writer(tmp_path, dropin_probe):
    import blqh_gb300 as B

    d = _data()
    _write_input(tmp_path / "in.txt", d)
    subprocess.run([dropin_probe, "write", str(tmp_path / "c.txt"), str(tmp_path / "in.txt")], check=True)
    B.save_lanczos_text(tmp_path / "py.txt", d["nHilbert"], d["n"], d["seed"], d["eigenvalues"], d["norm"],
                        d["overlap"], d["psi_0"], d["psi_n0"])
    assert (tmp_path / "c.txt").read_text() == (tmp_path / "py.txt").read_text()


@pytest.mark.skipif(not os.path.exists(REF_PROBE), reason="reference probe not built (oracle/build_ref.sh)")
def test_reference_and_dropin_files_identical_and_cross_readable(tmp_path, dropin_probe):
    d = _data(n=53, seed=9)
    _write_input(tmp_path / "in.txt", d)
    subprocess.run([REF_PROBE, "write", str(tmp_path / "ref.txt"), str(tmp_path / "in.txt")], check=True)
    subprocess.run([dropin_probe, "write", str(tmp_path / "ours.txt"), str(tmp_path / "in.txt")], check=True)
    assert (tmp_path / "ref.txt").read_text() == (tmp_path / "ours.txt").read_text()
    # the reference reads ours, we read the reference's: the same numbers
    a = subprocess.run([REF_PROBE, "read", str(tmp_path / "ours.txt")], capture_output=True, text=True, check=True)
    b = subprocess.run([dropin_probe, "read", str(tmp_path / "ref.txt")], capture_output=True, text=True, check=True)
    ha, la = _parse_dump(a.stdout)
    hb, lb = _parse_dump(b.stdout)
    assert ha == hb == [d["nHilbert"], d["n"], d["seed"]]
    for x, y in zip(la, lb):
        assert np.array_equal(x, y)


def test_first_components_of_tridiagonal_eigenvectors():
    """tridiag.h (host implicit QL, first row only) against numpy's eigh."""
    src = r'''
#include <cstdio>
#include <random>
#include "tridiag.h"
int main() {
  std::mt19937 g(7);
  std::normal_distribution<double> n;
  for (int m : {1, 2, 5, 40, 157}) {
    std::vector<double> a(m), b(m + 1);
    for (auto& x : a) x = n(g) - 3;
    for (auto& x : b) x = std::fabs(n(g)) * 0.7;
    std::vector<double> ev, fr;
    if (!tridiag_first_row(a.data(), b.data(), m, ev, fr)) return 1;
    printf("%d\n", m);
    for (int i = 0; i < m; i++) printf("%.17g %.17g %.17g %.17g\n", a[i], b[i + 1], ev[i], fr[i]);
  }
}
'''
    with tempfile.TemporaryDirectory() as t:
        cpp, exe = os.path.join(t, "t.cpp"), os.path.join(t, "t")
        open(cpp, "w").write(src)
        subprocess.run(["g++", "-O2", "-std=c++11", "-I", os.path.join(ROOT, "blqh_gb300", "dropin"), cpp, "-o", exe],
                       check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    i = 0
    while i < len(out) and out[i].strip():
        m = int(out[i])
        rows = np.array([[float(x) for x in out[i + 1 + k].split()] for k in range(m)])
        i += m + 1
        a, off, ev, fr = rows[:, 0], rows[:, 1], rows[:, 2], rows[:, 3]
        T = np.diag(a) + np.diag(off[:m - 1], 1) + np.diag(off[:m - 1], -1)
        w, V = np.linalg.eigh(T)
        assert np.max(np.abs(w - ev)) <= 1e-13 * max(1.0, np.max(np.abs(w)))
        assert np.max(np.abs(np.abs(V[0]) - np.abs(fr))) <= 1e-10
