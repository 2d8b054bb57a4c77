"""The C++ drop-in classes (blqh_gb300/dropin): the reference's main.cpp must
compile and link against them unmodified, and a program using them the way
main() does must reproduce the README numbers on the GPU."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, golden

DROPIN = os.path.join(ROOT, "blqh_gb300", "dropin")
LIBDIR = os.path.join(ROOT, "blqh_gb300")
REF = os.path.join(os.environ.get("BLQH_REFERENCE", "/root/reference"), "BLQH_without_spin")


def _ensure_built():
    from blqh_gb300 import build

    build.build()


def _compile(sources, out, extra=()):
    cmd = ["g++", "-O2", "-std=c++11", "-I", DROPIN, "-I", os.path.join(ROOT, "include"), *sources, "-o", out,
           "-L", LIBDIR, "-lblqh_dropin", "-lblqh_gpu", f"-Wl,-rpath,{LIBDIR}", *extra]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference checkout not present")
def test_reference_main_compiles_against_dropin():
    """main.cpp and init.cpp of the reference, unmodified, built against the drop-in
    headers (copied away from the reference headers so that the drop-in ones are found)."""
    _ensure_built()
    with tempfile.TemporaryDirectory() as tmp:
        for f in ("main.cpp", "init.cpp", "init.h"):
            shutil.copy(os.path.join(REF, f), tmp)
        _compile([os.path.join(tmp, "main.cpp"), os.path.join(tmp, "init.cpp")], os.path.join(tmp, "blqh"),
                 ("-w",))
        assert os.path.exists(os.path.join(tmp, "blqh"))


def test_driver_compiles():
    _ensure_built()
    with tempfile.TemporaryDirectory() as tmp:
        _compile([os.path.join(ROOT, "tests", "dropin_driver.cpp")], os.path.join(tmp, "drv"))


@pytest.mark.gpu
@pytest.mark.parametrize("d,e_readme,tol", [(0.0, -0.6367069257, 5e-11), (3.0, -1.235882219, 5e-10)])
def test_driver_reproduces_readme(d, e_readme, tol):
    _ensure_built()
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "drv")
        _compile([os.path.join(ROOT, "tests", "dropin_driver.cpp")], exe)
        r = subprocess.run([exe, "8", "8", "4", "4", "4", repr(d)], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr
        out = dict(line.split() for line in r.stdout.strip().splitlines())
        assert int(out["nHilbert"]) == 79
        assert abs(float(out["E_lanczos"]) - e_readme) < tol
        assert abs(float(out["E_dense"]) - e_readme) < tol
        g = golden("readme_d0" if d == 0.0 else "readme_d3")
        assert int(out["id0"]) == int(g["id"][0])
        if d == 0.0:
            assert abs(float(out["amax"]) - 0.3380617019) < 1e-9
