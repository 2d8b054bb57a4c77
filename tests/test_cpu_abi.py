"""CPU-side checks of the C-ABI library: it loads, exports every symbol the
headers declare, and its host-only pieces (start-vector RNG, dense state
index tables) agree with the oracle. No CUDA device is used here."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

build_needed = not os.path.exists(os.path.join(ROOT, "blqh_gb300", "libblqh_gpu.so"))


@pytest.fixture(scope="module")
def L():
    if build_needed:
        from blqh_gb300 import build

        build.build()
    from blqh_gb300._lib import lib

    return lib()


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"^\s*(?:int|const char\*|double)\s+(blqh_\w+)\s*\(", src, re.M))
    return names


def test_exports_every_declared_symbol(L):
    names = declared_symbols()
    assert len(names) >= 25
    for n in sorted(names):
        assert hasattr(L, n), n


def test_python_signatures_cover_header():
    from blqh_gb300._lib import DEBUG_SIGNATURES, SIGNATURES

    assert declared_symbols() == {s[0] for s in SIGNATURES + DEBUG_SIGNATURES}


def test_start_vector_matches_std_mt19937(L, oracle):
    """The reference's complex(draw(), draw()) as GCC evaluates it: imaginary part first."""
    import blqh_gb300 as B

    for seed in (1, 2, 12345):
        raw = oracle.mt19937(seed, 2 * 1000).astype(np.float64) / 4294967295.0 - 0.5
        x = B.start_vector(1000, seed, 0, is_complex=True)
        ref = raw[1::2] + 1j * raw[0::2]
        ref /= np.linalg.norm(ref)
        assert np.max(np.abs(x - ref)) < 1e-15
        y = oracle.start_vector(1000, seed)
        assert np.max(np.abs(x - y)) < 1e-15


def test_start_vector_mt64_known_answer(L):
    """mt19937-64 seeded with 5489 first draws 14514284786278117030 (std::mt19937_64's default stream)."""
    import blqh_gb300._lib as bl

    out = np.zeros(1)
    bl.check(L.blqh_start_vector(5489, 1, 1, 0, out.ctypes.data_as(ctypes.c_void_p)))
    u = ((14514284786278117030 >> 12) + 0.5) / 4503599627370496.0 - 0.5
    assert out[0] == np.sign(u)  # a single entry normalizes to +-1


@pytest.mark.parametrize("sec", [(8, 8, 4, 4, 4), (10, 10, 5, 5, 5), (6, 6, -1, 3, 2), (7, 6, -1, 1, 2),
                                 (12, 12, 6, 0, 0), (6, 6, 3, -1, 0), (9, 9, 4, 1, -1)])
def test_dense_index_is_reference_insertion_order(L, oracle, sec):
    from blqh_gb300._lib import Sector

    ob = oracle.Basis(*sec)
    ins = ob.inserted()
    s = Sector(*sec, 0)
    idx = np.zeros(len(ins), np.int64)
    nv = ctypes.c_int64()
    rc = L.blqh_debug_sector_index(ctypes.byref(s), len(ins), ins.ctypes.data_as(ctypes.c_void_p),
                                   idx.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nv))
    assert rc == 0
    assert nv.value == len(ins)
    assert np.array_equal(idx, np.arange(len(ins)))


def test_invalid_sector_rejected(L):
    from blqh_gb300._lib import Sector

    s = Sector(17, 8, 4, 0, 0, 0)
    rc = L.blqh_debug_sector_index(ctypes.byref(s), 0, None, None, None)
    assert rc == -4
    s = Sector(16, 16, -1, 0, 0, 0)  # free split needs 2*nphi < 32 (32-bit states in the reference)
    assert L.blqh_debug_sector_index(ctypes.byref(s), 0, None, None, None) == -4


def test_struct_layouts_match_header():
    """The ctypes mirrors of the header's structs have the C compiler's sizes and field offsets
    (a mismatch would shift every field after it across the C ABI)."""
    import subprocess
    import tempfile

    from blqh_gb300 import _lib as M

    pairs = {"blqh_sector": M.Sector, "blqh_params": M.Params, "blqh_sector_spin": M.SectorSpin,
             "blqh_params_spin": M.ParamsSpin, "blqh_sector_mono": M.SectorMono, "blqh_params_mono": M.ParamsMono,
             "blqh_lanczos_opts": M.LanczosOpts, "blqh_result": M.Result, "blqh_instance": M.Instance,
             "blqh_batch_opts": M.BatchOpts, "blqh_batch_result": M.BatchResult}
    src = ['#include <cstddef>', '#include <cstdio>', '#include "blqh_gpu.h"', "int main() {"]
    for cname, cls in pairs.items():
        src.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            cf = "lambda" if fname == "lambda_" else fname
            src.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {cf}));')
    src.append("  return 0;\n}")
    with tempfile.TemporaryDirectory() as tmp:
        p = os.path.join(tmp, "layout.cpp")
        with open(p, "w") as f:
            f.write("\n".join(src))
        exe = os.path.join(tmp, "layout")
        r = subprocess.run(["g++", "-I", os.path.join(ROOT, "include"), p, "-o", exe], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    seen = 0
    for line in out:
        if not line:
            continue
        cname, what, val = line.split()
        cls = pairs[cname]
        want = ctypes.sizeof(cls) if what == "size" else getattr(cls, what).offset
        assert int(val) == want, (cname, what, val, want)
        seen += 1
    assert seen == sum(1 + len(c._fields_) for c in pairs.values())
