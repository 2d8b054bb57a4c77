"""The autotuner (blqh_gb300/csrc/tune.cu): a batch created without an explicit
shape times its candidates once, writes the choice to the JSON cache, and a
second batch of the same class reads it back; the tuned shape gives the same
energies as an explicit one."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_shape_is_tuned_and_cached(tmp_path, monkeypatch):
    import blqh_gb300 as B

    cache = tmp_path / "tune.json"
    monkeypatch.setenv("BLQH_TUNE_CACHE", str(cache))
    monkeypatch.delenv("BLQH_TUNE", raising=False)
    inst = [B.instance(10, 10, 5, j, k, 1.0) for j in range(3) for k in range(3)]
    b = B.Batch(inst, lam=80)
    shape = b.shape()
    b.solve()
    e_tuned = np.array([r["energy"] for r in b.results()])
    b.close()
    data = json.loads(cache.read_text())
    keys = [k for k in data if k.startswith("batch|")]
    assert len(keys) == 1
    t, l, ms = data[keys[0]]
    assert (t, l) == (shape["threads"], shape["lanes_per_row"]) and ms > 0
    b2 = B.Batch(inst, lam=80)  # same class: read from the cache
    assert b2.shape() == shape
    b2.close()
    ref = B.batch_run(inst, lam=80, threads=256, lanes_per_row=8)
    assert np.max(np.abs(e_tuned - np.array([r["energy"] for r in ref]))) <= 1e-12


def test_spmv_lanes_tuned_on_large_matrix(tmp_path, monkeypatch):
    import blqh_gb300 as B

    cache = tmp_path / "tune.json"
    monkeypatch.setenv("BLQH_TUNE_CACHE", str(cache))
    b = B.Basis(14, 14, 7, 0, 0)
    H = B.Hamiltonian(b, 1.0, precision=B.VAL_FP32)
    L = B.Lanczos(H, max_steps=10, tol=0)
    L.iterate()
    data = json.loads(cache.read_text())
    keys = [k for k in data if k.startswith("spmv|")]
    assert len(keys) == 1 and data[keys[0]][0] in (4, 8, 16, 32)
