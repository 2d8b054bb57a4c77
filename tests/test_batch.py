"""The batched sweep (blqh_batch_*): many instances of uneven dimension, real and
complex, in one persistent launch, against the reference's eigenvalues (golden
fixtures) and against the single-sector path.

Tolerances: FP64 values |dE| <= 1e-10 against the reference's eigenvalues[0];
FP32 values (double-float SpMV, FP64 regenerated Rayleigh quotient)
|dE| <= 1e-9; identical inputs give bit-identical results (graph replay,
repeated solves)."""
import numpy as np
import pytest

from conftest import golden, golden_names

pytestmark = pytest.mark.gpu

NAMES = ["readme_d0", "readme_d3", "n6_j0_k0", "n6_j1_k2", "n6_j3_k3", "n6_all_j0_k0_sas", "n6_all_j3_k2_sas",
         "n8_j0_k1_d1", "n8_j2_k3_d05", "n8_j0_k0_bias", "n8_j4_k0_uneven", "n10_j5_k5_d1", "n10_j0_k3_d15",
         "n12_j0_k0_d1", "n12_j3_k5_d1"]


@pytest.fixture(scope="module")
def B():
    import blqh_gb300 as B

    return B


def spec(g):
    nphi, nel, nel_up, J, K, lam, seed = (int(v) for v in g["spec"])
    d, dsas, dv = (float(v) for v in g["params"])
    return nphi, nel, nel_up, J, K, d, dsas, dv


def golden_instances(B, names):
    out, ref = [], []
    for n in names:
        g = golden(n)
        nphi, nel, nel_up, J, K, d, dsas, dv = spec(g)
        out.append(B.instance(nphi, nel, nel_up, J, K, d, dsas, dv))
        ref.append(float(g["eigenvalues"][0]))
    return out, np.array(ref)


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 1e-9)])
def test_batch_matches_reference_eigenvalues(B, precision, tol):
    assert set(NAMES) <= set(golden_names())
    inst, ref = golden_instances(B, NAMES)
    res = B.batch_run(inst, lam=150, precision=precision)
    e = np.array([r["energy"] for r in res])
    assert np.all(np.abs(e - ref) <= tol), (e - ref)
    for r in res:
        assert r["steps"] <= min(150, r["dim"])
        assert r["resid"] < 1e-4


def test_batch_equals_single_sector(B):
    """Same sectors through blqh_ground_state: same energy to 1e-10; the batch's ground
    state is a unit eigenvector of the FP64 CSR (residual |H psi - E psi| <= 1e-6; an
    overlap test would be ill-posed where the sector's ground level is degenerate)."""
    secs = [(10, 10, 5, 0, 0, 1.0), (10, 10, 5, 2, 3, 0.5), (8, 8, 4, 4, 4, 2.0)]
    inst = [B.instance(*s[:5], s[5]) for s in secs]
    b = B.Batch(inst, lam=150, precision=B.VAL_FP64)
    b.solve()
    res = b.results()
    for i, s in enumerate(secs):
        one = B.ground_state(*s[:5], s[5], precision=B.VAL_FP64, max_steps=300, tol=1e-13)
        assert abs(res[i]["energy"] - one["energy"]) <= 1e-10
        psi = b.ground_state(i)
        assert abs(np.linalg.norm(psi) - 1) <= 1e-12
        H = B.Hamiltonian(B.Basis(*s[:5]), s[5])
        r = H.spmv(psi) - res[i]["energy"] * psi
        assert np.linalg.norm(r) <= 1e-6, np.linalg.norm(r)
    b.close()


def test_batch_shapes_agree(B):
    """Every (threads, lanes per row) shape gives the same energies (to 1e-12)."""
    inst = [B.instance(10, 10, 5, j, k, 1.0) for j, k in ((0, 0), (1, 2), (3, 5))]
    base = None
    for threads in (256, 512):
        for lpr in (4, 8, 16, 32):
            res = B.batch_run(inst, lam=120, precision=B.VAL_FP32, threads=threads, lanes_per_row=lpr)
            e = np.array([r["energy"] for r in res])
            if base is None:
                base = e
            assert np.max(np.abs(e - base)) <= 1e-12, (threads, lpr, e - base)


def test_batch_graph_replay_is_bit_identical(B):
    inst = [B.instance(10, 10, 5, j, (3 * j) % 10, d) for j in range(4) for d in (0.5, 1.5)]
    b = B.Batch(inst, lam=100, precision=B.VAL_FP32, graph=True)
    b.solve()
    r1 = b.results()
    b.solve()  # replay of the captured graph
    r2 = b.results()
    tm = b.timing()
    assert tm["lanczos_ms"] > 0 and tm["finish_ms"] > 0 and tm["launches"] == 1 + len(inst) + 1
    b.close()
    b2 = B.Batch(inst, lam=100, precision=B.VAL_FP32, graph=False)
    b2.solve()
    r3 = b2.results()
    b2.close()
    for a, c, d in zip(r1, r2, r3):
        assert a["energy"] == c["energy"] == d["energy"]
        assert a["ritz0"] == c["ritz0"] == d["ritz0"]


def test_batch_uneven_mixed_and_empty(B):
    """Nphi 8, 10 and 12 instances, real and complex, plus an empty sector, in one launch."""
    names = ["readme_d0", "n10_j5_k5_d1", "n12_j0_k0_d1"]
    inst, ref = golden_instances(B, names)
    inst.insert(1, B.instance(8, 8, 4, 9, 0, 1.0))  # J >= nphi: empty sector
    res = B.batch_run(inst, lam=150, precision=B.VAL_FP32)
    assert res[1]["dim"] == 0 and np.isnan(res[1]["energy"])
    e = np.array([res[i]["energy"] for i in (0, 2, 3)])
    assert np.all(np.abs(e - ref) <= 1e-9)


def test_batch_rejects_bad_options(B):
    inst = [B.instance(8, 8, 4, 4, 4, 1.0)]
    with pytest.raises(B.BlqhError):
        B.batch_run(inst, lam=1)
    with pytest.raises(B.BlqhError):
        B.batch_run(inst, lam=50, threads=384)
