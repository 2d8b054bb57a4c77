"""Parity of the CUDA path with the reference (golden fixtures) and the oracle.

Tolerances, stated once:
  * representatives, orbit periods, CSR row pointers and column indices: bit-exact;
  * CSR values (FP64): |dv| <= 2e-14 * max(1, |v|) -- the library sums the same
    terms in another order (it merges the reference's duplicate hops first);
  * energies (FP64 Lanczos, full reorthogonalization): |dE| <= 1e-10 against the
    reference's eigenvalues[0] (its Lanczos tridiagonal, = its dense ED);
  * mixed precision (FP32 values, FP64 vectors + FP64 regenerated Rayleigh
    quotient): |dE| <= 1e-9 against the FP64 run.
"""
import hashlib

import numpy as np
import pytest

from conftest import golden, golden_names

pytestmark = pytest.mark.gpu

SMALL = [n for n in golden_names() if not n.startswith(("n12", "n14"))]
LARGE = [n for n in golden_names() if n.startswith(("n12", "n14"))]


@pytest.fixture(scope="module")
def B():
    import blqh_gb300 as B

    return B


def spec(g):
    nphi, nel, nel_up, J, K, lam, seed = (int(v) for v in g["spec"])
    d, dsas, dv = (float(v) for v in g["params"])
    return nphi, nel, nel_up, J, K, d, dsas, dv


def check_vals(got, ref, is_complex):
    ref = np.asarray(ref)
    if not is_complex:
        assert np.max(np.abs(ref.imag), initial=0) < 1e-14
        ref = ref.real
    err = np.abs(got - ref)
    assert np.all(err <= 2e-14 * np.maximum(1.0, np.abs(ref))), float(err.max())


@pytest.mark.parametrize("name", SMALL + LARGE)
def test_basis_bit_exact(B, name):
    g = golden(name)
    nphi, nel, nel_up, J, K, *_ = spec(g)
    b = B.Basis(nphi, nel, nel_up, J, K)
    assert b.dim == len(g["id"])
    assert np.array_equal(b.id, g["id"])
    assert np.array_equal(b.period, g["period"])


@pytest.mark.parametrize("name", SMALL)
def test_csr_bit_exact_structure(B, name):
    g = golden(name)
    nphi, nel, nel_up, J, K, d, dsas, dv = spec(g)
    if not len(g["id"]):
        return
    b = B.Basis(nphi, nel, nel_up, J, K)
    H = B.Hamiltonian(b, d, dsas, dv)
    rp, col, val = H.csr()
    assert np.array_equal(rp, g["row_ptr"])
    assert np.array_equal(col, g["col"])
    check_vals(val, g["val"], H.is_complex)


@pytest.mark.parametrize("name", [n for n in LARGE if n.startswith("n12")])
def test_csr_large_digest(B, name):
    g = golden(name)
    nphi, nel, nel_up, J, K, d, dsas, dv = spec(g)
    b = B.Basis(nphi, nel, nel_up, J, K)
    H = B.Hamiltonian(b, d, dsas, dv)
    rp, col, val = H.csr()
    assert H.nnz == int(g["nnz"][0])
    h = hashlib.sha256()
    h.update(rp.astype(np.int64).tobytes())
    h.update(col.astype(np.int64).tobytes())
    assert h.hexdigest() == str(g["csr_digest"])
    diag = np.array([val[rp[i]:rp[i + 1]][col[rp[i]:rp[i + 1]] == i].sum() for i in range(H.dim)])
    check_vals(diag, g["diag"], H.is_complex)


@pytest.mark.parametrize("name", SMALL + LARGE)
def test_ground_energy_fp64(B, name):
    g = golden(name)
    nphi, nel, nel_up, J, K, d, dsas, dv = spec(g)
    if not len(g["id"]):
        return
    b = B.Basis(nphi, nel, nel_up, J, K)
    H = B.Hamiltonian(b, d, dsas, dv)
    L = B.Lanczos(H, max_steps=300, reorth=True, tol=1e-13, check_every=5, seed=1)
    L.iterate()
    e, y = L.eig()
    e_ref = float(g["eigenvalues"][0])
    assert abs(e[0] - e_ref) <= 1e-10, (e[0], e_ref)
    if "dense_eigenvalues" in g:
        # distinct converged Ritz values against dense ED (low-lying spectrum)
        de = g["dense_eigenvalues"]
        assert abs(e[0] - de[0]) <= 1e-10
    L.ritz_vector(copy=False)
    assert abs(L.rayleigh() - e_ref) <= 1e-10
    assert abs(L.rayleigh_fp64() - e_ref) <= 1e-10


@pytest.mark.parametrize("name", ["readme_d0", "readme_d3", "n8_j0_k1_d1", "n10_j5_k5_d1", "n12_j0_k0_d1",
                                  "n12_j3_k5_d1"])
def test_mixed_precision(B, name):
    g = golden(name)
    nphi, nel, nel_up, J, K, d, dsas, dv = spec(g)
    e64 = B.ground_state(nphi, nel, nel_up, J, K, d, dsas, dv, precision=B.VAL_FP64, max_steps=300, tol=1e-13)
    e32 = B.ground_state(nphi, nel, nel_up, J, K, d, dsas, dv, precision=B.VAL_FP32, max_steps=300, tol=1e-13)
    assert abs(e64["energy"] - float(g["eigenvalues"][0])) <= 1e-10
    assert abs(e32["energy"] - e64["energy"]) <= 1e-9


@pytest.mark.parametrize("sec", [(12, 12, 6, 0, 0), (12, 12, 6, 1, 5), (14, 14, 7, 0, 0)])
def test_rayleigh_from_stored_rests_equals_regeneration(B, monkeypatch, sec):
    """FP32-valued runs finish <psi|H|psi> from the FP32 values plus the stored FP32
    rests of the builder's FP64 values (one double-float SpMV and one pass over the
    rests); BLQH_RQ_REGEN=1 regenerates the FP64 elements with the row generator
    instead. Same psi, real and complex sectors: the two agree to 1e-12 relative."""
    b = B.Basis(*sec)
    H = B.Hamiltonian(b, 1.0, 0.05, precision=B.VAL_FP32)
    L = B.Lanczos(H, max_steps=300, tol=1e-12)
    L.iterate()
    L.ritz_vector(copy=False)
    e_res = L.rayleigh_fp64()
    monkeypatch.setenv("BLQH_RQ_REGEN", "1")
    e_regen = L.rayleigh_fp64()
    assert abs(e_res - e_regen) <= 1e-12 * abs(e_regen), (e_res, e_regen)


def test_readme_transcripts_through_lhamil(B):
    """README.md:58-63, 85-90: nHilbert 79 and Lanczos E_gs/Ne, through the reference-shaped classes."""
    for d, e_readme, tol in ((0.0, -0.6367069257, 5e-11), (3.0, -1.235882219, 5e-10)):
        lx, ly = B.torus(8)
        L = B.lhamil(200, 1)
        L.sector.init(8, 8, 4, 4, 4)
        assert L.sector.nbasis == 79
        L.set_hamil(lx, ly, 8, 0, d, 0.0, 0.0, 0, 0, 4)
        L.coeff_explicit_update()
        L.diag()
        L.eigenstates_reconstruction()
        E = L.ground_state_energy()
        assert abs(E / 8 - e_readme) < tol
    # README top amplitudes at d=0 as a multiset (README.md:65-74)
    lx, ly = B.torus(8)
    L = B.lhamil(200, 1)
    L.sector.init(8, 8, 4, 4, 4)
    L.set_hamil(lx, ly, 8, 0, 0.0, 0.0, 0.0)
    L.coeff_explicit_update()
    L.diag()
    L.eigenstates_reconstruction()
    amp = np.sort(np.abs(L.psir_0))[::-1]
    assert np.allclose(amp[:8], 0.3380617019, atol=1e-9)
    assert abs(amp[8] - 0.2390457219) < 1e-9
    assert abs(amp[9] - 0.1690308509) < 1e-9


@pytest.mark.parametrize("sec", [(8, 8, 4, 4, 4), (8, 8, 4, 0, 1), (10, 10, 5, 2, 3), (6, 6, -1, 3, 2)])
def test_min_representatives_vs_oracle(B, oracle, sec):
    ob = oracle.Basis(*sec, rep_mode=1)
    b = B.Basis(*sec, rep_mode=B.REP_MIN)
    assert np.array_equal(b.id, ob.id)
    assert np.array_equal(b.period, ob.period)
    oh = oracle.Hamil(ob, 1.0, 0.05, 0.02)
    H = B.Hamiltonian(b, 1.0, 0.05, 0.02)
    rp, col, val = H.csr()
    assert np.array_equal(rp, oh.row_ptr)
    assert np.array_equal(col, oh.col)
    check_vals(val, oh.val, H.is_complex)


@pytest.mark.parametrize("sec,params", [((7, 7, 3, 0, 0), (1.0, 0.0, 0.0)), ((7, 7, 3, 2, 3), (1.0, 0.0, 0.0)),
                                        ((7, 6, -1, 1, 2), (1.0, 0.1, 0.05)), ((9, 9, 4, 0, 4), (0.5, 0.0, 0.0)),
                                        ((6, 6, 3, -1, -1), (1.0, 0.0, 0.0)), ((8, 6, 3, 1, -1), (2.0, 0.0, 0.0))])
def test_odd_nphi_and_no_translation_vs_oracle(B, oracle, sec, params):
    ob = oracle.Basis(*sec)
    b = B.Basis(*sec)
    assert np.array_equal(b.id, ob.id)
    oh = oracle.Hamil(ob, *params)
    H = B.Hamiltonian(b, *params)
    rp, col, val = H.csr()
    assert np.array_equal(rp, oh.row_ptr)
    assert np.array_equal(col, oh.col)
    check_vals(val, oh.val, H.is_complex)


def test_spmv_vs_oracle(B, oracle):
    for sec in ((10, 10, 5, 0, 3), (10, 10, 5, 0, 0)):
        ob = oracle.Basis(*sec)
        oh = oracle.Hamil(ob, 1.0)
        b = B.Basis(*sec)
        for prec in (B.VAL_FP64, B.VAL_FP32):
            H = B.Hamiltonian(b, 1.0, precision=prec)
            rng = np.random.default_rng(7)
            x = rng.standard_normal(b.dim) + (1j * rng.standard_normal(b.dim) if H.is_complex else 0)
            y = H.spmv(x)
            yr = oh.spmv(np.asarray(x, np.complex128))
            tol = 1e-12 if prec == B.VAL_FP64 else 1e-5
            assert np.max(np.abs(y - (yr if H.is_complex else yr.real))) <= tol * np.max(np.abs(yr))


def test_empty_and_invalid_sectors(B):
    b = B.Basis(8, 8, 4, 9, 0)  # J >= nphi: no state has that momentum
    assert b.dim == 0
    with pytest.raises(B.BlqhError):
        B.Hamiltonian(b, 1.0)
    with pytest.raises(B.BlqhError):
        B.Basis(17, 8, 4, 0, 0)
    with pytest.raises(B.BlqhError):
        B.Basis(8, 8, 9, 0, 0)


def test_breakdown_small_dim(B):
    """dim < lambda: the reorthogonalized run stops at the invariant subspace."""
    b = B.Basis(6, 6, 3, 1, 2)
    H = B.Hamiltonian(b, 1.0)
    L = B.Lanczos(H, max_steps=200, reorth=True, tol=0.0, check_every=10)
    n = L.iterate()
    assert n <= b.dim
    e, _ = L.eig()
    rp, col, val = H.csr()
    M = np.zeros((b.dim, b.dim), val.dtype)
    for i in range(b.dim):
        M[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    ev = np.linalg.eigvalsh(M)
    assert abs(e[0] - ev[0]) < 1e-10


def test_nphi16_full_size_properties(B):
    """The Nphi=16, 8+8, (0,0) sector (dim 647079) at full size: Hermitian CSR,
    mixed precision within 1e-9 of FP64, Rayleigh quotient consistent with the Ritz value."""
    b = B.Basis(16, 16, 8, 0, 0)
    assert b.dim == 647079
    ids = b.id
    assert np.all(np.diff(ids.astype(np.int64)) > 0)
    r64 = B.ground_state(16, 16, 8, 0, 0, 1.0, 0.05, 0.0, precision=B.VAL_FP64, max_steps=300, tol=1e-12)
    r32 = B.ground_state(16, 16, 8, 0, 0, 1.0, 0.05, 0.0, precision=B.VAL_FP32, max_steps=300, tol=1e-12)
    assert abs(r64["energy"] - r64["ritz0"]) < 1e-9
    assert abs(r32["energy"] - r64["energy"]) < 1e-9
    assert r64["nnz"] == r32["nnz"]


def test_nphi16_blocked_spmv(B, monkeypatch):
    """At Nphi=16 (dim 647079, 2.4e8 nonzeros) the blocked SpMV (row blocks x
    column tiles, x staged in shared memory) matches an FP64 product with the
    same FP32 matrix to a relative 1e-12."""
    sp = pytest.importorskip("scipy.sparse")
    monkeypatch.setenv("BLQH_SPMV_BLOCKED", "1")
    b = B.Basis(16, 16, 8, 0, 0)
    H = B.Hamiltonian(b, 1.0, 0.05, precision=B.VAL_FP32)
    x = np.random.default_rng(11).standard_normal(b.dim)
    y = H.spmv(x)
    assert H.spmv_layout() == 1
    rp, col, val = H.csr()
    yref = sp.csr_matrix((val, col, rp), shape=(b.dim, b.dim)) @ x
    assert np.max(np.abs(y - yref)) <= 1e-12 * np.max(np.abs(yref))


def test_double_float_spmv_accuracy(B):
    """The double-float SpMV (FP32 values, FP32-pair accumulation) against an exact
    FP64 product with the same FP32-rounded matrix: relative error <= 1e-12."""
    for sec in ((12, 12, 6, 0, 0), (12, 12, 6, 0, 5)):
        b = B.Basis(*sec)
        H = B.Hamiltonian(b, 1.0, precision=B.VAL_FP32)
        rp, col, val = H.csr()
        rng = np.random.default_rng(3)
        x = rng.standard_normal(b.dim) + (1j * rng.standard_normal(b.dim) if H.is_complex else 0)
        y = H.spmv(x)
        rows = np.repeat(np.arange(b.dim), np.diff(rp))
        yref = np.zeros(b.dim, np.complex128 if H.is_complex else np.float64)
        np.add.at(yref, rows, val * x[col])
        assert np.max(np.abs(y - yref)) <= 1e-12 * np.max(np.abs(yref))


@pytest.mark.parametrize("sec", [(14, 14, 7, 0, 0), (14, 14, 7, 0, 3), (12, 12, 6, 1, 5), (10, 10, 5, 0, 0)])
def test_blocked_spmv(B, monkeypatch, sec):
    """The blocked SpMV (warp-owned row groups, x tiles in shared memory fed by
    cp.async.bulk, segmented runs) against an exact FP64 product with the same
    FP32 matrix, real and complex sectors; repeated products give identical bits."""
    monkeypatch.setenv("BLQH_SPMV_BLOCKED", "1")
    b = B.Basis(*sec)
    H = B.Hamiltonian(b, 1.0, precision=B.VAL_FP32)
    rp, col, val = H.csr()
    rows = np.repeat(np.arange(b.dim), np.diff(rp))
    rng = np.random.default_rng(5)
    for _ in range(2):
        x = rng.standard_normal(b.dim) + (1j * rng.standard_normal(b.dim) if H.is_complex else 0)
        y = H.spmv(x)
        yref = np.zeros(b.dim, np.complex128 if H.is_complex else np.float64)
        np.add.at(yref, rows, val * x[col])
        assert np.max(np.abs(y - yref)) <= 1e-12 * np.max(np.abs(yref))
        assert np.array_equal(H.spmv(x), y)
    assert H.spmv_layout() == 1
    monkeypatch.setenv("BLQH_SPMV_BLOCKED", "0")
    y0 = H.spmv(x)
    assert np.max(np.abs(y0 - yref)) <= 1e-12 * np.max(np.abs(yref))


@pytest.mark.parametrize("name,sec", [("n14_j0_k0_d1", (14, 14, 7, 0, 0))])
def test_blocked_spmv_ground_state(B, monkeypatch, name, sec):
    monkeypatch.setenv("BLQH_SPMV_BLOCKED", "1")
    e = B.ground_state(*sec, 1.0, precision=B.VAL_FP32, max_steps=300, tol=1e-12)["energy"]
    assert abs(e - float(golden(name)["eigenvalues"][0])) < 1e-9


def test_accumulate_modes_agree(B):
    """Mixed precision with double-float and with native FP64 accumulation: same E_gs to 1e-9."""
    e = {}
    for acc in (0, 1):
        e[acc] = B.ground_state(14, 14, 7, 0, 0, 1.0, precision=B.VAL_FP32, max_steps=300, tol=1e-12,
                                accumulate=acc)["energy"]
    e64 = B.ground_state(14, 14, 7, 0, 0, 1.0, precision=B.VAL_FP64, max_steps=300, tol=1e-12)["energy"]
    assert abs(e[0] - e64) < 1e-9 and abs(e[1] - e64) < 1e-9


@pytest.mark.parametrize("sec", [(16, 16, 8, 0, 0), (14, 14, 7, 2, 7), (12, 12, 6, 0, 0), (10, 10, 5, 0, 5)])
def test_dictionary_spmv(B, monkeypatch, sec):
    """Real sectors: the blocked SpMV in dictionary form (4-byte entries, column |
    index into a shared-memory table of the distinct off-diagonal FP32 values,
    diagonal apart; each tile's stream brought into shared memory by bulk copies,
    enabled by BLQH_SPMV_DICT=1)
    against an exact FP64 product with the same FP32 matrix (relative 1e-12),
    against the (2-byte column, FP32 value) form of the blocked kernel, and
    bit-identical on a repeated product."""
    sp = pytest.importorskip("scipy.sparse")
    monkeypatch.setenv("BLQH_SPMV_BLOCKED", "1")
    monkeypatch.setenv("BLQH_SPMV_DICT", "1")
    b = B.Basis(*sec)
    H = B.Hamiltonian(b, 1.0, 0.05, precision=B.VAL_FP32)
    assert not H.is_complex
    rng = np.random.default_rng(7)
    x = rng.standard_normal(b.dim)
    y = H.spmv(x)
    assert H.spmv_layout() == 2
    assert np.array_equal(H.spmv(x), y)
    rp, col, val = H.csr()
    yref = sp.csr_matrix((val, col, rp), shape=(b.dim, b.dim)) @ x
    assert np.max(np.abs(y - yref)) <= 1e-12 * np.max(np.abs(yref))
    H.close()
    monkeypatch.setenv("BLQH_SPMV_DICT", "0")
    H2 = B.Hamiltonian(b, 1.0, 0.05, precision=B.VAL_FP32)
    y2 = H2.spmv(x)
    assert H2.spmv_layout() == 1
    assert np.max(np.abs(y - y2)) <= 1e-12 * np.max(np.abs(yref))
