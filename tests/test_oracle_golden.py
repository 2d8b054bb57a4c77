"""Pins the CPU oracle against the reference's own outputs (CPU only).

The fixtures in tests/golden were produced by the reference's sources compiled
out-of-tree (tests/golden/make_golden.py); README.md:58-103 of the reference
gives the two published energies checked here as well.
"""
import numpy as np
import pytest

from conftest import golden, golden_names

SMALL = [n for n in golden_names() if not n.startswith(("n12", "n14"))]


def test_readme_energies(oracle):
    # README.md:60-63 (d=0) and 87-90 (d=3): nHilbert 79, Lanczos E_gs/Ne,
    # printed to 10 significant digits (tolerance = half a unit in the last place)
    for d, e_readme, tol in ((0.0, -0.6367069257, 5e-11), (3.0, -1.235882219, 5e-10)):
        B = oracle.Basis(8, 8, 4, 4, 4)
        assert B.dim == 79
        H = oracle.Hamil(B, d)
        a, b = H.lanczos(200, 1)
        e = oracle.tridiag_eigenvalues(a, b)[0] / 8
        assert abs(e - e_readme) < tol
        ed = np.linalg.eigvalsh(H.dense())[0] / 8
        assert abs(ed - e_readme) < tol


@pytest.mark.parametrize("name", SMALL)
def test_oracle_matches_reference(oracle, name):
    g = golden(name)
    nphi, nel, nel_up, J, K, lam, seed = (int(v) for v in g["spec"])
    d, dsas, dv = g["params"]
    B = oracle.Basis(nphi, nel, nel_up, J, K)
    # representatives and periods bit-exact (basis.cpp:61-119)
    assert np.array_equal(B.id, g["id"])
    assert np.array_equal(B.period, g["period"])
    if not len(g["id"]):
        return
    H = oracle.Hamil(B, d, dsas, dv)
    # CSR: columns bit-exact; values bit-exact (same += order as the reference)
    assert np.array_equal(H.row_ptr, g["row_ptr"])
    assert np.array_equal(H.col, g["col"].astype(np.int64))
    assert np.max(np.abs(H.val - g["val"]), initial=0) == 0.0
    # lowest eigenvalue of the matrix = reference Lanczos eigenvalues[0]
    e = np.linalg.eigvalsh(H.dense())
    assert abs(e[0] - g["eigenvalues"][0]) < 1e-10
    if "dense_eigenvalues" in g:
        assert np.max(np.abs(e - g["dense_eigenvalues"])) < 1e-10


@pytest.mark.parametrize("name", ["n12_j0_k0_d1", "n12_j3_k5_d1"])
def test_oracle_basis_large(oracle, name):
    g = golden(name)
    nphi, nel, nel_up, J, K, lam, seed = (int(v) for v in g["spec"])
    B = oracle.Basis(nphi, nel, nel_up, J, K)
    assert np.array_equal(B.id, g["id"])
    assert np.array_equal(B.period, g["period"])


def test_oracle_rows_n12_sample(oracle):
    """A slice of rows at Nphi=12 against the reference's diagonal and nnz."""
    g = golden("n12_j0_k0_d1")
    B = oracle.Basis(12, 12, 6, 0, 0)
    H = oracle.Hamil(B, 1.0, rows=(0, 200))
    diag = np.array([H.val[H.row_ptr[i]:H.row_ptr[i + 1]][H.col[H.row_ptr[i]:H.row_ptr[i + 1]] == i].sum()
                     for i in range(200)])
    assert np.max(np.abs(diag - g["diag"][:200])) == 0.0


def test_mt19937_stream(oracle):
    # std::mt19937 default-seeded 10000th output is 4123659995 (C++ standard, [rand.predef])
    a = oracle.mt19937(5489, 10000)
    assert int(a[-1]) == 4123659995


@pytest.mark.parametrize("name", ["n8_j0_k1_d1", "n8_j2_k3_d05", "n10_j0_k3_d15", "readme_d0", "n10_j5_k5_d1"])
def test_oracle_lanczos_coefficients(oracle, name):
    """The reference's plain recurrence from its std::mt19937 seed-1 start vector
    (lanczos_hamiltonian.cpp:453-579), imaginary part drawn first: the first 20
    alpha and beta agree with the reference's own to 1e-12 (relative to the
    spectrum's scale), complex sectors included."""
    g = golden(name)
    nphi, nel, nel_up, J, K, lam, seed = (int(v) for v in g["spec"])
    d, dsas, dv = g["params"]
    H = oracle.Hamil(oracle.Basis(nphi, nel, nel_up, J, K), d, dsas, dv)
    a, b = H.lanczos(20, seed)
    scale = np.max(np.abs(g["alpha"]))
    assert np.max(np.abs(a - g["alpha"][:20])) <= 1e-12 * scale
    assert np.max(np.abs(b[1:] - g["beta"][1:21])) <= 1e-12 * scale
