"""The monolayer model on the GPU (blqh_basis_build_mono, blqh_hamil_build_mono and the
Lanczos over its CSR) against the monolayer oracle and the reference's recorded outputs
(Monolayer/check, in tests/golden/mono/check.npz).

Tolerances: representatives, periods, row pointers and columns bit-exact; values
|dv| <= 1e-14 max(1, |v|) against the oracle (both add the reference's terms in the
reference's order); energies within 1e-10 of the oracle's dense or sparse eigenvalues and
within half a unit of the 6th significant digit of the reference's printed values."""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def B():
    import blqh_gb300 as B

    return B


def check():
    return dict(np.load(os.path.join(GOLDEN, "mono", "check.npz")))


def half_unit(v):
    return 0.5 * 10.0 ** (math.floor(math.log10(abs(v))) - 5) + 1e-12


def csr_parity(B, oracle, nphi, nel, J, K, gamma=1.0, nLL=0, rep_mode=0):
    b = B.basis_mono(nphi, nel, J, K, rep_mode=rep_mode)
    ob = oracle.MonoBasis(nphi, nel, J, K, rep_mode)
    assert b.dim == ob.dim
    assert np.array_equal(b.id, ob.id)
    assert np.array_equal(b.period, ob.period)
    if not b.dim:
        return b, None, None
    lx, ly = oracle.mono_torus(nphi, gamma)
    H = B.hamiltonian_mono(b, gamma, nLL)
    oh = oracle.MonoHamil(ob, lx, ly, nLL)
    rp, col, val = H.csr()
    assert np.array_equal(rp, oh.row_ptr)
    assert np.array_equal(col, oh.col)
    ref = oh.val if H.is_complex else oh.val.real
    assert H.is_complex == (not (K <= 0 or 2 * K == math.gcd(nphi, nel)))
    if not H.is_complex:
        assert np.max(np.abs(oh.val.imag), initial=0) < 1e-13
    assert np.all(np.abs(val - ref) <= 1e-14 * np.maximum(1.0, np.abs(ref)))
    return b, H, oh


SECTORS = [(18, 6, 0, 0), (18, 6, 3, 3), (18, 6, 1, 1), (18, 6, 2, 5), (12, 4, 0, 2), (12, 4, 5, 1),
           (15, 5, 0, 0), (15, 5, 7, 4), (14, 7, 0, 3), (12, 6, 1, 2), (9, 3, 0, 1), (10, 4, 3, 1),
           (11, 4, 2, 0), (13, 5, 6, 0), (16, 8, 0, 0), (16, 4, 0, 3), (20, 5, 10, 2), (21, 7, 0, 6)]


@pytest.mark.parametrize("sec", SECTORS)
def test_mono_basis_and_csr_bit_exact(B, oracle, sec):
    csr_parity(B, oracle, *sec)


@pytest.mark.parametrize("sec", [(12, 4, -1, -1), (10, 5, 2, -1), (8, 4, -1, -1), (12, 6, -1, 0), (9, 3, 0, -1)])
def test_mono_no_symmetry_sectors(B, oracle, sec):
    csr_parity(B, oracle, *sec)


@pytest.mark.parametrize("sec", [(12, 4, 0, 0), (18, 6, 3, 1), (15, 5, 5, 2)])
def test_mono_rep_min_and_landau_level(B, oracle, sec):
    csr_parity(B, oracle, *sec, rep_mode=1)
    csr_parity(B, oracle, *sec, gamma=1.5, nLL=1)


@pytest.mark.parametrize("sec", [(18, 6, 0, 0), (15, 5, 7, 4), (12, 4, -1, -1)])
def test_mono_rows_second_launch(B, oracle, sec, monkeypatch):
    """A 64-slot first table sends most rows to the second launch (the table that holds any
    row); the CSR stays bit-exact."""
    monkeypatch.setenv("BLQH_MONO_FIRST_CAP", "64")
    csr_parity(B, oracle, *sec)


def test_mono_edge_cases(B, oracle):
    # every orbital filled: one state, diagonal only
    csr_parity(B, oracle, 6, 6, 3, 0)
    csr_parity(B, oracle, 6, 6, -1, -1)
    # one electron: no pair terms
    csr_parity(B, oracle, 8, 1, 3, 0)
    # coprime nel, nphi: C = 1, no translation orbits
    csr_parity(B, oracle, 13, 4, 6, 0)
    # an empty sector
    b = B.basis_mono(4, 2, 3, 0)
    ob = oracle.MonoBasis(4, 2, 3, 0)
    assert b.dim == ob.dim
    with pytest.raises(B.BlqhError):
        B.basis_mono(12, 4, 0, 4)  # K >= gcd(nel, nphi)
    with pytest.raises(B.BlqhError):
        B.basis_mono(32, 4, 0, 0)  # more than 31 orbitals
    with pytest.raises(B.BlqhError):
        B.basis_mono(12, 13, 0, 0)
    with pytest.raises(B.BlqhError):
        B.Hamiltonian(B.basis_mono(12, 4, 0, 0), 1.0)
    with pytest.raises(B.BlqhError):
        B.hamiltonian_mono(B.Basis(8, 8, 4, 4, 4))


def test_mono_ek_spectrum_nphi18_nel6(B):
    """Every (J, K) of Monolayer/check/ek_nphi_18_nel_6: the 10 lowest levels of the GPU
    Hamiltonian (dense eigensolve of the downloaded CSR) and the GPU Lanczos ground level."""
    ek = check()["ek_nphi18_nel6"]
    for idx, row in enumerate(ek):
        J, K = idx // 6, idx % 6
        b = B.basis_mono(18, 6, J, K)
        H = B.hamiltonian_mono(b, 1.0)
        rp, col, val = H.csr()
        M = np.zeros((b.dim, b.dim), np.complex128)
        for i in range(b.dim):
            M[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
        ev = np.linalg.eigvalsh(M)[:10]
        for e, g in zip(ev, row[1:]):
            assert abs(e - g) <= half_unit(g), (J, K, e, g)
        r = B.ground_state_mono(18, 6, J, K, max_steps=400, tol=1e-13)
        assert abs(r["eigenvalues"][0] - ev[0]) < 1e-10
        assert abs(r["energy"] - ev[0]) < 1e-10


@pytest.mark.parametrize("nel", [4, 5, 6])
def test_mono_full_space_ground_energy(B, nel):
    """Monolayer/check/gs_energy_nel{4,5,6}: the full space (no momentum filter), aspect ratio
    nel / 4, ground energy per electron against filling nel / nphi; up to C(23, 6) = 100947 states."""
    gs = check()[f"gs_nel{nel}"]
    for nu, e_ref in gs:
        nphi = int(round(nel / nu))
        r = B.ground_state_mono(nphi, nel, -1, -1, gamma=nel / 4.0, max_steps=600, tol=1e-13)
        assert r["dim"] == math.comb(nphi, nel)
        assert abs(r["eigenvalues"][0] / nel - e_ref) <= half_unit(e_ref), (nphi, r["eigenvalues"][0] / nel, e_ref)
        assert abs(r["energy"] - r["eigenvalues"][0]) < 1e-9


def test_mono_ground_energy_vs_oracle(B, oracle):
    from scipy.sparse.linalg import eigsh

    for nphi, nel, J, K in ((18, 6, 3, 3), (21, 7, 0, 0), (24, 8, 0, 4), (15, 5, 0, 1)):
        ob = oracle.MonoBasis(nphi, nel, J, K)
        lx, ly = oracle.mono_torus(nphi, 1.0)
        oh = oracle.MonoHamil(ob, lx, ly)
        e_ref = eigsh(oh.sparse(), k=1, which="SA", tol=1e-13)[0][0]
        r = B.ground_state_mono(nphi, nel, J, K, max_steps=600, tol=1e-13)
        assert abs(r["eigenvalues"][0] - e_ref) < 1e-10, (nphi, nel, J, K)
        assert abs(r["energy"] - e_ref) < 1e-9


def test_mono_large_sector_properties(B):
    """nphi = 30, nel = 10 (filling 1/3, C = 10 translations): about 1e5 states per sector.
    The orbits of the K = 0 representatives cover the J sector exactly (sum of periods =
    the J sector's size), columns ascend in every row, and the real CSR is symmetric
    (z . H x = x . H z for random x, z)."""
    nphi, nel, J = 30, 10, 0
    full = B.basis_mono(nphi, nel, J, -1)
    b = B.basis_mono(nphi, nel, J, 0)
    assert int(np.sum(b.period.astype(np.int64))) == full.dim
    H = B.hamiltonian_mono(b, 1.0)
    rp, col, val = H.csr()
    assert not H.is_complex
    starts = np.zeros(len(col), bool)
    starts[rp[1:-1]] = True
    assert np.all((np.diff(col) > 0) | starts[1:])
    rng = np.random.default_rng(3)
    x, z = rng.standard_normal(b.dim), rng.standard_normal(b.dim)
    hx, hz = H.spmv(x), H.spmv(z)
    assert abs(z @ hx - x @ hz) < 1e-10 * abs(z @ hx) + 1e-9


def test_mono_gs_energy_driver_matches_reference_text(B, tmp_path):
    """run_gs_energy_mono + write_gs_energy_mono reproduce Monolayer/check/gs_energy_nel{4,5,6}
    line for line (the reference printed them with cout's default 6 significant digits)."""
    from blqh_gb300 import sweep as S

    for nel in (4, 5, 6):
        gs = check()[f"gs_nel{nel}"]
        nphis = [int(round(nel / nu)) for nu, _ in gs]
        rows = S.run_gs_energy_mono(nel, nphis)
        path = tmp_path / f"gs{nel}.txt"
        S.write_gs_energy_mono(path, rows)
        ref = [f"{nu:g} {e:g}" for nu, e in gs]
        assert path.read_text().splitlines() == ref


def test_mono_spectrum_driver(B, tmp_path):
    """run_spectrum_mono over every (J, K) of nphi = 18, nel = 6: the |K| column and the lowest
    level of each line equal Monolayer/check/ek_nphi_18_nel_6 as printed, and the distinct levels
    agree with the distinct values of the reference's list."""
    from blqh_gb300 import sweep as S

    ek = check()["ek_nphi18_nel6"]
    rows = S.run_spectrum_mono(18, 6)
    assert [(r["J"], r["K"]) for r in rows] == [(i // 6, i % 6) for i in range(108)]
    path = tmp_path / "ek.txt"
    S.write_spectrum_mono(path, rows)
    lines = path.read_text().splitlines()
    for line, ref in zip(lines, ek):
        f = line.split()
        assert f[0] == f"{ref[0]:g}"
        assert f[1] == f"{ref[1]:g}"
        distinct = [ref[1]]
        for v in ref[2:]:
            if abs(v - distinct[-1]) > 2e-5:
                distinct.append(v)
        for a, b in zip([float(x) for x in f[1:]], distinct):
            assert abs(a - b) <= half_unit(b) + 1e-5


def test_mono_instances_in_the_batch(B):
    """Every (J, K) of nphi = 18, nel = 6 as monolayer instances of one batch, mixed with spinless
    instances: each ground energy equals the reference's recorded lowest level (as printed) and
    the single-sector path's within 1e-10; the spinless ones are unaffected by the mix."""
    ek = check()["ek_nphi18_nel6"]
    insts = [B.instance_mono(18, 6, i // 6, i % 6) for i in range(108)]
    insts += [B.instance(8, 8, 4, 4, 4, 0.0), B.instance(8, 8, 4, 4, 4, 3.0)]
    res = B.batch_run(insts, lam=200, precision=B.VAL_FP64)
    for i in range(108):
        e = res[i]["energy"]
        assert abs(e - ek[i, 1]) <= half_unit(ek[i, 1]), (i, e, ek[i, 1])
    for i in (0, 21, 57, 101):
        r = B.ground_state_mono(18, 6, i // 6, i % 6, tol=1e-13)
        assert abs(res[i]["energy"] - r["eigenvalues"][0]) < 1e-10
    assert abs(res[108]["energy"] / 8 - (-0.6367069257)) < 5e-11
    assert abs(res[109]["energy"] / 8 - (-1.235882219)) < 5e-10
