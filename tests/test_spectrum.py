"""The excitation-spectrum driver (blqh_gb300.sweep.run_spectrum): every (J, K)
sector of one filling, the reference's loop in BLQH_without_spin/main.cpp:77-115.
CPU: the momentum formula, the distinct-level walk and the line format; GPU: all
36 sectors of Nphi = 6 (3 + 3) at d = 1 against the reference's fixtures."""
import math
import os

import numpy as np
import pytest

from conftest import ROOT, golden

from blqh_gb300 import sweep as S


def test_momentum_matches_reference_formula():
    # main.cpp:97 with t0 = s0 = nphi / 2 (integer), gamma = 1
    for nphi in (6, 7, 14):
        for J in range(nphi):
            for K in range(nphi):
                t0 = s0 = nphi // 2
                want = math.sqrt((K - s0) ** 2 + (J - t0) ** 2) * math.sqrt(2 * math.pi / nphi)
                assert abs(S.spectrum_momentum(nphi, J, K) - want) < 1e-15
    g = 0.8
    assert abs(S.spectrum_momentum(10, 2, 7, g) - math.sqrt(4 + (3 * g) ** 2) * math.sqrt(2 * math.pi / 10 / g)) < 1e-15


def test_distinct_levels_walk():
    e = [-5.0, -5.0, -5.0 + 5e-6, -4.0, -4.0, -3.5, -3.0, -2.0, -1.0, 0.0, 1.0, 2.0]
    assert S.distinct_levels(e) == [-4.0, -3.5, -3.0, -2.0, -1.0, 0.0]
    assert S.distinct_levels(e, count=2) == [-4.0, -3.5]
    assert S.distinct_levels([-1.0, -1.0]) == []


def test_write_spectrum_format(tmp_path):
    rows = [dict(J=0, K=1, d=1.0, momentum=1.5, energy=-12.0, eig0=-12.0, levels=[-11.5, -11.0]),
            dict(J=1, K=1, d=1.5, momentum=0.5, energy=-6.0, eig0=-6.0, levels=[])]
    p = tmp_path / "ek.txt"
    S.write_spectrum(p, rows, nel=6)
    lines = p.read_text().splitlines()
    assert lines[0] == "# d = 1"
    assert lines[1].split() == ["0", "1", "1.5", "-2", "-12", "-11.5", "-11"]
    assert lines[2] == "# d = 1.5" and lines[3].split() == ["1", "1", "0.5", "-1", "-6"]


@pytest.mark.gpu
def test_spectrum_nphi6_all_sectors():
    import blqh_gb300 as B

    # Ritz values are eigenvalues of the stored matrix: FP64 values give the
    # reference's to 1e-10, FP32 values to the matrix rounding (~1e-7 relative);
    # the ground energy is the FP64 Rayleigh quotient in both cases.
    for prec, tol in ((B.VAL_FP32, 1e-6), (B.VAL_FP64, 1e-10)):
        rows = S.run_spectrum(6, 3, 3, [1.0], lam=200, precision=prec, streams=2)
        assert len(rows) == 36
        for r in rows:
            g = golden(f"n6_j{r['J']}_k{r['K']}")
            assert r["dim"] == len(g["id"])
            e_ref = np.asarray(g["eigenvalues"])
            assert abs(r["eig0"] - e_ref[0]) <= tol * max(1.0, abs(e_ref[0]))
            assert abs(r["energy"] - e_ref[0]) <= 1e-9
            # excited levels against the exact spectrum of the reference's own CSR:
            # its lambda = 200 > dim Lanczos without reorthogonalization also lists
            # spurious Ritz values between the true ones
            rp, col, val = g["row_ptr"], g["col"], g["val"]
            M = np.zeros((r["dim"], r["dim"]), np.complex128)
            for i in range(r["dim"]):
                M[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
            want = S.distinct_levels(np.linalg.eigvalsh(M))
            k = min(len(want), 6)
            assert len(r["levels"]) >= k
            assert np.allclose(r["levels"][:k], want[:k], atol=max(tol * 10, 1e-9))


def _spin_fixture(name):
    return np.load(os.path.join(ROOT, "tests", "golden", "spin", name + ".npz"), allow_pickle=True)


def test_spin_sz_matches_reference_values():
    """sweep.spin_sz on the reference's own psir_0 gives the reference's Sz()."""
    for name in ("s6_su4_j0_k0", "s6_up2_j1_k3", "s4_all_j0_k0", "s5_all_j0_k2"):
        g = _spin_fixture(name)
        nphi, nel = int(g["spec"][0]), int(g["spec"][1])
        assert abs(S.spin_sz(g["id"], g["psir0"], nphi, nel) - float(g["obs"][0])) <= 1e-12


@pytest.mark.gpu
def test_spin_spectrum_nphi6():
    """The spinful spectrum loop over (t, s) in [0, 3]^2 against the reference's
    dense spectra and Sz (its fixtures at the same parameters). The Krylov space
    is run to its full dimension (lam >= dim) so that every printed level is an
    exact eigenvalue; at the reference's lam = 200 < dim the higher Ritz values
    are still converging."""
    cfg = dict(S.SPECTRUM_SPIN6)
    rows = S.run_spectrum_spin(cfg["nphi"], cfg["nel"], cfg["nel_up"], cfg["nel_su"], cfg["d"], cfg["delta_sas"],
                               cfg["delta_v"], cfg["delta_z"], lam=1000)
    assert len(rows) == 16
    for r in rows:
        g = _spin_fixture(f"s6_j{r['J']}_k{r['K']}")
        ev = np.asarray(g["dense_eigenvalues"])
        assert r["dim"] == len(g["id"])
        assert abs(r["eig0"] - ev[0]) <= 1e-10 and abs(r["energy"] - ev[0]) <= 1e-10
        want = S.distinct_levels(ev)
        k = min(len(want), 6)
        assert len(r["levels"]) >= k and np.allclose(r["levels"][:k], want[:k], atol=1e-9)
        if ev[1] - ev[0] > 1e-6:
            assert abs(r["Sz"] - float(g["obs"][0])) <= 1e-8
