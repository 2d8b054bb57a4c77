"""Pins the monolayer oracle against the reference's recorded outputs (CPU only).

Monolayer/check of the reference holds what its code printed: the 10 lowest
levels of every (J, K) sector of nphi = 18, nel = 6 (dense ED, square torus)
and the full-space ground energy per electron against filling for nel = 4, 5, 6
(aspect ratio nel / 4). tests/golden/make_golden_mono.py copied them into
tests/golden/mono/check.npz. Each printed value has 6 significant digits: the
tolerance is half a unit in the last printed place.
"""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN


def check():
    return dict(np.load(os.path.join(GOLDEN, "mono", "check.npz")))


def half_unit(v):
    """Half a unit in the 6th significant digit of v (the printed precision)."""
    e = math.floor(math.log10(abs(v)))
    return 0.5 * 10.0 ** (e - 5) + 1e-12


def test_ek_spectrum_nphi18_nel6(oracle):
    ek = check()["ek_nphi18_nel6"]
    assert ek.shape == (108, 11)
    lx, ly = oracle.mono_torus(18, 1.0)
    for idx, row in enumerate(ek):
        J, K = idx // 6, idx % 6
        B = oracle.MonoBasis(18, 6, J, K)
        H = oracle.MonoHamil(B, lx, ly)
        M = H.dense()
        assert np.abs(M - M.conj().T).max() < 1e-15
        ev = np.linalg.eigvalsh(M)[:10]
        for e, g in zip(ev, row[1:]):
            assert abs(e - g) <= half_unit(g), (J, K, e, g)


@pytest.mark.parametrize("nel", [4, 5, 6])
def test_full_space_ground_energy(oracle, nel):
    from scipy.sparse.linalg import eigsh

    gs = check()[f"gs_nel{nel}"]
    for nu, e_ref in gs:
        nphi = int(round(nel / nu))
        if math.comb(nphi, nel) > 20000:
            continue  # the GPU tests cover the larger spaces
        lx, ly = oracle.mono_torus(nphi, nel / 4.0)
        B = oracle.MonoBasis(nphi, nel)
        assert B.dim == math.comb(nphi, nel)
        H = oracle.MonoHamil(B, lx, ly)
        if B.dim <= 2000:
            e0 = np.linalg.eigvalsh(H.dense())[0]
        else:
            e0 = eigsh(H.sparse(), k=1, which="SA", tol=1e-12)[0][0]
        assert abs(e0 / nel - e_ref) <= half_unit(e_ref), (nphi, e0 / nel, e_ref)


def test_classical_energy_closed_form(oracle):
    """integral_1^inf t^-1/2 e^-zt dt = sqrt(pi / z) erfc(sqrt(z)); the reference integrates
    it numerically (GSL qagiu, 1e-6 tolerance), here the same QUADPACK-family quadrature
    (scipy quad on an infinite interval) agrees with the closed form to 3e-12 in E_cl."""
    from scipy.integrate import quad

    for nphi, gamma in ((18, 1.0), (23, 1.5), (9, 1.0)):
        lx, ly = oracle.mono_torus(nphi, gamma)
        e = -2.0
        for i in range(nphi):
            for j in range(nphi):
                if i or j:
                    z = (i * i * lx / ly + j * j * ly / lx) * math.pi
                    e += quad(lambda t: np.exp(-z * t) / np.sqrt(t), 1.0, np.inf, epsabs=1e-6, epsrel=1e-6,
                              limit=50000)[0]
        e /= math.sqrt(lx * ly)
        assert abs(oracle.mono_classical_energy(nphi, lx, ly) - e) < 3e-12


@pytest.mark.parametrize("nphi,nel", [(12, 4), (15, 5), (18, 6), (12, 6), (10, 4)])
def test_orbit_representatives(oracle, nphi, nel):
    """Every translation orbit of the J sector appears once per K (Monolayer/basis.cpp:66-89);
    periods are the smallest n with translate(id, n) == id (basis.cpp:110-118)."""
    C = math.gcd(nphi, nel)
    q = nphi // C
    mask = (1 << nphi) - 1
    for J in range(0, nphi, 3):
        full = set(int(c) for c in oracle.MonoBasis(nphi, nel, J, -1).id)
        B = oracle.MonoBasis(nphi, nel, J, 0)
        seen = set()
        for c, per in zip(B.id, B.period):
            c = int(c)
            orbit = {((c >> (q * n)) | (c << (nphi - q * n))) & mask for n in range(C)}
            assert not (orbit & seen)
            seen |= orbit
            p = next((n for n in range(1, C) if B.translate(c, n)[0] == c), C)
            assert per == p
        assert seen == full
        # the survivor choice depends only on J, not on K
        for K in range(1, C):
            assert np.array_equal(oracle.MonoBasis(nphi, nel, J, K).id, B.id)


def test_spectrum_driver_momentum_column():
    """The monolayer spectrum driver's |K| (blqh_gb300.sweep.mono_momentum, host code) prints the
    first column of Monolayer/check/ek_nphi_18_nel_6 exactly, line for line."""
    from blqh_gb300.sweep import mono_momentum

    ek = check()["ek_nphi18_nel6"]
    for idx, row in enumerate(ek):
        assert f"{mono_momentum(18, 6, idx // 6, idx % 6):g}" == f"{row[0]:g}"


def test_driver_line_formats(tmp_path):
    """write_gs_energy_mono / write_spectrum_mono print cout's default 6 significant digits: the
    reference's recorded lines come back unchanged when fed through the writers."""
    import numpy as np

    from blqh_gb300 import sweep as S

    gs = check()["gs_nel5"]
    S.write_gs_energy_mono(tmp_path / "gs.txt", [(nu, e) for nu, e in gs])
    assert (tmp_path / "gs.txt").read_text().splitlines() == [f"{nu:g} {e:g}" for nu, e in gs]
    ek = check()["ek_nphi18_nel6"][:4]
    rows = [dict(momentum=r[0], levels=np.array(r[1:])) for r in ek]
    S.write_spectrum_mono(tmp_path / "ek.txt", rows)
    for line, r in zip((tmp_path / "ek.txt").read_text().splitlines(), ek):
        assert [float(x) for x in line.split()] == [float(f"{v:g}") for v in r]
        assert line.endswith(" ")


@pytest.mark.parametrize("nphi,nel", [(12, 4), (15, 5), (18, 6)])
def test_smallest_member_convention(oracle, nphi, nel):
    """rep_mode 1 keeps the numerically smallest member of every orbit."""
    C = math.gcd(nphi, nel)
    q = nphi // C
    mask = (1 << nphi) - 1
    B = oracle.MonoBasis(nphi, nel, 0, 0, rep_mode=1)
    for c in B.id:
        c = int(c)
        orbit = {((c >> (q * n)) | (c << (nphi - q * n))) & mask for n in range(C)}
        assert c == min(orbit)
