"""Ground-state observables on the GPU (blqh_lanczos_observables) against the
reference's own pseudospin_Sz, pseudospin_Sx and occupatation_number
(tests/golden/obs/, from BLQH_without_spin compiled from its sources).

Tolerance 1e-6: both sides evaluate an approximate ground state (the energy
converged to ~1e-12 leaves the vector accurate to ~1e-6)."""
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

OBS = os.path.join(ROOT, "tests", "golden", "obs")
NAMES = sorted(f[:-4] for f in os.listdir(OBS) if f.endswith(".npz"))


@pytest.mark.parametrize("name", NAMES)
def test_observables_match_reference(name):
    import blqh_gb300 as B

    g = dict(np.load(os.path.join(OBS, name + ".npz")))
    nphi, nel, nup, J, K = (int(v) for v in g["spec"])
    d, dsas, dv = (float(v) for v in g["params"])
    b = B.Basis(nphi, nel, nup, J, K)
    H = B.Hamiltonian(b, d, dsas, dv)
    L = B.Lanczos(H, max_steps=400, tol=1e-14, check_every=5)
    L.iterate()
    L.ritz_vector(copy=False)
    assert abs(L.rayleigh() - float(g["eigenvalues"][0])) <= 1e-10
    o = L.observables(b)
    assert abs(o["Sz"] - float(g["Sz"][0])) <= 1e-6, (o["Sz"], g["Sz"])
    assert abs(o["Sx"] - float(g["Sx"][0])) <= 1e-6, (o["Sx"], g["Sx"])
    assert np.max(np.abs(o["occupation"] - g["occupation"])) <= 1e-6
    # sum rules: the occupations add up to the electron number (upper layer: nel_up)
    assert abs(o["occupation"].sum() - nel) <= 1e-9
    if nup >= 0:
        assert abs(o["occupation"][0].sum() - nup) <= 1e-9


def test_lhamil_observables_methods():
    import blqh_gb300 as B

    L = B.lhamil(200, 1)
    L.sector.init(6, 6, -1, 3, 2)
    L.set_hamil(*B.torus(6), 6, 0, 1.0, 0.1, 0.05)
    L.coeff_explicit_update()
    L.diag()
    L.eigenstates_reconstruction()
    g = dict(np.load(os.path.join(OBS, "n6_all_j3_k2_sas.npz")))
    assert abs(L.pseudospin_Sz() - float(g["Sz"][0])) <= 1e-6
    assert abs(L.pseudospin_Sx() - float(g["Sx"][0])) <= 1e-6
    assert abs(L.occupatation_number(1, 2) - float(g["occupation"][1][2])) <= 1e-6
