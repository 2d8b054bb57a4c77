"""The spinful model on the GPU (blqh_basis_build_spin, blqh_hamil_build_spin, and
spinful instances in the batch) against the reference's own outputs
(tests/golden/spin/, BLQH_with_spin compiled from its sources).

Tolerances: representatives, periods, row pointers and columns bit-exact;
values |dv| <= 2e-14 max(1, |v|); energies |dE| <= 1e-10 against the reference's
eigenvalues[0] (its Lanczos) and dense ED."""
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SPIN = os.path.join(ROOT, "tests", "golden", "spin")
NAMES = sorted(f[:-4] for f in os.listdir(SPIN) if f.endswith(".npz"))


@pytest.fixture(scope="module")
def B():
    import blqh_gb300 as B

    return B


def load(name):
    return dict(np.load(os.path.join(SPIN, name + ".npz")))


def spec(g):
    nphi, nel, nel_up, nel_su, J, K = (int(v) for v in g["spec"][:6])
    d, dsas, dv, dz = (float(v) for v in g["params"])
    return (nphi, nel, nel_up, nel_su, J, K), (d, dsas, dv, dz)


@pytest.mark.parametrize("name", NAMES)
def test_spin_basis_and_csr_bit_exact(B, name):
    g = load(name)
    sec, (d, dsas, dv, dz) = spec(g)
    b = B.basis_spin(*sec)
    assert b.dim == len(g["id"])
    assert np.array_equal(b.id, g["id"])
    assert np.array_equal(b.period, g["period"])
    if not b.dim:
        return
    H = B.hamiltonian_spin(b, d, dsas, dv, dz)
    rp, col, val = H.csr()
    assert np.array_equal(rp, g["row_ptr"])
    assert np.array_equal(col, g["col"])
    ref = g["val"] if H.is_complex else g["val"].real
    if not H.is_complex:
        assert np.max(np.abs(g["val"].imag), initial=0) < 1e-14
    assert np.all(np.abs(val - ref) <= 2e-14 * np.maximum(1.0, np.abs(ref)))


@pytest.mark.parametrize("name", NAMES)
def test_spin_ground_energy(B, name):
    g = load(name)
    sec, (d, dsas, dv, dz) = spec(g)
    b = B.basis_spin(*sec)
    if not b.dim:
        return
    H = B.hamiltonian_spin(b, d, dsas, dv, dz)
    L = B.Lanczos(H, max_steps=300, tol=1e-13, check_every=5)
    L.iterate()
    e, _ = L.eig()
    assert abs(e[0] - float(g["eigenvalues"][0])) <= 1e-10
    if "dense_eigenvalues" in g:
        assert abs(e[0] - float(g["dense_eigenvalues"][0])) <= 1e-10
    L.ritz_vector(copy=False)
    assert abs(L.rayleigh() - float(g["eigenvalues"][0])) <= 1e-10


def test_spin_batch_with_spinless(B):
    """The batched configuration's mix: spinful Nphi=6 sectors next to spinless ones, one launch."""
    from conftest import golden

    names = ["s6_j0_k0", "s6_j3_k3", "s6_j2_k5", "s6_j1_k0", "s4_all_j0_k0"]
    inst, ref = [], []
    for n in names:
        g = load(n)
        sec, (d, dsas, dv, dz) = spec(g)
        inst.append(B.instance_spin(*sec, d, dsas, dv, dz))
        ref.append(float(g["eigenvalues"][0]))
    gl = golden("n10_j5_k5_d1")
    inst.append(B.instance(10, 10, 5, 5, 5, 1.0))
    ref.append(float(gl["eigenvalues"][0]))
    for prec, tol in ((B.VAL_FP32, 1e-9), (B.VAL_FP64, 1e-10)):
        res = B.batch_run(inst, lam=150, precision=prec)
        e = np.array([r["energy"] for r in res])
        assert np.all(np.abs(e - np.array(ref)) <= tol), e - np.array(ref)


def test_spin_rep_min_is_orbit_minimum(B):
    from oracle import spin_ref as S

    b = B.basis_spin(6, 6, 3, 3, 1, 2, rep_mode=B.REP_MIN)
    g = load("s6_j1_k2")
    assert b.dim == len(g["id"])
    got = [int(c) for c in b.id]
    want = sorted(min(S.orbit(int(c), 6)) for c in g["id"])
    assert got == want


def test_spin_rejects_bad_input(B):
    with pytest.raises(B.BlqhError):
        B.basis_spin(16, 6, 3, 3, 0, 0)  # 4 nphi > 60
    b = B.basis_spin(6, 6, 3, 3, 0, 0)
    with pytest.raises(B.BlqhError):
        B.Hamiltonian(b, 1.0)  # spinless builder on a spinful basis


def _diag_observables(ids, period, nphi, K):
    """Per-state weights of the diagonal observables: upper_Sz, down_Sz and the 2 nphi
    occupations (translate-averaged), so that <O> = sum_i w_i |psi_i|^2."""
    mk = (1 << nphi) - 1
    n = [np.array([(int(x) >> (b * nphi)) & mk for x in ids], dtype=np.uint64) for b in range(4)]
    cnt = [np.array([bin(int(v)).count("1") for v in nb], float) for nb in n]
    up = (2.0 * cnt[0] - (cnt[0] + cnt[1])) / (2.0 * (cnt[0] + cnt[1]) + 1e-8)
    dn = (2.0 * cnt[2] - (cnt[2] + cnt[3])) / (2.0 * (cnt[2] + cnt[3]) + 1e-8)
    occ = np.zeros((2 * nphi, len(ids)))
    for i, x in enumerate(ids):
        D = 1 if K < 0 else int(period[i])
        for q in range(D):
            y = 0
            for b in range(4):  # rotate every block left by q (the translation; signs do not matter here)
                blk = (int(x) >> (b * nphi)) & mk
                y |= (((blk << q) | (blk >> (nphi - q))) & mk) << (b * nphi)
            for j in range(nphi):
                occ[j, i] += ((y >> j) & 1) / D
                occ[nphi + j, i] += ((y >> (nphi + j)) & 1) / D
    return [up, dn] + list(occ)


@pytest.mark.parametrize("name", [n for n in NAMES if "obs" in np.load(os.path.join(SPIN, n + ".npz")).files])
def test_spin_observables_on_gpu(B, name):
    """Sz, pseudospin_Sz, upper_Sz, down_Sz, pseudospin_Sx, spinflip_tunneling and the
    occupation numbers from the device kernel against the reference's own values
    (BLQH_with_spin/lanczos_hamiltonian.cpp:1217-1593), 1e-9. Many of these sectors
    (all of Nphi=6, 3+3, 3 spin up) have an exactly degenerate ground state; there
    the reference's upper_Sz, down_Sz and occupations belong to whichever vector of
    the ground space its unreorthogonalized recurrence ends on (rounding brings the
    second one in), so for those the device value must lie in the range the
    observable takes over the ground space (the eigenvalues of P^H O P, from the
    reference's own CSR), while Sz, pseudospin_Sz, pseudospin_Sx and
    spinflip_tunneling (equal over it) must match."""
    g = dict(np.load(os.path.join(SPIN, name + ".npz")))
    nphi, nel, nel_up, nel_su, J, K, lam, seed = (int(v) for v in g["spec"])
    d, dsas, dv, dz = (float(v) for v in g["params"])
    b = B.basis_spin(nphi, nel, nel_up, nel_su, J, K)
    H = B.hamiltonian_spin(b, d, dsas, dv, dz)
    L = B.Lanczos(H, max_steps=300, reorth=True, tol=1e-14, check_every=5, seed=1)
    L.iterate()
    L.eig()
    L.ritz_vector(copy=False)
    o = L.observables_spin(b)
    ref = g["obs"]
    rp, col, val = g["row_ptr"], g["col"], g["val"]
    M = np.zeros((b.dim, b.dim), np.complex128)
    for i in range(b.dim):
        M[i, col[rp[i]:rp[i + 1]]] = val[rp[i]:rp[i + 1]]
    e, V = np.linalg.eigh(M)
    P = V[:, np.abs(e - e[0]) < 1e-9]
    invariant = [o["Sz"], o["pseudospin_Sz"], o["pseudospin_Sx"], o["spinflip_tunneling"]]
    assert np.max(np.abs(np.array(invariant) - ref[[0, 1, 4, 5]])) < 1e-9
    state = [o["upper_Sz"], o["down_Sz"]] + list(o["occupation"].ravel())
    if P.shape[1] == 1:
        assert np.max(np.abs(np.array(state) - ref[[2, 3] + list(range(6, 6 + 2 * nphi))])) < 1e-9
    else:
        for got, w in zip(state, _diag_observables(g["id"], g["period"], nphi, K)):
            lo, hi = np.linalg.eigvalsh(P.conj().T @ (w[:, None] * P))[[0, -1]]
            assert lo - 1e-9 <= got <= hi + 1e-9, (got, lo, hi)


LARGE_DIR = os.path.join(ROOT, "tests", "golden", "spin_large")
LARGE = sorted(f[:-4] for f in os.listdir(LARGE_DIR) if f.endswith(".npz")) if os.path.isdir(LARGE_DIR) else []


@pytest.mark.parametrize("name", LARGE)
def test_spin_large_sector_against_reference(B, name):
    """Spinful sectors above 12 288 states (Nphi=8, Ne=8, 4+4 layers, 4 spin up:
    dim 16 046 and 16 024): basis digests, the whole CSR structure (SHA-256 of
    row_ptr and col), value checksums within 1e-12 relative, 256 sampled rows
    (columns bit-exact, values within 2e-14 max(1, |v|)), E_gs within 1e-10 of the
    reference's Lanczos, the observables that a degenerate ground space leaves
    unchanged within 1e-9 of the reference's, and the mixed-precision path (FP32 values, FP64 regenerated Rayleigh quotient) within 1e-9."""
    import hashlib

    g = dict(np.load(os.path.join(LARGE_DIR, name + ".npz")))
    nphi, nel, nel_up, nel_su, J, K, lam, seed = (int(v) for v in g["spec"])
    d, dsas, dv, dz = (float(v) for v in g["params"])
    b = B.basis_spin(nphi, nel, nel_up, nel_su, J, K)
    assert b.dim == int(g["dim"][0]) > 12288
    assert hashlib.sha256(b.id.astype(np.uint64).tobytes()).hexdigest() == str(g["id_sha"])
    assert hashlib.sha256(b.period.astype(np.int16).tobytes()).hexdigest() == str(g["period_sha"])
    H = B.hamiltonian_spin(b, d, dsas, dv, dz)
    assert H.nnz == int(g["nnz"][0])
    rp, col, val = H.csr()
    h = hashlib.sha256()
    h.update(rp.astype(np.int64).tobytes())
    h.update(col.astype(np.int64).tobytes())
    assert h.hexdigest() == str(g["csr_digest"])
    v = val.astype(np.complex128)
    w = (col % 7 + 1).astype(np.float64)
    got = np.array([v.sum(), np.abs(v).sum(), (v * w).sum()])
    assert np.all(np.abs(got - g["val_checks"]) <= 1e-12 * np.abs(g["val_checks"][1]))
    sel = np.concatenate([np.arange(rp[r], rp[r + 1]) for r in g["rows"]])
    assert np.array_equal(col[sel], g["row_col"])
    err = np.abs(v[sel] - g["row_val"])
    assert np.all(err <= 2e-14 * np.maximum(1.0, np.abs(g["row_val"])))
    e_ref = float(g["eigenvalues"][0])
    L = B.Lanczos(H, max_steps=300, reorth=True, tol=1e-13, check_every=5, seed=1)
    L.iterate()
    e, _ = L.eig()
    assert abs(e[0] - e_ref) <= 1e-10
    L.ritz_vector(copy=False)
    assert abs(L.rayleigh() - e_ref) <= 1e-10
    o = L.observables_spin(b)
    # the observables that are equal over a degenerate ground space (see test_spin_observables_on_gpu)
    got = [o["Sz"], o["pseudospin_Sz"], o["pseudospin_Sx"], o["spinflip_tunneling"]]
    assert np.max(np.abs(np.array(got) - g["obs"][[0, 1, 4, 5]])) < 1e-9
    L.close()
    H32 = B.hamiltonian_spin(b, d, dsas, dv, dz, precision=B.VAL_FP32)
    L32 = B.Lanczos(H32, max_steps=300, reorth=True, tol=1e-12, check_every=5, seed=1)
    L32.iterate()
    L32.eig()
    L32.ritz_vector(copy=False)
    assert abs(L32.rayleigh_fp64() - e_ref) <= 1e-9
