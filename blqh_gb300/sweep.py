"""Sweep driver: ground energies of many (J, K) sectors over a grid of layer
distances and tunnelling amplitudes, through the batched path (blqh_batch_*).

The reference keeps its sweeps as loops in its drivers (BLQH_without_spin/
main.cpp:77-115 over J and K at fixed d, :134-181 over d), each point a full
basis::init / set_hamil / coeff_explicit_update / diag /
eigenstates_reconstruction / ground_state_energy sequence, printing one line
per point. Here the points go to the GPU in waves (one persistent launch per
wave; a wave's CSRs and Krylov spaces are resident together), and the result
is a table that write_table() prints in the same "one line per point" spirit.
"""
from __future__ import annotations

import time

from . import VAL_FP32, Batch, Context, instance, instance_spin

# Config of the batched benchmark: Nphi = 12, Ne = 12 (6 + 6), every (J, K),
# d/l in {0.0, 0.2, ..., 3.0}, Delta_SAS in {0, 0.05, 0.1}, 150 Lanczos steps.
SWEEP12 = dict(nphi=12, nel=12, nel_up=6, ds=[round(0.2 * k, 10) for k in range(16)], sases=[0.0, 0.05, 0.1],
               lam=150)
# mixed into the same batch: every (J, K) of the spinful bilayer, Nphi = 6, Ne = 6
# (3 + 3 layers, 3 + 3 spins), Zeeman 0.02, bias 0.01, d/l = 1, Delta_SAS = 0.05
SWEEP12_SPIN = dict(nphi=6, nel=6, nel_up=3, nel_su=3, d=1.0, delta_sas=0.05, delta_v=0.01, delta_z=0.02)


def spin_points(nphi, nel, nel_up, nel_su, d, delta_sas, delta_v, delta_z):
    """(J, K) points of the spinful sweep and their instances."""
    pts = [(J, K) for J in range(nphi) for K in range(nphi)]
    return pts, [instance_spin(nphi, nel, nel_up, nel_su, J, K, d, delta_sas, delta_v, delta_z) for J, K in pts]


def sweep_points(nphi, nel, nel_up, ds, sases, Js=None, Ks=None, delta_v=0.0):
    """(J, K, d, Delta_SAS) points in the order J, K, d, Delta_SAS, and their instances."""
    Js = range(nphi) if Js is None else Js
    Ks = range(nphi) if Ks is None else Ks
    pts = [(J, K, d, s) for J in Js for K in Ks for d in ds for s in sases]
    return pts, [instance(nphi, nel, nel_up, J, K, d, s, delta_v) for (J, K, d, s) in pts]


def run_sweep(instances, lam=150, precision=VAL_FP32, wave=1728, graph=True, seed=1, ctx=None):
    """Solve every instance; returns dict(results=[...], create_s, solve_s, waves,
    lanczos_ms, finish_ms, launches).

    create_s: bases, CSRs and Krylov storage (blqh_batch_create); solve_s: the
    persistent Lanczos launch plus the finishers (blqh_batch_solve), summed
    over waves; both wall-clock seconds measured around the library calls.
    lanczos_ms / finish_ms: device time of those launches (CUDA events)."""
    ctx = ctx or Context.default()
    out, t_create, t_solve = [], 0.0, 0.0
    waves, lanczos_ms, finish_ms, launches = 0, 0.0, 0.0, 0
    for a in range(0, len(instances), wave):
        chunk = instances[a:a + wave]
        t0 = time.perf_counter()
        b = Batch(chunk, lam=lam, precision=precision, seed=seed, graph=graph, ctx=ctx)
        t1 = time.perf_counter()
        b.solve()
        t2 = time.perf_counter()
        out.extend(b.results())
        tm = b.timing() if any(r["dim"] for r in out[-len(chunk):]) else dict(lanczos_ms=0, finish_ms=0, launches=0)
        lanczos_ms += tm["lanczos_ms"]
        finish_ms += tm["finish_ms"]
        launches += tm["launches"]
        b.close()
        t_create += t1 - t0
        t_solve += t2 - t1
        waves += 1
    return dict(results=out, create_s=t_create, solve_s=t_solve, waves=waves, lanczos_ms=lanczos_ms,
                finish_ms=finish_ms, launches=launches)


def write_table(path, points, results, nel):
    """One line per point: J K d Delta_SAS dim steps E_gs E_gs/Ne."""
    with open(path, "w") as f:
        f.write("# J K d delta_sas dim steps E_gs E_gs_per_Ne\n")
        for (J, K, d, s), r in zip(points, results):
            f.write(f"{J} {K} {d:.4f} {s:.4f} {r['dim']} {r['steps']} {r['energy']:.12f} "
                    f"{r['energy'] / nel:.12f}\n")


# ---------------------------------------------------------------------------
# Excitation spectrum: every (J, K) sector of one filling at given layer
# distances, through the single-sector path (bases too large for the batched
# kernel's shared-memory vectors, e.g. Nphi = 14, dim 6e4).

# The all-sector configuration: Nphi = 14, Ne = 14 (7 + 7), d/l in {0.5, 1.0, 1.5}.
SPECTRUM14 = dict(nphi=14, nel_up=7, nel_down=7, ds=[0.5, 1.0, 1.5], lam=200)


def spectrum_momentum(nphi, J, K, gamma=1.0):
    """|K| of sector (J, K) as the reference's spectrum driver computes it
    (BLQH_without_spin/main.cpp:78-97): sqrt((s - s0)^2 + (t - t0)^2 gamma^2)
    sqrt(2 pi / (nphi gamma)) with t = J, s = K and t0 = s0 = nphi / 2
    (integer division, as in the reference)."""
    import math

    t0 = s0 = nphi // 2
    return math.sqrt((K - s0) ** 2 + ((J - t0) * gamma) ** 2) * math.sqrt(2.0 * math.pi / nphi / gamma)


def distinct_levels(eigenvalues, count=6, gap=1e-5):
    """The excited levels the reference's spectrum driver prints after
    eigenvalues[0] (BLQH_without_spin/main.cpp:103-110): walking up the Ritz
    values, each one more than `gap` above its predecessor, at most `count`
    (the walk stops at the end of the list, where the reference reads past it)."""
    out = []
    for i in range(1, len(eigenvalues)):
        if eigenvalues[i] - eigenvalues[i - 1] > gap:
            out.append(float(eigenvalues[i]))
            if len(out) >= count:
                break
    return out


def _solve_sectors(jobs, nphi, nel, nel_up, ds, lam, precision, gamma, device, rows, errors):
    from . import Basis, Hamiltonian, Lanczos

    try:
        ctx = Context(device)
        for J, K in jobs:
            b = Basis(nphi, nel, nel_up, J, K, ctx=ctx)
            if b.dim == 0:
                b.close()
                continue
            for d in ds:
                H = Hamiltonian(b, d, precision=precision, gamma=gamma)
                L = Lanczos(H, max_steps=min(lam, b.dim), tol=0.0)
                L.iterate()
                e, _ = L.eig()
                L.ritz_vector(copy=False)
                E = L.rayleigh_fp64() if precision == VAL_FP32 else L.rayleigh()
                rows.append(dict(J=J, K=K, d=d, momentum=spectrum_momentum(nphi, J, K, gamma), dim=b.dim,
                                 steps=L.steps, energy=E, eig0=float(e[0]), levels=distinct_levels(e)))
                L.close()
                H.close()
            b.close()
        ctx.synchronize()
    except Exception as exc:  # reported by run_spectrum
        errors.append(exc)


def run_spectrum(nphi, nel_up, nel_down, ds, lam=200, precision=VAL_FP32, Js=None, Ks=None, gamma=1.0,
                 streams=1, device=0):
    """Ground energy and the lowest distinct Ritz levels of every (J, K) sector
    at each layer distance in ds: the reference's excitation-spectrum loop
    (BLQH_without_spin/main.cpp:77-115) on the GPU. Each sector's basis is
    built once for all distances; the Lanczos runs lam steps (no early stop,
    as the reference's coeff_explicit_update), with full reorthogonalization.
    streams > 1 spreads the sectors over that many contexts (one CUDA stream
    each) driven from host threads, so small sectors overlap on the GPU.
    energy is the FP64 Rayleigh quotient (regenerated elements with FP32
    values); eig0 and levels are Ritz values of the stored matrix, so with FP32
    values they carry its rounding (~1e-7 relative).
    Returns the rows sorted by (d, J, K)."""
    import threading

    nel = nel_up + nel_down
    Js = range(nphi) if Js is None else Js
    Ks = range(nphi) if Ks is None else Ks
    sectors = [(J, K) for J in Js for K in Ks]
    rows, errors = [], []
    parts = [sectors[i::streams] for i in range(max(1, streams))]
    threads = [threading.Thread(target=_solve_sectors,
                                args=(p, nphi, nel, nel_up, ds, lam, precision, gamma, device, rows, errors))
               for p in parts if p]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise errors[0]
    rows.sort(key=lambda r: (r["d"], r["J"], r["K"]))
    return rows


def write_spectrum(path, rows, nel):
    """One line per (sector, d) in the reference driver's format
    (BLQH_without_spin/main.cpp:98-111): "t s K E_gs/Ne eigenvalues[0]" then the
    distinct excited levels; a comment line opens each layer distance."""
    with open(path, "w") as f:
        d_prev = None
        for r in rows:
            if r["d"] != d_prev:
                f.write(f"# d = {r['d']:g}\n")
                d_prev = r["d"]
            f.write(f"{r['J']} {r['K']} {r['momentum']:g} {r['energy'] / nel:g} {r['eig0']:g} "
                    + " ".join(f"{x:g}" for x in r["levels"]) + "\n")


# The spinful spectrum: Nphi = 6, Ne = 6 (3 + 3 layers, 3 spin up), the batched
# configuration's spinful parameters.
SPECTRUM_SPIN6 = dict(nphi=6, nel=6, nel_up=3, nel_su=3, d=1.0, delta_sas=0.05, delta_v=0.01, delta_z=0.02, lam=200)


def spin_sz(ids, psi, nphi, nel):
    """Sz of a spinful state as BLQH_with_spin/lanczos_hamiltonian.cpp:1246-1251:
    (2 <N_0 + N_2> - Ne) / (2 Ne), blocks 0 and 2 being the spin-up orbitals."""
    import numpy as np

    ids = np.asarray(ids, dtype=np.uint64)
    m = np.uint64((1 << nphi) - 1)
    up = np.zeros(len(ids))
    for blk in (0, 2):
        x = (ids >> np.uint64(blk * nphi)) & m
        up += np.array([bin(int(v)).count("1") for v in x], dtype=float)
    w = np.abs(np.asarray(psi)) ** 2
    return (2.0 * float(np.sum(up * w) / np.sum(w)) - nel) / (2.0 * nel)


def run_spectrum_spin(nphi, nel, nel_up, nel_su, d, delta_sas=0.0, delta_v=0.0, delta_z=0.0, lam=200, Js=None,
                      Ks=None, gamma=1.0, ctx=None):
    """The reference's spinful excitation-spectrum loop (BLQH_with_spin/main.cpp:145-178):
    sectors (t, s) in [0, nphi/2]^2, each with the ground energy, Sz, eigenvalues[0]
    and the distinct Ritz levels (lam Lanczos steps, no early stop, FP64 values)."""
    from . import Lanczos, basis_spin, hamiltonian_spin

    N = nphi // 2
    Js = range(N + 1) if Js is None else Js
    Ks = range(N + 1) if Ks is None else Ks
    rows = []
    for J in Js:
        for K in Ks:
            b = basis_spin(nphi, nel, nel_up, nel_su, J, K, ctx=ctx)
            if b.dim == 0:
                b.close()
                continue
            H = hamiltonian_spin(b, d, delta_sas, delta_v, delta_z, gamma=gamma)
            L = Lanczos(H, max_steps=min(lam, b.dim), tol=0.0)
            L.iterate()
            e, _ = L.eig()
            psi = L.ritz_vector()
            rows.append(dict(J=J, K=K, d=d, momentum=spectrum_momentum(nphi, J, K, gamma), dim=b.dim,
                             steps=L.steps, energy=L.rayleigh(), Sz=spin_sz(b.id, psi, nphi, nel),
                             eig0=float(e[0]), levels=distinct_levels(e)))
            L.close()
            H.close()
            b.close()
    return rows


def write_spectrum_spin(path, rows, nel):
    """One line per sector in the reference driver's format (BLQH_with_spin/
    main.cpp:164-176): "t s K E_gs/Ne Sz eigenvalues[0]" then the distinct levels."""
    with open(path, "w") as f:
        for r in rows:
            f.write(f"{r['J']} {r['K']} {r['momentum']:g} {r['energy'] / nel:g} {r['Sz']:g} {r['eig0']:g} "
                    + " ".join(f"{x:g}" for x in r["levels"]) + "\n")


# ---- monolayer drivers (the loops Monolayer/main.cpp keeps commented out, :120-195) ----
def mono_momentum(nphi, nel, J, K, gamma=1.0):
    """|K| of sector (J, K) in the monolayer spectrum driver (Monolayer/main.cpp:150-162):
    sqrt((J mod C - C/2)^2 + (K mod C - C/2)^2 gamma^2) sqrt(2 pi / (nphi gamma)), C = gcd(nel, nphi)
    (the driver's origin j0 = k0 = C/2, integer division, as its recorded output
    Monolayer/check/ek_nphi_18_nel_6 places it)."""
    import math

    C = math.gcd(nel, nphi)
    j0 = k0 = C // 2
    return math.sqrt((J % C - j0) ** 2 + ((K % C - k0) * gamma) ** 2) * math.sqrt(2.0 * math.pi / nphi / gamma)


def run_spectrum_mono(nphi, nel, gamma=1.0, Js=None, Ks=None, lam=400, count=10, ctx=None):
    """Every (J, K) of the monolayer: the sector's levels from a reorthogonalized Lanczos run to
    min(lam, dim) steps without a convergence stop (the whole Krylov space for small sectors),
    the lowest `count` distinct ones per sector. Monolayer/main.cpp:150-162 prints the 10 lowest
    eigenvalues of a dense solve instead, a degenerate level once per state."""
    import math

    import numpy as np

    from . import Lanczos, basis_mono, hamiltonian_mono

    C = math.gcd(nel, nphi)
    rows = []
    for J in (range(nphi) if Js is None else Js):
        for K in (range(C) if Ks is None else Ks):
            b = basis_mono(nphi, nel, J, K, ctx=ctx)
            if b.dim == 0:
                b.close()
                continue
            H = hamiltonian_mono(b, gamma)
            L = Lanczos(H, max_steps=min(lam, b.dim), tol=0.0)
            L.iterate()
            e, _ = L.eig()
            levels = [float(e[0])]
            for x in e[1:]:
                if x - levels[-1] > 1e-9 and len(levels) < count:
                    levels.append(float(x))
            rows.append(dict(J=J, K=K, dim=b.dim, momentum=mono_momentum(nphi, nel, J, K, gamma),
                             levels=np.array(levels)))
            L.close()
            H.close()
            b.close()
    return rows


def write_spectrum_mono(path, rows):
    """One line per sector as the monolayer driver prints it: "|K| e_0 e_1 ... " (cout's default
    6 significant digits, a space after every number)."""
    with open(path, "w") as f:
        for r in rows:
            f.write(f"{r['momentum']:g} " + "".join(f"{x:g} " for x in r["levels"]) + "\n")


def run_gs_energy_mono(nel, nphis=None, lam=600, ctx=None):
    """Ground energy per electron of the full space (no momentum filter) against filling
    (Monolayer/main.cpp:170-195): for each nphi, ly = sqrt(8 pi nphi / nel), lx = nel ly / 4;
    the reference loops nphi from 4 nel + 1 down to nel + 1. Rows (nu, E_gs / nel)."""
    from . import ground_state_mono

    nphis = list(range(4 * nel + 1, nel, -1)) if nphis is None else list(nphis)
    rows = []
    for nphi in nphis:
        r = ground_state_mono(nphi, nel, -1, -1, gamma=nel / 4.0, max_steps=lam, tol=1e-13, ctx=ctx)
        rows.append((nel * 1.0 / nphi, r["eigenvalues"][0] / nel))
    return rows


def write_gs_energy_mono(path, rows):
    """"nu E_gs/nel" per line, cout's default 6 significant digits (Monolayer/main.cpp:189)."""
    with open(path, "w") as f:
        for nu, e in rows:
            f.write(f"{nu:g} {e:g}\n")
