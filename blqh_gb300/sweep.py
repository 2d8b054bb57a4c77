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
