"""Benchmark: K-sector time-to-E_gs of the spinless bilayer on one GB300.

Workload (one step = the whole exact-diagonalization path for one K-sector):
  Nphi = 16 orbitals per layer, Ne = 16 electrons (8 upper + 8 lower), square
  torus, lowest Landau level, (J, K) = (0, 0), d/l = 1.0, Delta_SAS = 0.05
  (a no-op with a fixed layer split, as in the reference), Delta_V = 0:
  basis (dim 647079) -> Hamiltonian CSR (2.39e8 nonzeros) -> Lanczos with full
  FP64 reorthogonalization until the lowest Ritz value moves < 1e-12 between
  checks -> ground state -> Rayleigh quotient.
  Mixed precision (default): FP32 CSR values, FP64 vectors / dots /
  reorthogonalization, final FP64 Rayleigh quotient with regenerated elements.
  The same path in all-FP64 runs in the same job for comparison.

Inputs are the physics parameters; the start vector is generated on the device
(value) or copied from pinned host memory (e2e). Every step rebuilds the CSR
(1.9-2.9 GB), larger than the 129 MB L2, so no L2 flush is needed.

Output: one JSON line (see the keys below). Under torchrun, each rank works on
its own sector (J = rank mod Nphi, K = 0): independent K-sectors, no data-path
collective ("scaling": "weak"); rank 0 prints the max-over-ranks timing.

--impl reference: the reference's CPU algorithm (the oracle restatement in
oracle/, the only CPU implementation that runs on the GPU machine) on a bounded
sample of the same workload, extrapolated to one sector.

Other workloads, each its own JSON line (--workload): sweep12 (the batched
Nphi=12 sweep of every (J, K) x 16 d x 3 Delta_SAS plus the spinful Nphi=6
sectors), learned14 (the learned start vector at Nphi=14), spectrum14 (every
(J, K) of Nphi=14 at three layer distances, 200 Lanczos steps each) and mono30
(one monolayer K-sector, Nphi=30, Ne=10).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NPHI, NEL, NUP, K_SEC, D, DSAS, DV = 16, 16, 8, 0, 1.0, 0.05, 0.0
MAX_STEPS, TOL, CHECK = 300, 1e-12, 10
REF_STEPS = 200  # the reference's lambda (init.cpp:34): pass 1 + reconstruction pass + Rayleigh quotient


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


SPMV_KERNELS = {
    0: ("k_spmv_df_v4 (CSR rows, FP32 values / FP64 x, y)", "spmv_nphi16.md"),
    1: ("k_spmv_blocked (row blocks x column tiles, FP32 values, x tiles in shared memory)", "spmv_blocked_nphi16.md"),
    2: ("k_spmv_ring (row blocks x 4096-column tiles; each tile's x and entry stream brought into shared memory "
        "by bulk copies; 4-byte entries: column | index into a shared-memory table of the distinct FP32 values)",
        "spmv_ring_nphi16.md"),
}


def traffic_from_profile(prec_name, layout=0):
    """DRAM bytes per SpMV launch from the committed ncu summary of the kernel that ran."""
    path = os.path.join(ROOT, "profiles", SPMV_KERNELS.get(layout, SPMV_KERNELS[0])[1])
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(rf"traffic_per_launch_{prec_name}_bytes:\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.tmp = None

    def __enter__(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=self.tmp,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            with open(self.tmp.name) as f:
                for line in f:
                    parts = [p.strip() for p in line.split(",")]
                    if len(parts) >= 8:
                        rows.append(parts)
            os.unlink(self.tmp.name)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clocks unavailable"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def rank_sector(rank, nphi):
    """The K-sector momentum J a rank solves: every rank its own sector ("weak"
    scaling), no data crosses ranks."""
    return rank % nphi


def max_over_ranks(pg, v):
    if pg is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


# ---------------------------------------------------------------------------
def stride_rows(dim, n, seed):
    """n row indices spread over [0, dim): a seeded offset in [0, dim // n), then every dim // n."""
    import numpy as np

    step = max(1, dim // n)
    off = int(np.random.default_rng(seed).integers(step))
    return off + step * np.arange(min(n, dim), dtype=np.int64)


def cpu_sample(frac=0.01, copies=10, spmv_reps=5, threads=None, seed=1, basis=None):
    """The oracle (the reference's algorithm restated in C++, OpenMP over rows) on a
    bounded sample of one sector, scaled to the reference's whole run (basis + every
    Hamiltonian row + 2 lambda + 1 complex products, lambda = 200):
      * the basis, whole (its time is measured, not scaled; `basis` = (handle,
        seconds) reuses one already measured);
      * a fraction `frac` of the rows by seeded stride over the whole row range,
        timed and scaled by dim / rows;
      * products timed over `copies` distinct replicas of those rows (several times
        the host's last-level cache, so the matrix streams from DRAM like the whole
        sector's 5.8 GB while x is gathered over the whole sector), scaled per
        nonzero to the sector's nonzeros (estimated as the sampled rows' mean length
        times dim)."""
    from oracle import oracle as O

    threads = threads or os.cpu_count() or 1
    if basis is None:
        t0 = time.perf_counter()
        B = O.Basis(NPHI, NEL, NUP, 0, K_SEC)
        t_basis = time.perf_counter() - t0
    else:
        B, t_basis = basis
    rows = stride_rows(B.dim, max(1, int(B.dim * frac)), seed)
    t1 = time.perf_counter()
    H = O.Hamil(B, D, DSAS, DV, nthreads=threads, rows=rows)
    t_rows = time.perf_counter() - t1
    t_prod = H.spmv_stream_time(copies, spmv_reps)
    nnz_est = H.nnz * B.dim / len(rows)
    rows_factor = B.dim / len(rows)
    spmv_factor = nnz_est / (copies * H.nnz)
    t_build = t_rows * rows_factor
    t_spmv = t_prod * spmv_factor
    total = t_basis + t_build + (2 * REF_STEPS + 1) * t_spmv
    return {
        "value": 1.0 / total, "unit": "K-sectors/s", "cores": threads, "kind": "port",
        "time_to_egs_s": total,
        "sample": (f"oracle/blqh_oracle.cpp (reference algorithm, OpenMP {threads} threads): whole basis "
                   f"({t_basis:.1f} s, measured); {len(rows)} Hamiltonian rows by seeded stride ({frac:.2%} of "
                   f"{B.dim}, {t_rows:.2f} s, x{rows_factor:.0f}); complex products over {copies} replicas of those "
                   f"rows ({copies * H.nnz / 1e6:.1f} M nonzeros, {t_prod * 1e3:.0f} ms each, x{spmv_factor:.1f} "
                   f"by nonzeros); whole run = basis + all rows + {2 * REF_STEPS + 1} products "
                   f"(lambda={REF_STEPS} pass 1 + reconstruction + Rayleigh quotient)"),
        "extrapolation": {"rows_factor": rows_factor, "spmv_nnz_factor": spmv_factor},
        "stages_s": {"basis": t_basis, "rows_sample": t_rows, "build_extrapolated": t_build,
                     "spmv_each_extrapolated": t_spmv, "spmv_sample_each": t_prod},
        "_basis": (B, t_basis),
    }


def run_reference(args, world, rank, pg):
    """The reference's CPU algorithm (the oracle port, all host threads) on the same
    workload: the basis is built and timed once; every step then times a fresh 1 %
    row sample (a different seeded stride) and the products over its replicas, and
    the line reports the mean of the steps' whole-run estimates."""
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    import oracle.oracle as O

    O.build()
    vals, last, basis = [], None, None
    for it in range(args.warmup + args.steps):
        r = cpu_sample(threads=threads, seed=1 + it, basis=basis)
        basis = r["_basis"]
        if it >= args.warmup:
            vals.append(r["value"])
        last = r
    v = statistics.mean(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "K-sectors/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic (physics parameters only)",
        "config": CONFIG,
        "cpu_baseline": {k: last[k] for k in ("kind", "cores", "sample")} | {"value": v, "unit": "K-sectors/s"},
        "e2e": {"value": v, "unit": "K-sectors/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "time_to_egs_s": 1.0 / v, "stages_s": last["stages_s"], "extrapolation": last["extrapolation"],
        "spread": {"min": min(vals), "max": max(vals)},
    }
    print(json.dumps(line), flush=True)
    return 0


METRIC = "K-sector time-to-E_gs and SpMV GB/s, mixed vs FP64 Lanczos at |dE|<1e-9"
CONFIG = {"workload": "spinless bilayer Nphi=16 Ne=16 (8+8) (J,K)=(0,0) d=1.0 Delta_SAS=0.05: basis -> CSR -> "
                      "Lanczos (full FP64 reorth, tol 1e-12) -> Rayleigh quotient",
          "nphi": NPHI, "nel": NEL, "nel_up": NUP, "dim": 647079, "parallelism": "independent K-sectors per GPU",
          "l2": "inputs larger than L2 (CSR rebuilt every step, 1.9-2.9 GB)"}


def run_ours(args, world, rank, local, pg):
    import numpy as np

    import blqh_gb300 as B

    nphi, nel, nup = args.nphi, args.nel, args.nup
    J = rank_sector(rank, nphi)
    prec = B.VAL_FP32 if args.precision == "mixed" else B.VAL_FP64
    ctx = B.Context(local)

    def step(precision, start=None, psi=None, rng=2):
        return B.ground_state(nphi, nel, nup, J, args.k, D, DSAS, DV, precision=precision, max_steps=args.max_steps,
                              tol=TOL, check_every=CHECK, seed=1, rng=rng, start=start, want_psi=psi is not None,
                              ctx=ctx)

    for _ in range(args.warmup):
        step(prec)
    # ---- value: device-resident path, device-timed ----
    ctx.timers(True)
    ctx.reset_timers()
    gpu_index = local
    cvd = os.environ.get("CUDA_VISIBLE_DEVICES")
    if cvd:
        try:
            gpu_index = int(cvd.split(",")[local])
        except Exception:
            pass
    barrier(pg)
    ctx.synchronize()
    results = []
    with ClockSampler(gpu_index) as clk:
        ctx.mark(0)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            results.append(step(prec))
        ctx.mark(1)
        ctx.synchronize()
        t1 = time.perf_counter()
    barrier(pg)
    dev_ms = ctx.elapsed_ms(0, 1)
    tm = ctx.timers(False)
    clocks = clk.summary()
    step_s = max_over_ranks(pg, dev_ms / 1e3 / args.steps)
    wall_step_s = max_over_ranks(pg, (t1 - t0) / args.steps)
    launches = sum(v[1] for v in tm.values())
    # ---- SpMV roofline over the timed region ----
    r0 = results[-1]
    nnz, dim = r0["nnz"], r0["dim"]
    cplx_sec = not (args.k <= 0 or 2 * args.k == nphi)
    sv = (4 if prec == B.VAL_FP32 else 8) * (2 if cplx_sec else 1)
    bytes_spmv = nnz * (sv + 4) + (dim + 1) * 8 + 2 * dim * (16 if cplx_sec else 8)
    spmv_ms, spmv_n = tm["spmv"]
    spmv_avg_s = spmv_ms / 1e3 / max(spmv_n, 1)
    achieved = bytes_spmv / spmv_avg_s / 1e9
    peak, peak_kind = peaks()
    if args.profile:
        # the same steps, nothing else: the command the ncu summaries in profiles/ run
        if rank == 0:
            print(json.dumps({"profile": True, "nphi": nphi, "dim": dim, "nnz": nnz, "steps": r0["steps"],
                              "ms_per_step": step_s * 1e3, "spmv_gbs": achieved,
                              "kernel_ms": {k: v[0] for k, v in tm.items()},
                              "launches": {k: v[1] for k, v in tm.items()}}), flush=True)
        return 0
    # ---- FP64 comparison on the same GPU ----
    r64 = []
    ctx.mark(2)
    for _ in range(max(1, args.steps // 2)):
        r64.append(step(B.VAL_FP64))
    ctx.mark(3)
    fp64_step_s = ctx.elapsed_ms(2, 3) / 1e3 / len(r64)
    # ---- the configuration's complex sector, (J, K) = (J, 1): mixed and FP64 ----
    cplx = {}
    if args.k == K_SEC and nphi == NPHI:
        def stepk(precision):
            return B.ground_state(nphi, nel, nup, J, 1, D, DSAS, DV, precision=precision, max_steps=args.max_steps,
                                  tol=TOL, check_every=CHECK, seed=1, rng=2, ctx=ctx)
        stepk(prec)
        ctx.mark(4)
        rc = stepk(prec)
        ctx.mark(5)
        rc64 = stepk(B.VAL_FP64)
        ctx.mark(6)
        cplx = {"sector": f"(J,K)=({J},1), complex", "dim": rc["dim"], "nnz": rc["nnz"],
                "lanczos_steps": rc["steps"], "time_to_egs_s": ctx.elapsed_ms(4, 5) / 1e3,
                "fp64_time_to_egs_s": ctx.elapsed_ms(5, 6) / 1e3, "E_gs": rc["energy"], "E_gs_fp64": rc64["energy"],
                "abs_dE_mixed_vs_fp64": abs(rc["energy"] - rc64["energy"])}
    # ---- e2e: public API with host buffers ----
    dtype = np.float64
    try:
        import torch

        start_h = torch.empty(dim, dtype=torch.float64, pin_memory=True).numpy()
        psi_h = torch.empty(dim, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        start_h = np.empty(dim, dtype)
        psi_h = np.empty(dim, dtype)
    start_h[:] = B.start_vector(dim, 1, 0, False)
    barrier(pg)
    te0 = time.perf_counter()
    for _ in range(args.steps):
        B.ground_state(nphi, nel, nup, J, args.k, D, DSAS, DV, precision=prec, max_steps=args.max_steps, tol=TOL,
                       check_every=CHECK, start=start_h, psi_out=psi_h, ctx=ctx)
    te1 = time.perf_counter()
    barrier(pg)
    e2e_step_s = max_over_ranks(pg, (te1 - te0) / args.steps)
    e_mixed = r0["energy"]
    e_fp64 = r64[-1]["energy"]
    # which SpMV kernel the timed steps used (the tuner's choice, cached per matrix class)
    layout = 0
    acc_cmp = None
    if prec == B.VAL_FP32:
        hb = B.Basis(nphi, nel, nup, J, args.k, ctx=ctx)
        hh = B.Hamiltonian(hb, D, DSAS, DV, precision=prec)
        hl = B.Lanczos(hh, max_steps=2, tol=0)
        layout = hh.spmv_layout()
        # the same FP32 matrix with native FP64 accumulation (accumulate = 1): 20 Lanczos products
        ha = B.Lanczos(hh, max_steps=20, tol=0, accumulate=1, rng=2)
        ctx.timers(True)
        ctx.reset_timers()
        ha.iterate()
        ctx.synchronize()
        ta = ctx.timers(False)
        acc_cmp = {"double_float_ms_per_product": spmv_avg_s * 1e3,
                   "native_fp64_fma_ms_per_product": ta["spmv"][0] / max(ta["spmv"][1], 1)}
        ha.close()
        hl.close()
        hh.close()
        hb.close()
    traffic = traffic_from_profile("fp32" if prec == B.VAL_FP32 else "fp64", layout) if not cplx_sec else None
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_sample()
    if rank != 0:
        return 0
    value = world / step_s
    line = {
        "metric": METRIC, "value": value, "unit": "K-sectors/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-values/f64-vectors" if prec == B.VAL_FP32 else "f64",
        "data": "synthetic (physics parameters only; no dataset exists)", "config": CONFIG,
        "time_to_egs_s": step_s, "wall_s_per_step": wall_step_s, "fp64_time_to_egs_s": fp64_step_s,
        "mixed_over_fp64_time": step_s / fp64_step_s,
        "E_gs": e_mixed, "E_gs_fp64": e_fp64, "abs_dE_mixed_vs_fp64": abs(e_mixed - e_fp64),
        "E_gs_per_Ne": e_mixed / NEL, "lanczos_steps": r0["steps"], "nnz": nnz, "dim": dim,
        "spmv_gbs": achieved,
        "roofline": {"kernel": SPMV_KERNELS[layout][0] if prec == B.VAL_FP32 else "k_spmv (FP64)",
                     "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "bytes_per_launch": bytes_spmv, "avg_launch_ms": spmv_avg_s * 1e3, "launches": spmv_n,
                     "traffic": traffic}, 
        "kernel_ms": {k: v[0] for k, v in tm.items()},
        "spmv_accumulation": acc_cmp,
        "complex_sector": cplx,
        "e2e": {"value": world / e2e_step_s, "unit": "K-sectors/s", "h2d_bytes_per_step": dim * 8,
                "d2h_bytes_per_step": dim * 8 + 8, "s_per_step": e2e_step_s},
        "gpu_launches": launches,
        "clocks": clocks,
        "cpu_baseline": cpu and {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample", "extrapolation")},
        "cpu_time_to_egs_s": cpu and cpu["time_to_egs_s"],
    }
    if traffic:  # the same launches measured on the DRAM bytes they actually move (ncu)
        line["roofline"]["frac_dram"] = traffic / spmv_avg_s / 1e9 / peak
    print(json.dumps(line), flush=True)
    return 0


def fp64_peak_gflops():
    """cuBLAS FP64 GEMM (torch.matmul, 4096^3, best of 3): the FP64 denominator."""
    import torch

    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    best = 1e9
    for _ in range(4):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2 * 4096 ** 3 / (best * 1e-3) / 1e9


def batch_fp64_flops(kinds, results):
    """FP64 floating-point operations of the reorthogonalization and Ritz vector per
    instance as the batched kernel does them: step j takes dot products with and
    updates against the j+1 stored vectors plus the 1-2 vectors of the three-term
    step (2 flops per real product, 8 per complex), repeated passes counted.
    kinds: (nphi, K) per instance."""
    total = 0.0
    for (nphi, K), r in zip(kinds, results):
        if not r["dim"]:
            continue
        cplx = not (K <= 0 or 2 * K == nphi)
        f = 8 if cplx else 2
        m = r["steps"]
        vecs = sum((j + 1) + (2 if j > 0 else 1) for j in range(m))
        vecs += r["second_passes"] * m  # bound: a repeated pass covers at most m vectors
        total += 2.0 * vecs * r["dim"] * f + 2.0 * m * r["dim"] * (2 if cplx else 1)
    return total


def cpu_sample_sweep(nphi, nel, nup, lam, n_instances, threads=None):
    """The oracle on one complex instance of the sweep (basis, all rows, 10 SpMVs),
    extrapolated to the reference's per-point work (basis + rows + 2 lambda + 1
    products) and to every instance of the sweep."""
    import numpy as np

    from oracle import oracle as O

    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    Bo = O.Basis(nphi, nel, nup, 1, 1)
    t1 = time.perf_counter()
    H = O.Hamil(Bo, 1.0, 0.05, 0.0, nthreads=threads)
    t2 = time.perf_counter()
    x = np.ones(Bo.dim, np.complex128)
    for _ in range(10):
        H.spmv(x)
    t3 = time.perf_counter()
    per = (t1 - t0) + (t2 - t1) + (2 * lam + 1) * (t3 - t2) / 10
    return {"value": 1.0 / per, "unit": "instances/s", "cores": threads, "kind": "port",
            "sweep_s_extrapolated": per * n_instances,
            "sample": (f"oracle/blqh_oracle.cpp (reference algorithm, OpenMP {threads} threads) on one instance "
                       f"(Nphi={nphi}, (J,K)=(1,1), dim {Bo.dim}): basis {t1 - t0:.2f} s, all rows {t2 - t1:.2f} s, "
                       f"10 complex SpMVs; extrapolated to 2*{lam}+1 SpMVs per instance and {n_instances} "
                       f"instances"),
            "sample_wall_s": t3 - t0}


def run_sweep_workload(args):
    """The batched sweep: Nphi=12, 6+6, every (J, K) x 16 d/l x 3 Delta_SAS = 6912
    instances, 150 Lanczos steps each, FP32 values / FP64 vectors (and the same
    sweep with FP64 values for comparison). One step = the whole sweep."""
    import numpy as np

    import blqh_gb300 as B
    from blqh_gb300 import sweep as S

    cfg = dict(S.SWEEP12)
    pts, inst = S.sweep_points(cfg["nphi"], cfg["nel"], cfg["nel_up"], cfg["ds"], cfg["sases"])
    spts, sinst = S.spin_points(**S.SWEEP12_SPIN)
    kinds = [(cfg["nphi"], K) for (J, K, d, s) in pts] + [(S.SWEEP12_SPIN["nphi"], K) for (J, K) in spts]
    inst = sinst + inst  # the spinful instances ride in the first wave
    kinds = kinds[len(pts):] + kinds[:len(pts)]
    lam = cfg["lam"]
    ctx = B.Context.default()
    for _ in range(max(args.warmup, 1)):
        S.run_sweep(inst[:304], lam=lam, ctx=ctx)
    with ClockSampler(0) as cs:
        runs = [S.run_sweep(inst, lam=lam, ctx=ctx) for _ in range(max(args.steps, 1))]
    clocks = cs.summary()
    r64 = S.run_sweep(inst, lam=lam, precision=B.VAL_FP64, ctx=ctx)
    run = min(runs, key=lambda r: r["solve_s"])
    e32 = np.array([r["energy"] for r in run["results"]])
    e64 = np.array([r["energy"] for r in r64["results"]])
    ok = ~np.isnan(e64)
    flops = batch_fp64_flops(kinds, run["results"])
    peak = fp64_peak_gflops()
    achieved = flops / (run["lanczos_ms"] * 1e-3) / 1e9
    n = len(inst)
    line = {
        "metric": "batched sweep: instances to E_gs per second (mixed precision, FP64 regenerated finisher)",
        "workload": "sweep12",
        "value": n / run["solve_s"], "unit": "instances/s", "n_gpus": 1, "steps": len(runs),
        "warmup": max(args.warmup, 1), "higher_is_better": True, "dtype": "f32 values / f64 vectors",
        "data": "synthetic (physics parameters only)",
        "config": {"workload": (f"Nphi={cfg['nphi']} Ne={cfg['nel']} ({cfg['nel_up']}+{cfg['nel'] - cfg['nel_up']}) "
                                f"all {cfg['nphi']}x{cfg['nphi']} (J,K) x d/l 0.0..3.0 step 0.2 x Delta_SAS "
                                f"{cfg['sases']}, plus the spinful Nphi=6 Ne=6 (3+3, 3 spin up) bilayer, all 36 "
                                f"(J,K), Zeeman 0.02, Delta_V 0.01; lambda={lam}"), "instances": n,
                   "spinful_instances": len(sinst), "waves": run["waves"],
                   "l2": "inputs larger than L2 (each wave holds ~45 GB of CSRs and Krylov spaces)"},
        "sweep_solve_s": run["solve_s"], "sweep_create_s": run["create_s"],
        "fp64_sweep_solve_s": r64["solve_s"], "fp64_over_mixed_solve": r64["solve_s"] / run["solve_s"],
        "max_abs_dE_mixed_vs_fp64": float(np.max(np.abs(e32[ok] - e64[ok]))),
        "roofline": {"kernel": "k_batch_lanczos (reorthogonalization + Ritz vector in FP64)", "bound": "fp64",
                     "achieved": achieved, "peak": peak, "unit": "GFLOP/s", "frac": achieved / peak,
                     "peak_source": "measured (cuBLAS FP64 GEMM through torch.matmul, 4096^3)",
                     "flops": flops, "lanczos_ms": run["lanczos_ms"], "finish_ms": run["finish_ms"]},
        "e2e": {"value": n / (run["create_s"] + run["solve_s"]), "unit": "instances/s",
                "h2d_bytes_per_step": n * ctypes_sizeof_instance(), "d2h_bytes_per_step": n * 48},
        "gpu_launches": run["launches"], "clocks": clocks,
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_sample_sweep(cfg["nphi"], cfg["nel"], cfg["nel_up"], lam, n)
    print(json.dumps(line), flush=True)
    return 0


def cpu_sample_spectrum(nphi, nel, nup, lam, n_sectors, n_ds, frac=0.1, copies=10, spmv_reps=5, threads=None,
                        seed=1):
    """The oracle on one complex sector of the spectrum, sampled as cpu_sample does
    (whole basis; a fraction `frac` of the rows by seeded stride, scaled by dim /
    rows; complex products over `copies` replicas of those rows, scaled per
    nonzero), extrapolated to the reference's per-point work (basis once per
    sector, all rows and 2 lambda + 1 products per layer distance) and to every
    point of the spectrum."""
    from oracle import oracle as O

    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    Bo = O.Basis(nphi, nel, nup, 1, 1)
    t_basis = time.perf_counter() - t0
    rows = stride_rows(Bo.dim, max(1, int(Bo.dim * frac)), seed)
    t1 = time.perf_counter()
    H = O.Hamil(Bo, 1.0, nthreads=threads, rows=rows)
    t_rows = time.perf_counter() - t1
    t_prod = H.spmv_stream_time(copies, spmv_reps)
    rows_factor = Bo.dim / len(rows)
    spmv_factor = (H.nnz * rows_factor) / (copies * H.nnz)
    t_build = t_rows * rows_factor
    t_spmv = t_prod * spmv_factor
    per_sector = t_basis + n_ds * (t_build + (2 * lam + 1) * t_spmv)
    total = per_sector * n_sectors
    return {"value": n_sectors * n_ds / total, "unit": "points/s", "cores": threads, "kind": "port",
            "spectrum_s_extrapolated": total,
            "sample": (f"oracle/blqh_oracle.cpp (reference algorithm, OpenMP {threads} threads) on one sector "
                       f"(Nphi={nphi}, (J,K)=(1,1), dim {Bo.dim}): basis {t_basis:.2f} s (measured); {len(rows)} "
                       f"rows by seeded stride ({frac:.0%}, {t_rows:.2f} s, x{rows_factor:.0f}); complex products "
                       f"over {copies} replicas of those rows ({t_prod * 1e3:.1f} ms each, x{spmv_factor:.1f} by "
                       f"nonzeros); per point all rows + 2*{lam}+1 products, {n_ds} distances per sector, "
                       f"{n_sectors} sectors"),
            "sample_wall_s": time.perf_counter() - t0}


def run_spectrum_workload(args):
    """The all-sector spectrum: Nphi=14, 7+7, every (J, K) x d/l in {0.5, 1.0, 1.5},
    lambda = 200 Lanczos steps each (no early stop, as the reference), the ground
    energy (FP64 regenerated Rayleigh quotient) and the lowest distinct Ritz
    levels per point. One step = the whole spectrum."""
    import numpy as np

    import blqh_gb300 as B
    from blqh_gb300 import sweep as S

    cfg = dict(S.SPECTRUM14)
    nphi, nup, ndn, ds, lam = cfg["nphi"], cfg["nel_up"], cfg["nel_down"], cfg["ds"], cfg["lam"]
    nel = nup + ndn
    streams = args.streams
    for _ in range(max(args.warmup, 1)):
        S.run_spectrum(nphi, nup, ndn, ds, lam=lam, Js=[0], Ks=range(streams), streams=streams)
    walls, rows = [], None
    with ClockSampler(0) as cs:
        for _ in range(max(args.steps, 1)):
            t0 = time.perf_counter()
            rows = S.run_spectrum(nphi, nup, ndn, ds, lam=lam, streams=streams)
            walls.append(time.perf_counter() - t0)
    clocks = cs.summary()
    wall = min(walls)
    n = len(rows)
    # FP64 values at d/l = 1.0 for the precision check
    r64 = S.run_spectrum(nphi, nup, ndn, [1.0], lam=lam, precision=B.VAL_FP64, streams=streams)
    e64 = {(r["J"], r["K"]): r["energy"] for r in r64}
    dE = max(abs(r["energy"] - e64[(r["J"], r["K"])]) for r in rows if r["d"] == 1.0)
    # roofline of the SpMV on one complex sector (CUDA events on the context stream)
    ctx = B.Context(0)
    ctx.timers(True)
    b = B.Basis(nphi, nel, nup, 1, 1, ctx=ctx)
    H = B.Hamiltonian(b, 1.0, precision=B.VAL_FP32)
    L = B.Lanczos(H, max_steps=lam, tol=0.0)
    ctx.reset_timers()
    L.iterate()
    ctx.synchronize()
    tm = ctx.timers(False)
    blocked = H.spmv_layout() == 1
    spmv_ms, spmv_n = tm["spmv"]
    nnz, dim = H.nnz, b.dim
    bytes_spmv = nnz * (8 + 4) + (dim + 1) * 8 + 2 * dim * 16
    achieved = bytes_spmv / (spmv_ms / 1e3 / max(spmv_n, 1)) / 1e9
    peak, peak_kind = peaks()
    L.close()
    H.close()
    b.close()
    line = {
        "metric": "all-sector spectrum: (sector, d) points to E_gs and levels per second (mixed precision)",
        "workload": "spectrum14", "value": n / wall, "unit": "points/s", "n_gpus": 1, "steps": len(walls),
        "warmup": max(args.warmup, 1), "higher_is_better": True, "dtype": "f32 values / f64 vectors",
        "data": "synthetic (physics parameters only)",
        "config": {"workload": (f"Nphi={nphi} Ne={nel} ({nup}+{ndn}) all {nphi}x{nphi} (J,K) x d/l {ds}; "
                                f"lambda={lam} Lanczos steps per point, full FP64 reorthogonalization"),
                   "points": n, "streams": streams, "l2": "each sector's CSR (~120-190 MB) and Krylov space "
                   "(~100-190 MB) exceed L2"},
        "spectrum_s": wall, "max_abs_dE_mixed_vs_fp64_at_d1": dE,
        "roofline": {"kernel": ("k_spmv_blocked" if blocked else "k_spmv_df_v4") + " on sector (1,1), complex",
                     "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)", "bytes_per_launch": bytes_spmv,
                     "avg_launch_ms": spmv_ms / max(spmv_n, 1), "traffic": None},
        "e2e": {"value": n / wall, "unit": "points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": n * 8 * 8},
        "clocks": clocks,
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_sample_spectrum(nphi, nel, nup, lam, nphi * nphi, len(ds))
    print(json.dumps(line), flush=True)
    return 0


def run_learned_workload(args):
    """Learned start vector: Nphi=14, 7+7, (J,K)=(0,0); train on d/l in {0, 0.25, ..., 3.0} with the
    library's BF16 kernels, then at the 12 held-out midpoints compare the plain FP64 path from the
    reference's random start with the mixed-precision path from the learned start."""
    import blqh_gb300 as B
    from blqh_gb300 import learned as Lr

    train_steps = args.train_steps
    B.ground_state(10, 10, 5, 0, 0, 1.0)  # warm-up: module loads
    r = Lr.run(nphi=14, nel=14, nup=7, steps=train_steps, lr=2e-3, timing=True)
    pts = r["points"]
    t64 = sum(p["fp64_random_s"] for p in pts)
    t32 = sum(p["mixed_learned_s"] for p in pts)
    rows = r["dim"] * 13
    flops = Lr.train_flops(rows, 32, 256) * train_steps
    peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"] if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else 1900.0
    line = {
        "metric": "learned start: wall time to E_gs at held-out d, mixed + learned vs plain FP64 (random start)",
        "workload": "learned14", "unit": "s", "higher_is_better": False,
        "value": t32, "fp64_random_total_s": t64, "fp64_over_mixed_learned": t64 / t32,
        "config": {"workload": "Nphi=14 Ne=14 (7+7) (J,K)=(0,0), train d/l 0..3 step 0.25, test 0.125..2.875",
                   "dim": r["dim"], "train_steps": train_steps, "mlp": "in 2*14+2 (pad 32) -> 3x256 tanh -> 1"},
        "iterations_random_mean": sum(p["iterations_random"] for p in pts) / len(pts),
        "iterations_learned_mean": sum(p["iterations_learned"] for p in pts) / len(pts),
        "fallbacks": sum(1 for p in pts if not p["used_learned"]),
        "overlap_exact_mean": sum(p["overlap_exact"] for p in pts) / len(pts),
        "max_abs_dE": max(p["abs_dE"] for p in pts),
        "train_loss": [r["loss_first"], r["loss_last"]], "train_s": r["train_s"],
        "train_tensor_tflops": flops / r["train_s"] / 1e12, "bf16_peak_tflops": peak,
        "train_tensor_frac": flops / r["train_s"] / 1e12 / peak,
        "points": pts,
    }
    print(json.dumps(line), flush=True)
    return 0


def ctypes_sizeof_instance():
    import ctypes

    from blqh_gb300._lib import Instance

    return ctypes.sizeof(Instance)


MONO30 = dict(nphi=30, nel=10, J=0, K=0, gamma=1.0, lam=400)


def cpu_sample_mono(nphi, nel, J, K, gamma, lam, rows=1500, spmv_reps=10, threads=None):
    """The monolayer oracle on the sector: the full basis, `rows` Hamiltonian rows
    from the middle of the sector and `spmv_reps` products over them,
    extrapolated to all rows and to the reference's 2 lambda + 1 products
    (lambda = 400, Monolayer/main.cpp:25: pass 1, reconstruction, Rayleigh quotient)."""
    import numpy as np

    from oracle import oracle as O

    threads = threads or os.cpu_count() or 1
    lx, ly = O.mono_torus(nphi, gamma)
    t0 = time.perf_counter()
    Bo = O.MonoBasis(nphi, nel, J, K)
    t1 = time.perf_counter()
    rows = min(rows, Bo.dim)
    r0 = Bo.dim // 2
    H = O.MonoHamil(Bo, lx, ly, nthreads=threads, rows=(r0, r0 + rows))
    t2 = time.perf_counter()
    x = np.ones(Bo.dim, np.complex128)
    for _ in range(spmv_reps):
        H.spmv(x)
    t3 = time.perf_counter()
    t_build = (t2 - t1) * Bo.dim / rows
    t_spmv = (t3 - t2) / spmv_reps * Bo.dim / rows
    total = (t1 - t0) + t_build + (2 * lam + 1) * t_spmv
    return {"value": 1.0 / total, "unit": "K-sectors/s", "cores": threads, "kind": "port",
            "time_to_egs_s_extrapolated": total,
            "sample": (f"oracle/mono_oracle.cpp (reference algorithm, OpenMP {threads} threads): full basis "
                       f"(dim {Bo.dim}) {t1 - t0:.2f} s, rows {r0}..{r0 + rows} {t2 - t1:.2f} s, {spmv_reps} "
                       f"complex SpMVs over them; extrapolated to all rows and 2*{lam}+1 SpMVs"),
            "sample_wall_s": t3 - t0}


def run_mono_workload(args):
    """The monolayer (Monolayer/ of the reference): Nphi=30, Ne=10 (filling 1/3),
    (J,K)=(0,0), square torus. One step = basis -> FP64 CSR -> Lanczos (full FP64
    reorthogonalization, tol 1e-12, at most 400 steps) -> Ritz vector -> Rayleigh
    quotient, timed with CUDA events on the context stream."""
    import blqh_gb300 as B

    cfg = dict(MONO30)
    nphi, nel, J, K, gamma, lam = cfg["nphi"], cfg["nel"], cfg["J"], cfg["K"], cfg["gamma"], cfg["lam"]
    ctx = B.Context(0)

    def step(rng=2, want_psi=False):
        b = B.basis_mono(nphi, nel, J, K, ctx=ctx)
        H = B.hamiltonian_mono(b, gamma)
        L = B.Lanczos(H, max_steps=min(lam, b.dim), tol=1e-12, rng=rng)
        n = L.iterate()
        e, _ = L.eig()
        psi = L.ritz_vector(copy=want_psi)
        E = L.rayleigh()
        out = dict(E=E, ritz0=float(e[0]), steps=n, dim=b.dim, nnz=H.nnz, psi=psi)
        L.close()
        H.close()
        b.close()
        return out

    for _ in range(max(args.warmup, 3)):
        r = step()
    times = []
    with ClockSampler(0) as cs:
        for _ in range(max(args.steps, 1)):
            ctx.synchronize()
            ctx.mark(0)
            r = step()
            ctx.mark(1)
            ctx.synchronize()
            times.append(ctx.elapsed_ms(0, 1) / 1e3)
    clocks = cs.summary()
    t = sorted(times)[len(times) // 2]
    # end to end through the public API: host start vector in, ground state out
    e2e = []
    for _ in range(max(args.steps, 1)):
        t0 = time.perf_counter()
        g = B.ground_state_mono(nphi, nel, J, K, gamma=gamma, max_steps=lam, tol=1e-12, want_psi=True, rng=0,
                                ctx=ctx)
        e2e.append(time.perf_counter() - t0)
    te = sorted(e2e)[len(e2e) // 2]
    # kernel classes of one step
    ctx.timers(True)
    ctx.reset_timers()
    step()
    ctx.synchronize()
    tm = ctx.timers(False)
    spmv_ms, spmv_n = tm["spmv"]
    dim, nnz = r["dim"], r["nnz"]
    bytes_spmv = nnz * (8 + 4) + (dim + 1) * 8 + 2 * dim * 8
    achieved = bytes_spmv / (spmv_ms / 1e3 / max(spmv_n, 1)) / 1e9
    peak, peak_kind = peaks()
    line = {
        "metric": "monolayer K-sector time-to-E_gs (FP64 Lanczos, |dE| vs oracle reference values)",
        "workload": "mono30", "value": 1.0 / t, "unit": "K-sectors/s", "n_gpus": 1, "steps": len(times),
        "warmup": max(args.warmup, 3), "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (physics parameters only; no dataset exists)",
        "config": {"workload": (f"monolayer Nphi={nphi} Ne={nel} (filling 1/3) (J,K)=({J},{K}) square torus: basis "
                                f"-> FP64 CSR -> Lanczos (full FP64 reorth, tol 1e-12, <= {lam} steps) -> Rayleigh "
                                f"quotient"), "nphi": nphi, "nel": nel, "dim": dim,
                   "l2": "inputs larger than L2 (CSR rebuilt every step)"},
        "E_gs": r["E"], "E_gs_per_Ne": r["E"] / nel, "ritz0": r["ritz0"], "lanczos_steps": r["steps"], "nnz": nnz,
        "kernel_ms": {k: v[0] for k, v in tm.items()},
        "roofline": {"kernel": "k_spmv (FP64 CSR row kernel) in the Lanczos steps", "bound": "hbm",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)", "bytes_per_launch": bytes_spmv,
                     "avg_launch_ms": spmv_ms / max(spmv_n, 1), "launches": spmv_n, "traffic": None},
        "e2e": {"value": 1.0 / te, "unit": "K-sectors/s", "h2d_bytes_per_step": dim * 8,
                "d2h_bytes_per_step": dim * 8, "s_per_step": te},
        "E_gs_e2e": g["energy"],
        "clocks": clocks,
    }
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_sample_mono(nphi, nel, J, K, gamma, lam)
    print(json.dumps(line), flush=True)
    return 0


def _solve_arm(sectors, precision, streams, results, max_steps, starts=None):
    """Every listed (J, K) sector of the configuration through the public one-call API,
    spread over `streams` contexts driven from host threads; results[(J, K)] = result."""
    import threading

    import blqh_gb300 as B

    errors = []

    def work(part):
        try:
            ctx = B.Context(0)
            for J, K in part:
                st = starts.get((J, K)) if starts else None
                results[(J, K)] = B.ground_state(NPHI, NEL, NUP, J, K, D, DSAS, DV, precision=precision,
                                                 max_steps=max_steps, tol=TOL, check_every=CHECK, seed=1,
                                                 rng=2, start=st, ctx=ctx)
            ctx.close()
        except Exception as e:  # re-raised in the caller
            errors.append(e)

    parts = [sectors[i::streams] for i in range(streams)]
    ts = [threading.Thread(target=work, args=(p,)) for p in parts if p]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    if errors:
        raise errors[0]


def run_all16_workload(args):
    """Every (J, K) sector of the configuration (Nphi=16, 8+8, d/l=1, Delta_SAS=0.05):
    256 sectors of dimension ~6.5e5 (32 real, 224 complex), each basis -> CSR ->
    Lanczos (full reorthogonalization, tol 1e-12) -> Rayleigh quotient, as the
    reference's excitation-spectrum loop runs them (BLQH_without_spin/main.cpp:84-115).
    Arm 1: FP64 values from random starts; arm 2: FP32 values with the FP64
    regenerated Rayleigh quotient from random starts. Wall time of each arm
    (host clock around the whole arm; every call returns its energy to the host)."""
    import numpy as np

    sectors = [(J, K) for J in range(NPHI) for K in range(NPHI)]
    if args.sectors:
        sectors = sectors[: args.sectors]
    import blqh_gb300 as B

    warm = {}
    _solve_arm([(0, 0), (0, 1)] * max(1, args.streams), B.VAL_FP32, args.streams, warm, args.max_steps)
    _solve_arm([(0, 0), (0, 1)] * max(1, args.streams), B.VAL_FP64, args.streams, warm, args.max_steps)
    arms = {}
    with ClockSampler(0) as cs:
        for name, prec in (("fp64", B.VAL_FP64), ("mixed", B.VAL_FP32)):
            res = {}
            t0 = time.perf_counter()
            _solve_arm(sectors, prec, args.streams, res, args.max_steps)
            arms[name] = (time.perf_counter() - t0, res)
    clocks = cs.summary()
    t64, r64 = arms["fp64"]
    t32, r32 = arms["mixed"]
    dE = {s: abs(r32[s]["energy"] - r64[s]["energy"]) for s in sectors}
    worst = max(dE, key=dE.get)
    cplx = [s for s in sectors if not (s[1] == 0 or 2 * s[1] == NPHI)]
    e_min = min(sectors, key=lambda s: r64[s]["energy"])
    line = {
        "metric": "every K-sector ground energy of Nphi=16 Ne=16 (8+8): mixed vs FP64 wall time at |dE|<1e-9",
        "workload": "all16", "value": len(sectors) / t32, "unit": "K-sectors/s", "n_gpus": 1, "steps": 1,
        "warmup": 1, "higher_is_better": True, "dtype": "f32 values / f64 vectors (arm 2), f64 (arm 1)",
        "data": "synthetic (physics parameters only)",
        "config": {"workload": (f"spinless bilayer Nphi={NPHI} Ne={NEL} ({NUP}+{NEL - NUP}) every (J,K), d={D}, "
                                f"Delta_SAS={DSAS}: basis -> CSR -> Lanczos (full reorth, tol {TOL}) -> RQ"),
                   "sectors": len(sectors), "complex_sectors": len(cplx), "streams": args.streams,
                   "starts": "random (counter-based, seed 1) in both arms"},
        "fp64_wall_s": t64, "mixed_wall_s": t32, "mixed_over_fp64_time": t32 / t64, "target_ratio": 1 / 1.5,
        "max_abs_dE_mixed_vs_fp64": dE[worst], "worst_sector": list(worst),
        "lanczos_steps_mean": {"fp64": float(np.mean([r64[s]["steps"] for s in sectors])),
                               "mixed": float(np.mean([r32[s]["steps"] for s in sectors]))},
        "lowest_E_gs": {"sector": list(e_min), "E_gs": r64[e_min]["energy"],
                        "E_gs_per_Ne": r64[e_min]["energy"] / NEL},
        "clocks": clocks,
    }
    if args.out:
        with open(args.out, "w") as f:
            json.dump({f"{J},{K}": {"dim": r64[(J, K)]["dim"], "nnz": r64[(J, K)]["nnz"],
                                    "E_fp64": r64[(J, K)]["energy"], "E_mixed": r32[(J, K)]["energy"],
                                    "steps_fp64": r64[(J, K)]["steps"], "steps_mixed": r32[(J, K)]["steps"]}
                       for J, K in sectors}, f, indent=0)
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="sector16",
                    choices=["sector16", "sweep12", "learned14", "spectrum14", "mono30", "all16"],
                    help="sector16: one Nphi=16 K-sector (default); sweep12: the batched Nphi=12 sweep; "
                         "learned14: the learned start vector at Nphi=14; spectrum14: every (J, K) of Nphi=14; "
                         "mono30: one monolayer K-sector at Nphi=30, Ne=10; all16: every (J, K) of the "
                         "Nphi=16 configuration, mixed vs FP64")
    ap.add_argument("--sectors", type=int, default=0, help="all16: only the first n sectors (0: all 256)")
    ap.add_argument("--out", default="", help="all16: per-sector results as JSON")
    ap.add_argument("--train-steps", type=int, default=2000, help="learned14: Adam steps")
    ap.add_argument("--streams", type=int, default=4, help="spectrum14: contexts (CUDA streams) driven in parallel")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--profile", action="store_true",
                    help="only the timed mixed-precision steps (no FP64 comparison, e2e or CPU sample)")
    ap.add_argument("--nphi", type=int, default=NPHI)
    ap.add_argument("--nel", type=int, default=NEL)
    ap.add_argument("--nup", type=int, default=NUP)
    ap.add_argument("--k", type=int, default=K_SEC, help="sector momentum K (0: real sector)")
    ap.add_argument("--max-steps", type=int, default=MAX_STEPS)
    args = ap.parse_args()
    if (args.nphi, args.nel, args.nup) != (NPHI, NEL, NUP) and not args.profile:
        ap.error("--nphi/--nel/--nup change the workload; they are only for --profile runs")
    if args.workload == "sweep12":
        return run_sweep_workload(args)
    if args.workload == "learned14":
        return run_learned_workload(args)
    if args.workload == "spectrum14":
        return run_spectrum_workload(args)
    if args.workload == "mono30":
        return run_mono_workload(args)
    if args.workload == "all16":
        if args.streams == 4 and "--streams" not in sys.argv:
            args.streams = 2
        return run_all16_workload(args)
    world, rank, local, pg = dist_setup()
    try:
        if args.impl == "reference":
            return run_reference(args, world, rank, pg)
        return run_ours(args, world, rank, local, pg)
    finally:
        if pg is not None:
            pg.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
