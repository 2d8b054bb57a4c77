"""GB300 exact diagonalization of quantum-Hall systems on the torus (qiongz/BLQH): the spinless
and spinful bilayers and the monolayer.

Host-side mirror of the reference's interface over the C ABI of libblqh_gpu.so
(include/blqh_gpu.h). Every computation runs on the GPU; this module only
moves parameters and host copies. There is no CPU fallback: without the
library, or without a CUDA device, calls raise.

Two layers:
  * ``Context``, ``Basis``, ``Hamiltonian``, ``Lanczos`` and ``ground_state``:
    thin owners of the library's handles;
  * ``basis`` and ``lhamil``: the reference's classes (BLQH_without_spin/basis.h:25,
    lanczos_hamiltonian.h:11) with the same method names and public members.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import (MODEL_MONOLAYER, MODEL_SPINFUL, MODEL_SPINLESS, REP_MIN, REP_REFERENCE, VAL_FP32,
                   VAL_FP64, BatchOpts, BatchResult, BlqhError, Instance, LanczosOpts, Params, ParamsMono,
                   ParamsSpin, Result, Sector, SectorMono, SectorSpin, check, lib)

__all__ = ["Context", "Basis", "Hamiltonian", "Lanczos", "Batch", "MLP", "instance", "instance_spin", "basis_spin",
           "hamiltonian_spin", "ground_state", "batch_run", "basis_mono", "hamiltonian_mono", "ground_state_mono",
           "mono_torus", "mono_classical_energy", "instance_mono",
           "start_vector", "torus", "basis",
           "lhamil", "BlqhError", "REP_REFERENCE", "REP_MIN", "VAL_FP64", "VAL_FP32"]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def torus(nphi, gamma=1.0):
    """lx, ly of the torus with aspect ratio gamma (BLQH_without_spin/main.cpp:20-21)."""
    ly = math.sqrt(nphi * 2.0 * math.pi / gamma)
    return ly * gamma, ly


class Context:
    """One device and one CUDA stream. Not thread-safe."""

    _default = None

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        check(lib().blqh_ctx_create(device, ctypes.byref(h)))
        self.h = h

    @classmethod
    def default(cls):
        if cls._default is None:
            cls._default = Context(0)
        return cls._default

    def check(self, rc):
        return check(rc, self.h)

    def synchronize(self):
        self.check(lib().blqh_ctx_synchronize(self.h))

    def timers(self, enable=None):
        ms = (ctypes.c_double * 5)()
        n = (ctypes.c_int64 * 5)()
        self.check(lib().blqh_ctx_timers(self.h, -1 if enable is None else int(enable), ms, n))
        keys = ("spmv", "reorth", "build", "basis", "misc")
        return {k: (ms[i], n[i]) for i, k in enumerate(keys)}

    def reset_timers(self):
        self.check(lib().blqh_ctx_reset_timers(self.h))

    def mark(self, slot):
        """Record event marker `slot` (0..7) on the context's stream."""
        self.check(lib().blqh_ctx_mark(self.h, slot))

    def elapsed_ms(self, a, b):
        """Device time between two recorded markers."""
        ms = ctypes.c_double()
        self.check(lib().blqh_ctx_elapsed_ms(self.h, a, b, ctypes.byref(ms)))
        return ms.value

    def close(self):
        if getattr(self, "h", None):
            lib().blqh_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _params(nphi, d, delta_sas=0.0, delta_v=0.0, nLL=0, gamma=1.0, theta_x=0.0, theta_y=0.0, lx=None, ly=None):
    if lx is None:
        lx, ly = torus(nphi, gamma)
    return Params(lx, ly, d, delta_sas, delta_v, theta_x, theta_y, nLL)


class Basis:
    """Sector basis on the device (K1)."""

    def __init__(self, nphi, nel, nel_up, J, K, rep_mode=REP_REFERENCE, ctx=None, _spin=None, _mono=None):
        self.ctx = ctx or Context.default()
        h = ctypes.c_void_p()
        self.monolayer = _mono is not None
        if _mono is not None:
            self.sector = _mono
            self.spinful = False
            self.ctx.check(lib().blqh_basis_build_mono(self.ctx.h, ctypes.byref(self.sector), ctypes.byref(h)))
        elif _spin is None:
            self.sector = Sector(nphi, nel, nel_up, J, K, rep_mode)
            self.spinful = False
            self.ctx.check(lib().blqh_basis_build(self.ctx.h, ctypes.byref(self.sector), ctypes.byref(h)))
        else:
            self.sector = _spin
            self.spinful = True
            self.ctx.check(lib().blqh_basis_build_spin(self.ctx.h, ctypes.byref(self.sector), ctypes.byref(h)))
        self.h = h
        n = ctypes.c_int64()
        self.ctx.check(lib().blqh_basis_size(self.h, ctypes.byref(n)))
        self.dim = n.value
        self._id = self._period = None

    def _fetch(self):
        self._id = np.zeros(self.dim, np.uint64)
        self._period = np.zeros(self.dim, np.int16)
        if self.dim:
            self.ctx.check(lib().blqh_basis_get(self.ctx.h, self.h, _ptr(self._id), _ptr(self._period)))

    @property
    def id(self):
        if self._id is None:
            self._fetch()
        return self._id

    @property
    def period(self):
        if self._period is None:
            self._fetch()
        return self._period

    def close(self):
        if getattr(self, "h", None):
            lib().blqh_basis_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def basis_spin(nphi, nel, nel_up, nel_su, J, K, rep_mode=REP_REFERENCE, ctx=None):
    """Spinful sector basis (BLQH_with_spin basis::init(nphi, nel, nel_up, nel_su, J, K))."""
    return Basis(nphi, nel, nel_up, J, K, rep_mode, ctx, _spin=SectorSpin(nphi, nel, nel_up, nel_su, J, K, rep_mode))


def mono_torus(nphi, gamma=1.0):
    """lx, ly of the monolayer torus with aspect ratio gamma = lx / ly (Monolayer/main.cpp:33-34)."""
    ly = math.sqrt(2.0 * math.pi * nphi / gamma)
    return ly * gamma, ly


def mono_classical_energy(nphi, lx, ly):
    """E_cl of the monolayer diagonal (Monolayer/lanczos_hamiltonian.cpp:68-74), closed form."""
    e = ctypes.c_double()
    check(lib().blqh_mono_classical_energy(nphi, lx, ly, ctypes.byref(e)))
    return e.value


def basis_mono(nphi, nel, J=-1, K=-1, rep_mode=REP_REFERENCE, ctx=None):
    """Monolayer sector basis (Monolayer basis::init(nphi, nel, J, K)); K in [0, gcd(nel, nphi))."""
    return Basis(nphi, nel, nel, J, K, rep_mode, ctx, _mono=SectorMono(nphi, nel, J, K, rep_mode))


def hamiltonian_mono(basis, gamma=1.0, nLL=0, lx=None, ly=None):
    """Monolayer Hamiltonian (Monolayer lhamil::set_hamil(sector, lx, ly, nphi, nLL)), FP64 values."""
    if not getattr(basis, "monolayer", False):
        raise BlqhError(-1, "hamiltonian_mono needs a basis from basis_mono()")
    if lx is None:
        lx, ly = mono_torus(basis.sector.nphi, gamma)
    return Hamiltonian._mono(basis, ParamsMono(lx, ly, nLL))


def ground_state_mono(nphi, nel, J=-1, K=-1, gamma=1.0, nLL=0, max_steps=400, tol=1e-12, check_every=10, seed=1,
                      lx=None, ly=None, n_levels=1, want_psi=False, rng=0, ctx=None):
    """Monolayer sector ground state: basis -> CSR -> Lanczos (full FP64 reorthogonalization) -> Ritz
    vector -> Rayleigh quotient. Returns the lowest n_levels Ritz values (the reference's
    eigenvalues[0..], lanczos_hamiltonian.cpp:338-360), the Rayleigh quotient of the Ritz vector and,
    with want_psi, the ground state (host copy). rng 0 draws the start vector on the host
    (std::mt19937, as the reference), 2 on the device."""
    B = basis_mono(nphi, nel, J, K, ctx=ctx)
    H = hamiltonian_mono(B, gamma, nLL, lx, ly)
    L = Lanczos(H, max_steps=min(max_steps, B.dim), tol=tol, check_every=check_every, seed=seed, rng=rng)
    steps = L.iterate()
    e, _ = L.eig()
    psi = L.ritz_vector(copy=want_psi)
    energy = L.rayleigh()
    out = dict(energy=energy, eigenvalues=np.array(e[:n_levels]), steps=steps, dim=B.dim, nnz=H.nnz,
               is_complex=H.is_complex)
    if want_psi:
        out["psi"] = psi
    L.close()
    H.close()
    B.close()
    return out


def _params_spin(nphi, d, delta_sas=0.0, delta_v=0.0, delta_z=0.0, theta_b=0.0, nLL=0, gamma=1.0, theta_x=0.0,
                 theta_y=0.0):
    lx, ly = torus(nphi, gamma)
    return ParamsSpin(lx, ly, d, delta_sas, delta_v, delta_z, theta_b, theta_x, theta_y, nLL)


def hamiltonian_spin(basis, d, delta_sas=0.0, delta_v=0.0, delta_z=0.0, theta_b=0.0, nLL=0, gamma=1.0, theta_x=0.0,
                     theta_y=0.0, precision=VAL_FP64):
    """Spinful Hamiltonian (BLQH_with_spin lhamil::set_hamil); precision = VAL_FP32 stores FP32 values
    (finish with Lanczos.rayleigh_fp64, which regenerates the FP64 elements)."""
    return Hamiltonian._spin(basis, _params_spin(basis.sector.nphi, d, delta_sas, delta_v, delta_z, theta_b, nLL,
                                                 gamma, theta_x, theta_y), precision)


class Hamiltonian:
    """CSR Hamiltonian of a sector on the device (K2)."""

    def __init__(self, basis: Basis, d, delta_sas=0.0, delta_v=0.0, nLL=0, gamma=1.0, theta_x=0.0, theta_y=0.0,
                 precision=VAL_FP64, lx=None, ly=None):
        self.basis = basis
        self.ctx = basis.ctx
        h = ctypes.c_void_p()
        if getattr(basis, "spinful", False):
            raise BlqhError(-1, "spinful basis: use hamiltonian_spin()")
        if getattr(basis, "monolayer", False):
            raise BlqhError(-1, "monolayer basis: use hamiltonian_mono()")
        self.params = _params(basis.sector.nphi, d, delta_sas, delta_v, nLL, gamma, theta_x, theta_y, lx, ly)
        self.ctx.check(lib().blqh_hamil_build(self.ctx.h, basis.h, ctypes.byref(self.params), precision,
                                              ctypes.byref(h)))
        self._finish(h)

    @classmethod
    def _spin(cls, basis, params, precision=VAL_FP64):
        self = cls.__new__(cls)
        self.basis, self.ctx, self.params = basis, basis.ctx, params
        h = ctypes.c_void_p()
        self.ctx.check(lib().blqh_hamil_build_spin_prec(self.ctx.h, basis.h, ctypes.byref(params), precision,
                                                        ctypes.byref(h)))
        self._finish(h)
        return self

    @classmethod
    def _mono(cls, basis, params):
        self = cls.__new__(cls)
        self.basis, self.ctx, self.params = basis, basis.ctx, params
        h = ctypes.c_void_p()
        self.ctx.check(lib().blqh_hamil_build_mono(self.ctx.h, basis.h, ctypes.byref(params), ctypes.byref(h)))
        self._finish(h)
        return self

    def _finish(self, h):
        self.h = h
        dim, nnz, cplx, prec = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int(), ctypes.c_int()
        self.ctx.check(lib().blqh_csr_info(self.h, ctypes.byref(dim), ctypes.byref(nnz), ctypes.byref(cplx),
                                           ctypes.byref(prec)))
        self.dim, self.nnz, self.is_complex, self.precision = dim.value, nnz.value, bool(cplx.value), prec.value

    def csr(self):
        """Host copy: (row_ptr int64, col int32, val float64 or complex128)."""
        rp = np.zeros(self.dim + 1, np.int64)
        col = np.zeros(self.nnz, np.int32)
        val = np.zeros(self.nnz * (2 if self.is_complex else 1), np.float64)
        self.ctx.check(lib().blqh_csr_get(self.ctx.h, self.h, _ptr(rp), _ptr(col), _ptr(val)))
        if self.is_complex:
            val = val.view(np.complex128)
        return rp, col, val

    def spmv(self, x):
        dt = np.complex128 if self.is_complex else np.float64
        x = np.ascontiguousarray(x, dt)
        y = np.zeros(self.dim, dt)
        self.ctx.check(lib().blqh_spmv(self.ctx.h, self.h, _ptr(x), _ptr(y)))
        return y

    def spmv_layout(self):
        """1 when the blocked copy used by the mixed-precision SpMV exists, else 0."""
        return lib().blqh_debug_spmv_layout(self.h)

    def close(self):
        if getattr(self, "h", None):
            lib().blqh_csr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Lanczos:
    """Lanczos on the device (K3-K8) for one Hamiltonian."""

    def __init__(self, H: Hamiltonian, max_steps=200, reorth=True, tol=1e-12, check_every=10, seed=1, rng=0,
                 start=None, accumulate=0):
        self.H = H
        self.ctx = H.ctx
        self.opts = LanczosOpts(max_steps, int(reorth), tol, check_every, seed, rng, accumulate)
        h = ctypes.c_void_p()
        self.ctx.check(lib().blqh_lanczos_create(self.ctx.h, H.h, ctypes.byref(self.opts), ctypes.byref(h)))
        self.h = h
        self.steps = 0
        if start is not None:
            dt = np.complex128 if H.is_complex else np.float64
            s = np.ascontiguousarray(start, dt)
            self.ctx.check(lib().blqh_lanczos_set_start(self.h, _ptr(s)))

    def iterate(self):
        n = ctypes.c_int()
        self.ctx.check(lib().blqh_lanczos_iterate(self.h, ctypes.byref(n)))
        self.steps = n.value
        return self.steps

    def coeffs(self):
        a = np.zeros(self.steps)
        b = np.zeros(self.steps + 1)
        self.ctx.check(lib().blqh_lanczos_coeffs(self.h, _ptr(a), _ptr(b)))
        return a, b

    def eig(self):
        e = np.zeros(self.steps)
        y = np.zeros(self.steps)
        self.ctx.check(lib().blqh_lanczos_eig(self.h, _ptr(e), _ptr(y)))
        return e, y

    def ritz_vector(self, copy=True):
        dt = np.complex128 if self.H.is_complex else np.float64
        psi = np.zeros(self.H.dim, dt) if copy else None
        self.ctx.check(lib().blqh_lanczos_ritz_vector(self.h, _ptr(psi)))
        return psi

    def rayleigh(self):
        e = ctypes.c_double()
        self.ctx.check(lib().blqh_lanczos_rayleigh(self.h, ctypes.byref(e)))
        return e.value

    def observables(self, basis=None):
        """pseudospin Sz, Sx and occupation numbers [2][nphi] of the ground state (after ritz_vector)."""
        basis = basis or self.H.basis
        sz, sx = ctypes.c_double(), ctypes.c_double()
        occ = np.zeros(2 * basis.sector.nphi)
        self.ctx.check(lib().blqh_lanczos_observables(self.h, basis.h, ctypes.byref(sz), ctypes.byref(sx),
                                                      _ptr(occ)))
        return dict(Sz=sz.value, Sx=sx.value, occupation=occ.reshape(2, -1))

    def rayleigh_fp64(self):
        e = ctypes.c_double()
        fn = lib().blqh_lanczos_rayleigh_fp64_spin if getattr(self.H.basis, "spinful", False) else \
            lib().blqh_lanczos_rayleigh_fp64
        self.ctx.check(fn(self.h, self.H.basis.h, ctypes.byref(self.H.params), ctypes.byref(e)))
        return e.value

    def observables_spin(self, basis=None):
        """Spinful ground-state observables (after ritz_vector), as BLQH_with_spin/
        lanczos_hamiltonian.cpp:1217-1593 defines them, computed on the device."""
        basis = basis or self.H.basis
        nphi = basis.sector.nphi
        out = np.zeros(6 + 2 * nphi)
        self.ctx.check(lib().blqh_lanczos_observables_spin(self.h, basis.h, _ptr(out)))
        keys = ("Sz", "pseudospin_Sz", "upper_Sz", "down_Sz", "pseudospin_Sx", "spinflip_tunneling")
        r = {k: float(out[i]) for i, k in enumerate(keys)}
        r["occupation"] = out[6:].reshape(2, nphi)
        return r

    def rayleigh_conj(self, regenerate=None):
        """The reference's printed energy <conj(psi)|H|conj(psi)> (its conjugated
        reconstruction, lanczos_hamiltonian.cpp:610-656); the ground energy in real
        sectors only. regenerate (default: FP32-valued matrices) uses FP64 matrix
        elements regenerated on the fly instead of the stored values."""
        if regenerate is None:
            regenerate = self.H.precision != VAL_FP64
        e = ctypes.c_double()
        b, p = (self.H.basis.h, ctypes.byref(self.H.params)) if regenerate else (None, None)
        self.ctx.check(lib().blqh_lanczos_rayleigh_conj(self.h, b, p, ctypes.byref(e)))
        return e.value

    def close(self):
        if getattr(self, "h", None):
            lib().blqh_lanczos_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ground_state(nphi, nel, nel_up, J, K, d, delta_sas=0.0, delta_v=0.0, nLL=0, gamma=1.0, precision=VAL_FP64,
                 max_steps=200, reorth=True, tol=1e-12, check_every=10, seed=1, rng=0, start=None, want_psi=False,
                 rep_mode=REP_REFERENCE, ctx=None, psi_out=None, accumulate=0):
    """Whole path in one library call: basis -> CSR -> Lanczos -> Rayleigh quotient.

    start: optional host start vector; psi_out: optional preallocated host array
    (length dim) that receives the ground state (want_psi allocates one)."""
    ctx = ctx or Context.default()
    s = Sector(nphi, nel, nel_up, J, K, rep_mode)
    p = _params(nphi, d, delta_sas, delta_v, nLL, gamma)
    o = LanczosOpts(max_steps, int(reorth), tol, check_every, seed, rng, accumulate)
    r = Result()
    st = None if start is None else np.ascontiguousarray(start)
    psi = psi_out
    if psi is None and want_psi:
        cplx = not (K <= 0 or 2 * K == nphi)
        b = Basis(nphi, nel, nel_up, J, K, rep_mode, ctx)
        psi = np.zeros(b.dim, np.complex128 if cplx else np.float64)
        b.close()
    want_psi = psi is not None
    ctx.check(lib().blqh_ground_state(ctx.h, ctypes.byref(s), ctypes.byref(p), precision, ctypes.byref(o), _ptr(st),
                                      _ptr(psi), ctypes.byref(r)))
    out = dict(energy=r.energy, ritz0=r.ritz0, steps=r.steps, dim=r.dim, nnz=r.nnz)
    if want_psi:
        out["psi"] = psi
    return out


def instance(nphi, nel, nel_up, J, K, d, delta_sas=0.0, delta_v=0.0, nLL=0, gamma=1.0, theta_x=0.0, theta_y=0.0,
             rep_mode=REP_REFERENCE):
    """One spinless (sector, parameter point) of a batched sweep."""
    return Instance(MODEL_SPINLESS, Sector(nphi, nel, nel_up, J, K, rep_mode),
                    _params(nphi, d, delta_sas, delta_v, nLL, gamma, theta_x, theta_y))


def instance_spin(nphi, nel, nel_up, nel_su, J, K, d, delta_sas=0.0, delta_v=0.0, delta_z=0.0, theta_b=0.0, nLL=0,
                  gamma=1.0, theta_x=0.0, theta_y=0.0, rep_mode=REP_REFERENCE):
    """One spinful (sector, parameter point) of a batched sweep."""
    i = Instance()
    i.model = MODEL_SPINFUL
    i.ssector = SectorSpin(nphi, nel, nel_up, nel_su, J, K, rep_mode)
    i.sparams = _params_spin(nphi, d, delta_sas, delta_v, delta_z, theta_b, nLL, gamma, theta_x, theta_y)
    return i


def instance_mono(nphi, nel, J, K, gamma=1.0, nLL=0, rep_mode=REP_REFERENCE, lx=None, ly=None):
    """One monolayer sector of a batched sweep (FP64 values, finished with them)."""
    if lx is None:
        lx, ly = mono_torus(nphi, gamma)
    i = Instance()
    i.model = MODEL_MONOLAYER
    i.msector = SectorMono(nphi, nel, J, K, rep_mode)
    i.mparams = ParamsMono(lx, ly, nLL)
    return i


class Batch:
    """K9: many instances in one persistent launch (blqh_batch_*).

    instances: list of Instance (see instance()); lam: Lanczos steps each."""

    def __init__(self, instances, lam=150, precision=VAL_FP32, seed=1, threads=0, lanes_per_row=0, graph=False,
                 ctx=None):
        self.ctx = ctx or Context.default()
        self.n = len(instances)
        self._inst = (Instance * max(1, self.n))(*instances)
        self.opts = BatchOpts(lam, precision, seed, threads, lanes_per_row, int(graph))
        h = ctypes.c_void_p()
        self.ctx.check(lib().blqh_batch_create(self.ctx.h, self._inst, self.n, ctypes.byref(self.opts),
                                               ctypes.byref(h)))
        self.h = h

    def solve(self):
        self.ctx.check(lib().blqh_batch_solve(self.h))

    def results(self):
        """List of dicts: energy, ritz0, resid, dim, nnz, steps, second_passes."""
        out = (BatchResult * max(1, self.n))()
        self.ctx.check(lib().blqh_batch_results(self.h, out))
        return [dict(energy=r.energy, ritz0=r.ritz0, resid=r.resid, dim=r.dim, nnz=r.nnz, steps=r.steps,
                     second_passes=r.second_passes) for r in out[:self.n]]

    def ground_state(self, i):
        r = self.results()[i]
        ins = self._inst[i]
        if ins.model == MODEL_SPINFUL:
            s, p = ins.ssector, ins.sparams
            cplx = not ((s.K <= 0 or 2 * s.K == s.nphi) and p.theta_y == 0.0 and p.theta_b == 0.0)
        else:
            s, p = ins.sector, ins.params
            cplx = not ((s.K <= 0 or 2 * s.K == s.nphi) and p.theta_y == 0.0)
        psi = np.zeros(r["dim"] * (2 if cplx else 1))
        self.ctx.check(lib().blqh_batch_ground_state(self.h, i, _ptr(psi)))
        return psi.view(np.complex128) if cplx else psi

    def shape(self):
        t, l, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.ctx.check(lib().blqh_batch_shape(self.h, ctypes.byref(t), ctypes.byref(l), ctypes.byref(b)))
        return dict(threads=t.value, lanes_per_row=l.value, blocks_per_sm=b.value)

    def timing(self):
        """Device time of the last solve: lanczos_ms (persistent launch), finish_ms, launches."""
        a, c, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        self.ctx.check(lib().blqh_batch_timing(self.h, ctypes.byref(a), ctypes.byref(c), ctypes.byref(n)))
        return dict(lanczos_ms=a.value, finish_ms=c.value, launches=n.value)

    def close(self):
        if getattr(self, "h", None):
            lib().blqh_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_run(instances, lam=150, precision=VAL_FP32, seed=1, threads=0, lanes_per_row=0, ctx=None):
    """create + solve + results in one call."""
    b = Batch(instances, lam, precision, seed, threads, lanes_per_row, False, ctx)
    try:
        b.solve()
        return b.results()
    finally:
        b.close()


class MLP:
    """K11: learned start vector (blqh_mlp_*). n_bits = 2 nphi of the bases it is used with."""

    def __init__(self, n_bits, width=256, seed=1, ctx=None):
        self.ctx = ctx or Context.default()
        h = ctypes.c_void_p()
        self.ctx.check(lib().blqh_mlp_create(self.ctx.h, n_bits, width, seed, ctypes.byref(h)))
        self.h = h
        n = ctypes.c_int64()
        self.ctx.check(lib().blqh_mlp_num_params(self.h, ctypes.byref(n)))
        self.num_params, self.n_bits, self.width = n.value, n_bits, width
        self.k0 = (n_bits + 2 + 31) // 32 * 32

    def params(self):
        w = np.zeros(self.num_params, np.float32)
        self.ctx.check(lib().blqh_mlp_get_params(self.h, _ptr(w)))
        return w

    def set_params(self, w):
        w = np.ascontiguousarray(w, np.float32)
        assert w.size == self.num_params
        self.ctx.check(lib().blqh_mlp_set_params(self.h, _ptr(w)))

    def predict(self, basis, d, delta_sas=0.0):
        psi = np.zeros(basis.dim)
        self.ctx.check(lib().blqh_mlp_predict(self.h, basis.h, d, delta_sas, _ptr(psi)))
        return psi

    @staticmethod
    def _pack(conds, targets):
        c = np.ascontiguousarray(np.asarray(conds, np.float64).reshape(-1, 2))
        t = np.ascontiguousarray(np.asarray(targets, np.float64).reshape(len(c), -1))
        return c, t

    def loss_grad(self, basis, conds, targets):
        c, t = self._pack(conds, targets)
        loss = ctypes.c_double()
        g = np.zeros(self.num_params, np.float32)
        self.ctx.check(lib().blqh_mlp_loss_grad(self.h, basis.h, len(c), _ptr(c), _ptr(t), ctypes.byref(loss),
                                                _ptr(g)))
        return loss.value, g

    def train(self, basis, conds, targets, steps=100, lr=1e-3):
        """Full-batch Adam steps; returns the loss before each step."""
        c, t = self._pack(conds, targets)
        losses = np.zeros(steps)
        self.ctx.check(lib().blqh_mlp_train(self.h, basis.h, len(c), _ptr(c), _ptr(t), steps, lr, _ptr(losses)))
        return losses

    def close(self):
        if getattr(self, "h", None):
            lib().blqh_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def start_vector(dim, seed=1, rng=0, is_complex=False):
    """Start vector drawn as the reference does (std::mt19937 or mt19937-64), normalized."""
    out = np.zeros(dim * (2 if is_complex else 1))
    check(lib().blqh_start_vector(seed, rng, dim, int(is_complex), _ptr(out)))
    return out.view(np.complex128) if is_complex else out


# ---------------------------------------------------------------------------
# The reference's classes.
class basis:
    """BLQH_without_spin/basis.h:25-56: the sector basis (members nphi, nel, nel_up,
    nel_down, J, K, nbasis, id, basis_C), built on the GPU by init()."""

    def __init__(self, nphi=0, nel=0, nel_up=-1, J=-1, K=-1):
        self.nphi, self.nel, self.nel_up, self.J, self.K = nphi, nel, nel_up, J, K
        self.nel_down = nel - nel_up if nel_up >= 0 else -1
        self.nbasis = 0
        self.id = np.zeros(0, np.uint64)
        self.basis_C = np.zeros(0, np.int16)
        self._b = None

    def init(self, nphi=None, nel=None, nel_up=None, J=None, K=None, ctx=None):
        if nphi is not None:
            self.nphi, self.nel = nphi, nel
            self.nel_up = -1 if nel_up is None else nel_up
            self.J = -1 if J is None else J
            self.K = -1 if K is None else K
            self.nel_down = self.nel - self.nel_up if self.nel_up >= 0 else -1
        self._b = Basis(self.nphi, self.nel, self.nel_up, self.J, self.K, REP_REFERENCE, ctx)
        self.nbasis = self._b.dim
        self.id = self._b.id
        self.basis_C = self._b.period


def save_lanczos_text(filename, nHilbert, n, seed, eigenvalues, norm, overlap, psi_0, psi_n0):
    """Writes the reference's Lanczos checkpoint text: nHilbert, lambda, seed, then
    "name:=  [ v , ... ,  ] " lists with 8 significant digits (as C++ iostreams
    print them with setprecision(8)); norm has n + 1 entries, the others n."""
    def lst(name, v, count):
        vals = [(float(v[i]) if i < len(v) else 0.0) for i in range(count)]
        return name + " [ ".rjust(10) + "".join("%.8g , " % x for x in vals) + " ] \n"

    with open(filename, "w") as f:
        f.write("nHilbert:=" + " ".rjust(10) + str(int(nHilbert)) + "\n")
        f.write("lambda:=" + " ".rjust(10) + str(int(n)) + "\n")
        f.write("seed:=" + " ".rjust(10) + str(int(seed)) + "\n")
        f.write(lst("eigenvalues:=", eigenvalues, n))
        f.write(lst("norm:=", norm, n + 1))
        f.write(lst("overlap:=", overlap, n))
        f.write(lst("psi_0:=", psi_0, n))
        f.write(lst("psi_n0:=", psi_n0, n))


def read_lanczos_text(filename):
    """Reads the checkpoint text as the reference's read_from_file does: token by token."""
    tok = open(filename).read().split()
    pos = 0

    def nxt():
        nonlocal pos
        pos += 1
        return tok[pos - 1]

    out = {}
    for key in ("nHilbert", "lambda", "seed"):
        nxt()
        out[key] = int(nxt())
    n = out["lambda"]
    for key, count in (("eigenvalues", n), ("norm", n + 1), ("overlap", n), ("psi_0", n), ("psi_n0", n)):
        nxt()
        nxt()
        vals = []
        for _ in range(count):
            vals.append(float(nxt()))
            nxt()
        nxt()
        out[key] = vals
    return out


class lhamil:
    """BLQH_without_spin/lanczos_hamiltonian.h:11-75 on the GPU.

    set_hamil builds the CSR on the device; coeff_explicit_update runs Lanczos
    pass 1 (full FP64 reorthogonalization, stopping at convergence or at an
    invariant subspace, at most lambda steps); diag solves the tridiagonal on
    the device; eigenstates_reconstruction forms the ground state from the
    stored Krylov basis; ground_state_energy returns <psi|H|psi>.
    precision = VAL_FP32 stores FP32 values and finishes with the FP64
    regenerated Rayleigh quotient."""

    def __init__(self, lambda_=200, seed=1, precision=VAL_FP64, tol=1e-12, reorth=True, compat_conj=False):
        self.compat_conj = compat_conj  # ground_state_energy as the reference prints it (conjugated state)
        self.lambda_ = lambda_
        self.seed = seed
        self.precision = precision
        self.tol = tol
        self.reorth = reorth
        self.sector = basis()
        self.nHilbert = 0
        self.norm, self.overlap, self.eigenvalues, self.psi_0 = [], [], [], []
        self.psir_0 = np.zeros(0, np.complex128)
        self.E0 = 0.0
        self.H = None
        self._L = None

    def set_hamil(self, lx, ly, nphi, nLL, d, Delta_SAS, Delta_V, theta_x=0.0, theta_y=0.0, nthread=1):
        if self.sector._b is None:
            self.sector.init()
        self.nphi, self.lx, self.ly, self.d = nphi, lx, ly, d
        self.H = Hamiltonian(self.sector._b, d, Delta_SAS, Delta_V, nLL, 1.0, theta_x, theta_y, self.precision,
                             lx=lx, ly=ly)
        self.nHilbert = self.H.dim

    def coeff_explicit_update(self):
        self._L = Lanczos(self.H, self.lambda_, self.reorth, self.tol, 10, self.seed, 0)
        self._L.iterate()
        a, b = self._L.coeffs()
        self.overlap, self.norm = list(a), list(b)

    def diag(self):
        e, y = self._L.eig()
        self.eigenvalues, self.psi_0 = list(e), list(y)
        # first components of the Ritz vectors in the Krylov basis (lanczos_hamiltonian.cpp:597-603)
        m = len(self.overlap)
        T = np.diag(np.asarray(self.overlap, float)) + np.diag(np.asarray(self.norm[1:m], float), 1) \
            + np.diag(np.asarray(self.norm[1:m], float), -1)
        self.psi_n0 = list(np.linalg.eigh(T)[1][0]) if m else []

    def save_to_file(self, filename):
        """The reference's checkpoint text (lanczos_hamiltonian.cpp:738-766); lambda
        is written as the number of steps taken, the length of every list."""
        save_lanczos_text(filename, self.nHilbert, len(self.overlap), self.seed, self.eigenvalues, self.norm,
                          self.overlap, self.psi_0, getattr(self, "psi_n0", []))

    def read_from_file(self, filename):
        """lanczos_hamiltonian.cpp:768-819."""
        d = read_lanczos_text(filename)
        self.nHilbert, self.lambda_, self.seed = d["nHilbert"], d["lambda"], d["seed"]
        self.eigenvalues, self.norm, self.overlap = d["eigenvalues"], d["norm"], d["overlap"]
        self.psi_0, self.psi_n0 = d["psi_0"], d["psi_n0"]

    def eigenstates_reconstruction(self):
        self.E0 = self.eigenvalues[0]
        self.psir_0 = self._L.ritz_vector().astype(np.complex128)

    def occupatation_number(self, alpha, j):
        """lanczos_hamiltonian.cpp:658-678 (the reference's spelling)."""
        return float(self._L.observables(self.sector._b)["occupation"][alpha][j])

    def pseudospin_Sz(self):
        """lanczos_hamiltonian.cpp:680-689."""
        return self._L.observables(self.sector._b)["Sz"]

    def pseudospin_Sx(self):
        """lanczos_hamiltonian.cpp:691-736."""
        return self._L.observables(self.sector._b)["Sx"]

    def ground_state_energy(self):
        if self.compat_conj:
            return self._L.rayleigh_conj()
        if self.precision == VAL_FP64:
            return self._L.rayleigh()
        return self._L.rayleigh_fp64()
