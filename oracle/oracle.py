"""ctypes wrapper over the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py`` -- never by the product package
``blqh_gb300``. The C++ restatement it wraps (oracle/blqh_oracle.cpp) follows
BLQH_without_spin/{basis,lanczos_hamiltonian}.cpp of the reference line by line.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_lib = None


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        vp, i64, u64, i32, d = ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint64, ctypes.c_int, ctypes.c_double
        L.orc_basis_new.restype = vp
        L.orc_basis_new.argtypes = [i32, i32, i32, i32, i32, i32]
        L.orc_basis_free.argtypes = [vp]
        L.orc_basis_size.restype = i64
        L.orc_basis_size.argtypes = [vp]
        L.orc_basis_ids.argtypes = [vp, vp]
        L.orc_basis_periods.argtypes = [vp, vp]
        L.orc_basis_inserted.restype = i64
        L.orc_basis_inserted.argtypes = [vp, vp]
        L.orc_basis_iterated.restype = i64
        L.orc_basis_iterated.argtypes = [vp, vp]
        L.orc_translate.restype = u64
        L.orc_translate.argtypes = [vp, u64, i32, i32, ctypes.POINTER(i32)]
        L.orc_coulomb_tables.argtypes = [i32, i32, i32, d, d, d, d, vp, vp, vp]
        L.orc_hamil_new.restype = vp
        L.orc_hamil_new.argtypes = [vp, d, d, i32, d, d, d, d, d, i32, i64, i64]
        L.orc_hamil_new_rows.restype = vp
        L.orc_hamil_new_rows.argtypes = [vp, d, d, i32, d, d, d, d, d, i32, vp, i64]
        L.orc_hamil_free.argtypes = [vp]
        L.orc_hamil_nnz.restype = i64
        L.orc_hamil_nnz.argtypes = [vp]
        L.orc_hamil_rows.restype = i64
        L.orc_hamil_rows.argtypes = [vp]
        L.orc_hamil_csr.argtypes = [vp, vp, vp, vp]
        L.orc_spmv.argtypes = [vp, vp, vp, i32]
        L.orc_start_vector.argtypes = [i64, ctypes.c_uint32, vp]
        L.orc_spmv_stream_time.restype = d
        L.orc_spmv_stream_time.argtypes = [vp, i32, i32, i32]
        L.orc_mt19937.argtypes = [ctypes.c_uint32, i64, vp]
        L.orc_lanczos.argtypes = [vp, i32, vp, vp, vp, i32]
        L.orc_mono_basis_new.restype = vp
        L.orc_mono_basis_new.argtypes = [i32, i32, i32, i32, i32]
        L.orc_mono_basis_free.argtypes = [vp]
        L.orc_mono_basis_size.restype = i64
        L.orc_mono_basis_size.argtypes = [vp]
        L.orc_mono_basis_ids.argtypes = [vp, vp]
        L.orc_mono_basis_periods.argtypes = [vp, vp]
        L.orc_mono_translate.restype = u64
        L.orc_mono_translate.argtypes = [vp, u64, i32, i32, ctypes.POINTER(i32)]
        L.orc_mono_classical_energy.restype = d
        L.orc_mono_classical_energy.argtypes = [i32, d, d]
        L.orc_mono_coulomb_table.argtypes = [i32, d, d, i32, vp]
        L.orc_mono_hamil_new.restype = vp
        L.orc_mono_hamil_new.argtypes = [vp, d, d, i32, i32, i64, i64]
        L.orc_mono_hamil_rows.restype = i64
        L.orc_mono_hamil_rows.argtypes = [vp]
        L.orc_mono_spmv.argtypes = [vp, vp, vp, i32]
        L.orc_mono_hamil_free.argtypes = [vp]
        L.orc_mono_hamil_nnz.restype = i64
        L.orc_mono_hamil_nnz.argtypes = [vp]
        L.orc_mono_hamil_csr.argtypes = [vp, vp, vp, vp]
        _lib = L
    return _lib


def torus(nphi: int, gamma: float = 1.0):
    """lx, ly of the square (gamma = 1) torus, as BLQH_without_spin/main.cpp:20-21."""
    ly = np.sqrt(nphi * 2.0 * np.pi / gamma)
    return ly * gamma, ly


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


class Basis:
    """Sector basis (basis.cpp:61-119). rep_mode 0 keeps the reference's survivor."""

    def __init__(self, nphi, nel, nel_up, J, K, rep_mode=0):
        self.nphi, self.nel, self.nel_up, self.J, self.K = nphi, nel, nel_up, J, K
        self.h = lib().orc_basis_new(nphi, nel, nel_up, J, K, rep_mode)
        if not self.h:
            raise ValueError("oracle: unsupported sector")
        n = lib().orc_basis_size(self.h)
        self.id = np.zeros(n, np.uint64)
        self.period = np.zeros(n, np.int16)
        if n:
            lib().orc_basis_ids(self.h, _ptr(self.id))
            lib().orc_basis_periods(self.h, _ptr(self.period))

    @property
    def dim(self):
        return len(self.id)

    def inserted(self):
        n = lib().orc_basis_inserted(self.h, None)
        a = np.zeros(n, np.uint64)
        if n:
            lib().orc_basis_inserted(self.h, _ptr(a))
        return a

    def iterated(self):
        n = lib().orc_basis_iterated(self.h, None)
        a = np.zeros(n, np.uint64)
        if n:
            lib().orc_basis_iterated(self.h, _ptr(a))
        return a

    def translate(self, c, k, inverse=False):
        s = ctypes.c_int(0)
        r = lib().orc_translate(self.h, int(c), int(k), int(inverse), ctypes.byref(s))
        return int(r), s.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_basis_free(self.h)
            self.h = None


def coulomb_tables(nphi, K, d, nLL=0, gamma=1.0, theta_x=0.0):
    lx, ly = torus(nphi, gamma)
    V = np.zeros(2 * nphi * nphi)
    Ec = np.zeros(1)
    FT = np.zeros(nphi * nphi, np.complex128)
    lib().orc_coulomb_tables(nphi, K, nLL, lx, ly, d, theta_x, _ptr(V), _ptr(Ec), _ptr(FT))
    return V.reshape(2, nphi, nphi), float(Ec[0]), FT.reshape(nphi, nphi)


class Hamil:
    """Row generator of lanczos_hamiltonian.cpp:87-358 into complex CSR: all rows, rows=(r0, r1)
    for [r0, r1), or rows=<array of row indices> for those rows in that order."""

    def __init__(self, basis: Basis, d, dsas=0.0, dv=0.0, nLL=0, gamma=1.0, theta_x=0.0, theta_y=0.0,
                 nthreads=None, rows=None):
        self.basis = basis
        lx, ly = torus(basis.nphi, gamma)
        nthreads = nthreads or os.cpu_count() or 1
        if rows is not None and not isinstance(rows, tuple):  # an explicit row list
            self.rows = np.ascontiguousarray(rows, np.int64)
            self.h = lib().orc_hamil_new_rows(basis.h, lx, ly, nLL, d, dsas, dv, theta_x, theta_y, nthreads,
                                              _ptr(self.rows), len(self.rows))
        else:
            r0, r1 = rows if rows is not None else (0, -1)
            self.h = lib().orc_hamil_new(basis.h, lx, ly, nLL, d, dsas, dv, theta_x, theta_y, nthreads, r0, r1)
        self.nthreads = nthreads
        nnz = lib().orc_hamil_nnz(self.h)
        nrows = lib().orc_hamil_rows(self.h)
        self.row_ptr = np.zeros(nrows + 1, np.int64)
        self.col = np.zeros(nnz, np.int64)
        self.val = np.zeros(nnz, np.complex128)
        lib().orc_hamil_csr(self.h, _ptr(self.row_ptr), _ptr(self.col), _ptr(self.val))

    @property
    def nnz(self):
        return len(self.col)

    def dense(self):
        n = self.basis.dim
        M = np.zeros((n, n), np.complex128)
        for i in range(n):
            s, e = self.row_ptr[i], self.row_ptr[i + 1]
            M[i, self.col[s:e]] = self.val[s:e]
        return M

    def spmv(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.complex128)
        y = np.zeros(len(self.row_ptr) - 1, np.complex128)
        lib().orc_spmv(self.h, _ptr(x), _ptr(y), self.nthreads)
        return y

    def spmv_stream_time(self, copies=10, reps=5):
        """Seconds per product over `copies` distinct replicas of this handle's rows (a timing probe)."""
        return float(lib().orc_spmv_stream_time(self.h, copies, reps, self.nthreads))

    def lanczos(self, lam=200, seed=1):
        """Reference recurrence (lanczos_hamiltonian.cpp:453-579): alpha[lam], beta[lam+1]."""
        n = self.basis.dim
        x = start_vector(n, seed)
        a = np.zeros(lam)
        b = np.zeros(lam + 1)
        lib().orc_lanczos(self.h, lam, _ptr(x), _ptr(a), _ptr(b), self.nthreads)
        return a, b

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_hamil_free(self.h)
            self.h = None


def start_vector(dim, seed):
    x = np.zeros(dim, np.complex128)
    lib().orc_start_vector(dim, seed, _ptr(x))
    return x


def mt19937(seed, n):
    a = np.zeros(n, np.uint32)
    lib().orc_mt19937(seed, n, _ptr(a))
    return a


def tridiag_eigenvalues(alpha, beta):
    """Eigenvalues of the Lanczos tridiagonal (diag alpha, off-diagonal beta[1:])."""
    from scipy.linalg import eigh_tridiagonal

    lam = len(alpha)
    return eigh_tridiagonal(alpha, beta[1:lam], eigvals_only=True)


# ---- monolayer (Monolayer/basis.cpp, Monolayer/lanczos_hamiltonian.cpp) ----
def mono_torus(nphi: int, gamma: float):
    """lx, ly of Monolayer/main.cpp:33-34 (ly = sqrt(2 pi nphi / gamma), lx = gamma ly)."""
    ly = np.sqrt(2.0 * np.pi * nphi / gamma)
    return ly * gamma, ly


class MonoBasis:
    """Monolayer sector basis (Monolayer/basis.cpp:59-119); rep_mode 0 keeps the reference's survivor."""

    def __init__(self, nphi, nel, J=-1, K=-1, rep_mode=0):
        self.nphi, self.nel, self.J, self.K = nphi, nel, J, K
        self.C = int(np.gcd(nphi, nel))
        self.h = lib().orc_mono_basis_new(nphi, nel, J, K, rep_mode)
        n = lib().orc_mono_basis_size(self.h)
        self.id = np.zeros(n, np.uint64)
        self.period = np.zeros(n, np.int16)
        if n:
            lib().orc_mono_basis_ids(self.h, _ptr(self.id))
            lib().orc_mono_basis_periods(self.h, _ptr(self.period))

    @property
    def dim(self):
        return len(self.id)

    def translate(self, c, k, inverse=False):
        s = ctypes.c_int(0)
        r = lib().orc_mono_translate(self.h, int(c), int(k), int(inverse), ctypes.byref(s))
        return int(r), s.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mono_basis_free(self.h)
            self.h = None


def mono_classical_energy(nphi, lx, ly):
    return float(lib().orc_mono_classical_energy(nphi, lx, ly))


def mono_coulomb_table(nphi, lx, ly, nLL=0):
    V = np.zeros(nphi * nphi)
    lib().orc_mono_coulomb_table(nphi, lx, ly, nLL, _ptr(V))
    return V.reshape(nphi, nphi)


class MonoHamil:
    """Monolayer row generator (Monolayer/lanczos_hamiltonian.cpp:77-198) into complex CSR."""

    def __init__(self, basis: MonoBasis, lx, ly, nLL=0, nthreads=None, rows=None):
        self.basis = basis
        nthreads = nthreads or os.cpu_count() or 1
        self.nthreads = nthreads
        r0, r1 = rows if rows is not None else (0, -1)
        self.h = lib().orc_mono_hamil_new(basis.h, lx, ly, nLL, nthreads, r0, r1)
        nnz = lib().orc_mono_hamil_nnz(self.h)
        self.row_ptr = np.zeros(lib().orc_mono_hamil_rows(self.h) + 1, np.int64)
        self.col = np.zeros(nnz, np.int64)
        self.val = np.zeros(nnz, np.complex128)
        lib().orc_mono_hamil_csr(self.h, _ptr(self.row_ptr), _ptr(self.col), _ptr(self.val))

    @property
    def nnz(self):
        return len(self.col)

    def dense(self):
        n = self.basis.dim
        M = np.zeros((n, n), np.complex128)
        for i in range(n):
            s, e = self.row_ptr[i], self.row_ptr[i + 1]
            M[i, self.col[s:e]] = self.val[s:e]
        return M

    def sparse(self):
        from scipy.sparse import csr_matrix

        n = self.basis.dim
        return csr_matrix((self.val, self.col, self.row_ptr), shape=(len(self.row_ptr) - 1, n))

    def spmv(self, x):
        x = np.ascontiguousarray(x, np.complex128)
        y = np.zeros(len(self.row_ptr) - 1, np.complex128)
        lib().orc_mono_spmv(self.h, _ptr(x), _ptr(y), self.nthreads)
        return y

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mono_hamil_free(self.h)
            self.h = None
