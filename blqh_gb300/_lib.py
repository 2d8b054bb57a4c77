"""Loads libblqh_gpu.so and declares the C ABI of include/blqh_gpu.h for ctypes."""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libblqh_gpu.so")

OK = 0
ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_UNSUPPORTED, ERR_CAPACITY, ERR_STATE, ERR_TIMEOUT = -1, -2, -3, -4, -5, -6, -7
REP_REFERENCE, REP_MIN = 0, 1
VAL_FP64, VAL_FP32 = 0, 1


class BlqhError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"blqh error {code}: {msg}")
        self.code = code


class Sector(ctypes.Structure):
    _fields_ = [("nphi", ctypes.c_int), ("nel", ctypes.c_int), ("nel_up", ctypes.c_int), ("J", ctypes.c_int),
                ("K", ctypes.c_int), ("rep_mode", ctypes.c_int)]


class Params(ctypes.Structure):
    _fields_ = [("lx", ctypes.c_double), ("ly", ctypes.c_double), ("d", ctypes.c_double),
                ("delta_sas", ctypes.c_double), ("delta_v", ctypes.c_double), ("theta_x", ctypes.c_double),
                ("theta_y", ctypes.c_double), ("nLL", ctypes.c_int)]


class LanczosOpts(ctypes.Structure):
    _fields_ = [("max_steps", ctypes.c_int), ("reorth", ctypes.c_int), ("tol", ctypes.c_double),
                ("check_every", ctypes.c_int), ("seed", ctypes.c_uint64), ("rng", ctypes.c_int),
                ("accumulate", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("ritz0", ctypes.c_double), ("steps", ctypes.c_int),
                ("dim", ctypes.c_int64), ("nnz", ctypes.c_int64)]


MODEL_SPINLESS, MODEL_SPINFUL, MODEL_MONOLAYER = 0, 1, 2


class SectorSpin(ctypes.Structure):
    _fields_ = [("nphi", ctypes.c_int), ("nel", ctypes.c_int), ("nel_up", ctypes.c_int), ("nel_su", ctypes.c_int),
                ("J", ctypes.c_int), ("K", ctypes.c_int), ("rep_mode", ctypes.c_int)]


class ParamsSpin(ctypes.Structure):
    _fields_ = [("lx", ctypes.c_double), ("ly", ctypes.c_double), ("d", ctypes.c_double),
                ("delta_sas", ctypes.c_double), ("delta_v", ctypes.c_double), ("delta_z", ctypes.c_double),
                ("theta_b", ctypes.c_double), ("theta_x", ctypes.c_double), ("theta_y", ctypes.c_double),
                ("nLL", ctypes.c_int)]


class SectorMono(ctypes.Structure):
    _fields_ = [("nphi", ctypes.c_int), ("nel", ctypes.c_int), ("J", ctypes.c_int), ("K", ctypes.c_int),
                ("rep_mode", ctypes.c_int)]


class ParamsMono(ctypes.Structure):
    _fields_ = [("lx", ctypes.c_double), ("ly", ctypes.c_double), ("nLL", ctypes.c_int)]


class Instance(ctypes.Structure):
    _fields_ = [("model", ctypes.c_int), ("sector", Sector), ("params", Params), ("ssector", SectorSpin),
                ("sparams", ParamsSpin), ("msector", SectorMono), ("mparams", ParamsMono)]


class BatchOpts(ctypes.Structure):
    _fields_ = [("lambda_", ctypes.c_int), ("value_precision", ctypes.c_int), ("seed", ctypes.c_uint64),
                ("threads", ctypes.c_int), ("lanes_per_row", ctypes.c_int), ("use_graph", ctypes.c_int)]


class BatchResult(ctypes.Structure):
    _fields_ = [("energy", ctypes.c_double), ("ritz0", ctypes.c_double), ("resid", ctypes.c_double),
                ("dim", ctypes.c_int64), ("nnz", ctypes.c_int64), ("steps", ctypes.c_int),
                ("second_passes", ctypes.c_int)]


# (name, restype, argtypes) for every entry point of include/blqh_gpu.h
_vp, _i, _i64, _u64, _d = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double
_P = ctypes.POINTER
SIGNATURES = [
    ("blqh_ctx_create", _i, [_i, _P(_vp)]),
    ("blqh_ctx_destroy", _i, [_vp]),
    ("blqh_last_error", ctypes.c_char_p, [_vp]),
    ("blqh_ctx_synchronize", _i, [_vp]),
    ("blqh_ctx_timers", _i, [_vp, _i, _P(_d), _P(_i64)]),
    ("blqh_ctx_reset_timers", _i, [_vp]),
    ("blqh_ctx_mark", _i, [_vp, _i]),
    ("blqh_ctx_elapsed_ms", _i, [_vp, _i, _i, _P(_d)]),
    ("blqh_basis_build", _i, [_vp, _P(Sector), _P(_vp)]),
    ("blqh_basis_size", _i, [_vp, _P(_i64)]),
    ("blqh_basis_get", _i, [_vp, _vp, _vp, _vp]),
    ("blqh_basis_destroy", _i, [_vp]),
    ("blqh_hamil_build", _i, [_vp, _vp, _P(Params), _i, _P(_vp)]),
    ("blqh_csr_info", _i, [_vp, _P(_i64), _P(_i64), _P(_i), _P(_i)]),
    ("blqh_csr_get", _i, [_vp, _vp, _vp, _vp, _vp]),
    ("blqh_csr_destroy", _i, [_vp]),
    ("blqh_spmv", _i, [_vp, _vp, _vp, _vp]),
    ("blqh_lanczos_create", _i, [_vp, _vp, _P(LanczosOpts), _P(_vp)]),
    ("blqh_lanczos_set_start", _i, [_vp, _vp]),
    ("blqh_lanczos_iterate", _i, [_vp, _P(_i)]),
    ("blqh_lanczos_coeffs", _i, [_vp, _vp, _vp]),
    ("blqh_lanczos_eig", _i, [_vp, _vp, _vp]),
    ("blqh_lanczos_ritz_vector", _i, [_vp, _vp]),
    ("blqh_lanczos_rayleigh", _i, [_vp, _P(_d)]),
    ("blqh_lanczos_rayleigh_fp64", _i, [_vp, _vp, _vp, _P(_d)]),
    ("blqh_lanczos_rayleigh_conj", _i, [_vp, _vp, _vp, _P(_d)]),
    ("blqh_lanczos_observables_spin", _i, [_vp, _vp, _vp]),
    ("blqh_lanczos_rayleigh_fp64_spin", _i, [_vp, _vp, _vp, _P(_d)]),
    ("blqh_hamil_build_spin_prec", _i, [_vp, _vp, _vp, _i, _vp]),
    ("blqh_lanczos_destroy", _i, [_vp]),
    ("blqh_ground_state", _i, [_vp, _P(Sector), _P(Params), _i, _P(LanczosOpts), _vp, _vp, _P(Result)]),
    ("blqh_start_vector", _i, [_u64, _i, _i64, _i, _vp]),
    ("blqh_spmv_f32_noalloc", _i, [_vp, _vp, _vp, _i64, _vp, _vp, _vp]),
]
SIGNATURES += [
    ("blqh_lanczos_observables", _i, [_vp, _vp, _P(_d), _P(_d), _vp]),
]

SIGNATURES += [
    ("blqh_basis_build_spin", _i, [_vp, _P(SectorSpin), _P(_vp)]),
    ("blqh_hamil_build_spin", _i, [_vp, _vp, _P(ParamsSpin), _P(_vp)]),
]

SIGNATURES += [
    ("blqh_basis_build_mono", _i, [_vp, _P(SectorMono), _P(_vp)]),
    ("blqh_hamil_build_mono", _i, [_vp, _vp, _P(ParamsMono), _P(_vp)]),
    ("blqh_mono_classical_energy", _i, [_i, _d, _d, _P(_d)]),
    ("blqh_mono_coulomb_table", _i, [_i, _d, _d, _i, _vp]),
]

SIGNATURES += [
    ("blqh_batch_create", _i, [_vp, _P(Instance), _i, _P(BatchOpts), _P(_vp)]),
    ("blqh_batch_solve", _i, [_vp]),
    ("blqh_batch_results", _i, [_vp, _P(BatchResult)]),
    ("blqh_batch_ground_state", _i, [_vp, _i, _vp]),
    ("blqh_batch_shape", _i, [_vp, _P(_i), _P(_i), _P(_i)]),
    ("blqh_batch_timing", _i, [_vp, _P(_d), _P(_d), _P(_i)]),
    ("blqh_batch_destroy", _i, [_vp]),
    ("blqh_batch_run", _i, [_vp, _P(Instance), _i, _P(BatchOpts), _P(BatchResult)]),
]

_f = ctypes.c_float
SIGNATURES += [
    ("blqh_mlp_create", _i, [_vp, _i, _i, _u64, _P(_vp)]),
    ("blqh_mlp_num_params", _i, [_vp, _P(_i64)]),
    ("blqh_mlp_get_params", _i, [_vp, _vp]),
    ("blqh_mlp_set_params", _i, [_vp, _vp]),
    ("blqh_mlp_predict", _i, [_vp, _vp, _d, _d, _vp]),
    ("blqh_mlp_loss_grad", _i, [_vp, _vp, _i, _vp, _vp, _P(_d), _vp]),
    ("blqh_mlp_train", _i, [_vp, _vp, _i, _vp, _vp, _i, _d, _vp]),
    ("blqh_mlp_destroy", _i, [_vp]),
]

DEBUG_SIGNATURES = [
    ("blqh_debug_sector_index", _i, [_P(Sector), _i64, _vp, _vp, _P(_i64)]),
    ("blqh_debug_spmv_layout", _i, [_vp]),
]

_lib = None


def lib():
    """The loaded library. Raises if it was not built: there is no fallback."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m blqh_gb300.build` "
                               "(the CUDA library is required; there is no CPU path)")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES + DEBUG_SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc, ctx=None):
    if rc != OK:
        msg = lib().blqh_last_error(ctx)
        raise BlqhError(rc, msg.decode() if msg else "")
    return rc
