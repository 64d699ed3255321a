"""ctypes binding of libjcg.so (the C ABI declared in include/jcg.h).

The library is loaded from this package's directory.  There is no fallback: if
``libjcg.so`` is missing or a call fails, an exception is raised.  Errors map to
the exceptions the reference raises for the same conditions (``ValueError`` for
an odd Simpson N, scipy/integrate.py:193; ``NotImplementedError`` for
unsupported options, transfer.py:155 / power.py:226).
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libjcg.so")

ABI_VERSION = 3
MAX_TRACERS = 16
MAX_PAIRS = MAX_TRACERS * (MAX_TRACERS + 1) // 2
MAX_ELL = 4096
MAX_LIMBER = 4096
NOALLOC_SCRATCH_BYTES = 32 * 1024 * 1024

OK = 0
ERR_ARG = -1
ERR_SHAPE = -2
ERR_ODD_N = -3
ERR_VALUE = -4
ERR_WORKSPACE = -5
ERR_CUDA = -6
ERR_UNSUPPORTED = -7
ERR_TIMEOUT = -8
ERR_ABI = -9

TRACER_WL = 0
TRACER_NC = 1
BIAS_NONE, BIAS_CONSTANT, BIAS_INV_GROWTH, BIAS_DES_Y1 = 0, 1, 2, 3
NZ_SMAIL, NZ_TABLE, NZ_DELTA = 0, 1, 2
FP64 = 0
FP32C = 1
# physics switches (jcg_geometry.physics; bits 8+ of jcg_eval_points' what)
PK_TAKAHASHI2012, PK_SMITH2003, PK_LINEAR = 0, 1, 2
TF_NOWIGGLE = 0x10
GROWTH_GAMMA = 0x20

EVAL_CHI, EVAL_GROWTH, EVAL_H, EVAL_DCHI, EVAL_TRANSFER, EVAL_PLIN, EVAL_PNL = range(7)
EVAL_KNL, EVAL_NEFF, EVAL_C = 7, 8, 9
EVAL_TRANSVERSE, EVAL_DA, EVAL_A_OF_CHI, EVAL_GROWTH_RATE = 10, 11, 12, 13

REQ_CL, REQ_JACOBIAN, REQ_LOGLIKE_GRAD = 0, 1, 2
MAX_REQUESTS = 65536
# jcg_request (include/jcg.h): eight pointers, filled column-wise for a batch
REQUEST_DTYPE = np.dtype([(n, np.uint64) for n in ("g", "geo", "params", "cl", "jac", "data", "prec", "out")])


class JcgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libjcg error {code}: {msg}")
        self.code = code


class Geometry(ctypes.Structure):
    """Mirror of ``jcg_geometry`` (include/jcg.h)."""

    _fields_ = [
        ("abi_version", ctypes.c_int),
        ("n_tracers", ctypes.c_int),
        ("n_ell", ctypes.c_int),
        ("n_limber", ctypes.c_int),
        ("n_nodes", ctypes.c_int),
        ("zmax", ctypes.c_double),
        ("kind", ctypes.c_int * MAX_TRACERS),
        ("nz_a", ctypes.c_double * MAX_TRACERS),
        ("nz_b", ctypes.c_double * MAX_TRACERS),
        ("nz_z0", ctypes.c_double * MAX_TRACERS),
        ("nz_zmax", ctypes.c_double * MAX_TRACERS),
        ("probe_zmax", ctypes.c_double * MAX_TRACERS),
        ("bias", ctypes.c_double * MAX_TRACERS),
        ("mult", ctypes.c_double * MAX_TRACERS),
        ("noise", ctypes.c_double * MAX_TRACERS),
        ("bias_kind", ctypes.c_int * MAX_TRACERS),
        ("bias_eta", ctypes.c_double * MAX_TRACERS),
        ("bias_z0", ctypes.c_double * MAX_TRACERS),
        ("nz_kind", ctypes.c_int * MAX_TRACERS),
        ("physics", ctypes.c_int),
    ]


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_SZ = ctypes.c_size_t
_PSZ = ctypes.POINTER(ctypes.c_size_t)
_PG = ctypes.POINTER(Geometry)

# name -> argtypes (all return int unless listed in _RESTYPES)
SIGNATURES = {
    "jcg_abi_version": [],
    "jcg_last_error_string": [],
    "jcg_geometry_size": [_PG, _PSZ],
    "jcg_geometry_build": [_PG, _P, _P, _SZ, _P],
    "jcg_geometry_build_nodes": [_PG, _P, _P, _P, _SZ, _P],
    "jcg_geometry_nz_points": [_PG, _P, _P, _PSZ, _P],
    "jcg_geometry_build_nz": [_PG, _P, _P, _P, _SZ, _P, _SZ, _P],
    "jcg_workspace_size": [_PG, _I, _I, _PSZ],
    "jcg_angular_cl": [_PG, _P, _P, _I, _I, _P, _P, _SZ, _P],
    "jcg_angular_cl_noalloc": [_PG, _P, _P, _I, _I, _P, _P],
    "jcg_host_workspace_size": [_PG, _I, _I, _PSZ],
    "jcg_angular_cl_host": [_PG, _P, _P, _I, _I, _P, _P, _SZ, _P],
    "jcg_stage_cosmo_tables": [_PG, _P, _I, _I, _P, _SZ, _P],
    "jcg_stage_halofit_rows": [_PG, _P, _P, _I, _I, _P, _SZ, _P],
    "jcg_stage_tracer_kernels": [_PG, _P, _P, _I, _I, _P, _SZ, _P],
    "jcg_stage_limber": [_PG, _P, _P, _I, _I, _P, _P, _SZ, _P],
    "jcg_workspace_read": [_PG, _I, _I, _P, _I, _I, _P, _SZ, _P],
    "jcg_eval_points": [_P, _I, _P, _P, _I, _I, _P, _P, _SZ, _P],
    "jcg_eval_workspace_size": [_I, _PSZ],
    "jcg_gaussian_covariance": [_P, _I, _I, _P, _P, _P, _I, _D, _I, _P, _P],
    "jcg_gaussian_loglike_sparse": [_P, _P, _P, _I, _I, _I, _I, _P, _P, _P, _P, _SZ, _P],
    "jcg_loglike_workspace_size": [_I, _I, _I, _PSZ],
    "jcg_gaussian_loglike_dense": [_P, _P, _P, _I, _I, _I, _I, _P, _P, _P, _P, _SZ, _P],
    "jcg_jacobian_workspace_size": [_PG, _I, _I, _PSZ],
    "jcg_angular_cl_jacobian": [_PG, _P, _P, _I, _I, _P, _P, _P, _SZ, _P],
    "jcg_angular_cl_jacobian_dir": [_PG, _P, _P, _I, _I, _I, _P, _P, _P, _SZ, _P],
    "jcg_angular_cl_jacobian_branch": [_PG, _P, _P, _I, _P, _P, _P, _P, _P, _SZ, _P],
    "jcg_vjp_workspace_size": [_PG, _I, _I, _PSZ],
    "jcg_angular_cl_vjp": [_PG, _P, _P, _I, _I, _I, _P, _P, _P, _P, _SZ, _P],
    "jcg_requests_workspace_size": [_P, _I, _I, _I, _PSZ, _PSZ],
    "jcg_requests_run": [_P, _I, _I, _I, _P, _SZ, _P],
    "jcg_sparse_inv_batched": [_P, _I, _I, _I, _P, _P],
    "jcg_sparse_dot_sparse": [_P, _I, _I, _I, _I, _P, _P, _P],
    "jcg_sparse_dot_dense": [_P, _I, _I, _I, _P, _I, _P, _P],
    "jcg_dense_dot_sparse": [_P, _I, _P, _I, _I, _I, _P, _P],
    "jcg_dense_dot_sparse_dot_dense": [_P, _I, _P, _I, _I, _I, _P, _I, _P, _P, _P],
    "jcg_calib_peak_fp64": [_P, _I, _I, _P],
    "jcg_calib_peak_mufu": [_P, _I, _I, _P],
    "jcg_calib_vjp_stages": [_PG, _P, _P, _I, _P, _P, _P, _P, _SZ, ctypes.c_uint, _P],
    "jcg_sparse_inv": [_P, _I, _I, _P, _P],
    "jcg_sparse_slogdet": [_P, _I, _I, _P, _P, _P, _P],
    "jcg_sparse_to_dense": [_P, _I, _I, _I, _P, _P],
    "jcg_sparse_dot_vec": [_P, _I, _I, _I, _P, _I, _P, _P],
}
_RESTYPES = {"jcg_last_error_string": ctypes.c_char_p}

_lib = None
_lock = threading.Lock()


def load():
    """Load libjcg.so (once).  Raises if it is not built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with `python -m jax_cosmo_gb300.build` "
                "(there is no CPU fallback)"
            )
        lib = ctypes.CDLL(LIB_PATH)
        for name, argtypes in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argtypes
            fn.restype = _RESTYPES.get(name, ctypes.c_int)
        if lib.jcg_abi_version() != ABI_VERSION:
            raise RuntimeError("libjcg ABI version mismatch")
        _lib = lib
        return lib


def check(rc):
    if rc == OK:
        return
    msg = load().jcg_last_error_string().decode(errors="replace")
    if rc == ERR_ODD_N:
        raise ValueError(msg)
    if rc == ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if rc in (ERR_ARG, ERR_SHAPE, ERR_VALUE, ERR_ABI):
        raise ValueError(msg)
    raise JcgError(rc, msg)


def call(name, *args):
    check(getattr(load(), name)(*args))


def ptr(t):
    """Device pointer of a tensor (or None)."""
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def stream_of(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def require_cuda(device=None):
    if not torch.cuda.is_available():
        raise RuntimeError("jax_cosmo_gb300 needs a CUDA GPU (there is no CPU fallback)")
    load()
    return torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)


def workspace(nbytes, device):
    """A 256-byte aligned device buffer from torch's caching allocator."""
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
