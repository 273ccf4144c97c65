"""ctypes binding of the C oracle (TEST INFRASTRUCTURE ONLY).

The checker for the CUDA library: only tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` import this module.  Every function is a
thin wrapper over ``stencil_oracle.c``; see ``stencil_oracle.h`` for the
reference lines each one restates.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np

from . import build as _build

LEGACY = 0
JACOBI = 1

_lib = None
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        i, u64, sz, d = ctypes.c_int, ctypes.c_uint64, ctypes.c_size_t, ctypes.c_double
        L.oracle_sweep_f32.argtypes = [_f32p, _f32p, i, i, i, i, i, i, i]
        L.oracle_sweep_f64.argtypes = [_f64p, _f64p, i, i, i, i, i, i, i]
        L.oracle_run_f32.argtypes = [_f32p, _f32p, i, i, i, i, i, i, i, i]
        L.oracle_run_f32.restype = i
        L.oracle_run_f64.argtypes = [_f64p, _f64p, i, i, i, i, i, i, i, i]
        L.oracle_run_f64.restype = i
        L.oracle_init_reference.argtypes = [_f32p, i, i, i, i]
        L.oracle_uniform01.argtypes = [u64, u64]
        L.oracle_uniform01.restype = ctypes.c_float
        L.oracle_init_uniform.argtypes = [_f32p, sz, u64]
        L.oracle_copy_border.argtypes = [_f32p, _f32p, i, i, i, i, i]
        L.oracle_sq_err.argtypes = [_f32p, _f32p, sz]
        L.oracle_sq_err.restype = d
        L.oracle_max_rel_err.argtypes = [_f32p, _f32p, sz, d, ctypes.POINTER(sz)]
        L.oracle_max_rel_err.restype = d
        L.oracle_max_rel_err_f64.argtypes = [_f32p, _f64p, sz, d, ctypes.POINTER(sz)]
        L.oracle_max_rel_err_f64.restype = d
        L.oracle_rel_residual.argtypes = [_f32p, i, i, i, i, i, i]
        L.oracle_rel_residual.restype = d
        _lib = L
    return _lib


def _p32(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_f32p)


def _p64(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_f64p)


def _shape(a: np.ndarray):
    """numpy layout is [z][y][x] (x fastest), matching idx = i + j*NX + k*NX*NY."""
    if a.ndim == 2:
        return 2, a.shape[1], a.shape[0], 1
    if a.ndim == 3:
        return 3, a.shape[2], a.shape[1], a.shape[0]
    raise ValueError("grid must be 2-D or 3-D")


def default_threads() -> int:
    return int(os.environ.get("STENCIL_ORACLE_THREADS", os.cpu_count() or 1))


def sweep(src: np.ndarray, dst: np.ndarray, radius: int, mode: int, threads: int = 1):
    dims, nx, ny, nz = _shape(src)
    if src.dtype == np.float64:
        lib().oracle_sweep_f64(_p64(src), _p64(dst), dims, nx, ny, nz, radius, mode, threads)
    else:
        lib().oracle_sweep_f32(_p32(src), _p32(dst), dims, nx, ny, nz, radius, mode, threads)


def run(u1: np.ndarray, u2: np.ndarray, radius: int, mode: int, iterations: int,
        threads: int = 1) -> np.ndarray:
    """Ping-pong ``iterations`` sweeps in place; returns the array holding the result."""
    dims, nx, ny, nz = _shape(u1)
    if u1.dtype == np.float64:
        which = lib().oracle_run_f64(_p64(u1), _p64(u2), dims, nx, ny, nz, radius, mode,
                                     iterations, threads)
    else:
        which = lib().oracle_run_f32(_p32(u1), _p32(u2), dims, nx, ny, nz, radius, mode,
                                     iterations, threads)
    return u1 if which == 0 else u2


def init_reference(shape) -> np.ndarray:
    u = np.empty(shape, np.float32)
    dims, nx, ny, nz = _shape(u)
    lib().oracle_init_reference(_p32(u), dims, nx, ny, nz)
    return u


def uniform(shape, seed: int) -> np.ndarray:
    u = np.empty(shape, np.float32)
    lib().oracle_init_uniform(_p32(u), u.size, seed)
    return u


def uniform01(seed: int, idx: int) -> float:
    return lib().oracle_uniform01(seed, idx)


def copy_border(src: np.ndarray, dst: np.ndarray, radius: int):
    dims, nx, ny, nz = _shape(src)
    lib().oracle_copy_border(_p32(src), _p32(dst), dims, nx, ny, nz, radius)


def sq_err(a: np.ndarray, b: np.ndarray) -> float:
    return lib().oracle_sq_err(_p32(a), _p32(b), a.size)


def max_rel_err(a: np.ndarray, b: np.ndarray, floor: float = 1e-6):
    """Returns (max relative error, count of non-finite cells)."""
    bad = ctypes.c_size_t(0)
    a = np.ascontiguousarray(a, np.float32)
    if b.dtype == np.float64:
        e = lib().oracle_max_rel_err_f64(_p32(a), _p64(np.ascontiguousarray(b)), a.size,
                                         floor, ctypes.byref(bad))
    else:
        e = lib().oracle_max_rel_err(_p32(a), _p32(np.ascontiguousarray(b)), a.size, floor,
                                     ctypes.byref(bad))
    return e, bad.value


def rel_residual(u: np.ndarray, radius: int, threads: int = 1) -> float:
    dims, nx, ny, nz = _shape(u)
    return lib().oracle_rel_residual(_p32(np.ascontiguousarray(u, np.float32)), dims, nx,
                                     ny, nz, radius, threads)


def rms(a: np.ndarray, b: np.ndarray) -> float:
    """RMS as printed by include/stencil_error_checker.h:21."""
    return math.sqrt(sq_err(a, b) / a.size)
