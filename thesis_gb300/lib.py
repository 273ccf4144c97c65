"""ctypes binding of libstencil_gb300.so (the C ABI in include/stencil_dispatch.h).

The library is the in-tree build next to this file; importing this module
never falls back to anything else: if the shared library is missing or fails
to load, ``load()`` raises.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libstencil_gb300.so")
HEADER_DIR = os.path.join(os.path.dirname(HERE), "include")

OK, EINVAL, ENOMEM, ECUDA, ETIMEOUT, EUNSUPPORTED, ENODEVICE = 0, -1, -2, -3, -4, -5, -6
MODE_LEGACY, MODE_JACOBI = 0, 1
VARIANT_AUTO, VARIANT_BASE, VARIANT_SMEM, VARIANT_SMEM_PADDED = 0, 1, 2, 3
VARIANT_SMEM_REGISTER, VARIANT_COOP, VARIANT_CLUSTER = 4, 5, 6
VARIANT_NAMES = {
    "auto": VARIANT_AUTO, "base": VARIANT_BASE, "smem": VARIANT_SMEM,
    "smem_padded": VARIANT_SMEM_PADDED, "smem_register": VARIANT_SMEM_REGISTER,
    "coop": VARIANT_COOP, "cluster": VARIANT_CLUSTER,
}


class StencilError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        msg = "%s failed: %s (%d)" % (where, _strerror(status), status)
        if detail:
            msg += ": " + detail
        super().__init__(msg)


class BatchJob(ctypes.Structure):
    _fields_ = [
        ("d_u1", ctypes.c_void_p), ("d_u2", ctypes.c_void_p), ("dims", ctypes.c_int),
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("radius", ctypes.c_int), ("iterations", ctypes.c_int), ("mode", ctypes.c_int),
        ("temporal", ctypes.c_int), ("tile_x", ctypes.c_int), ("tile_y", ctypes.c_int),
        ("team", ctypes.c_int), ("reserved", ctypes.c_int * 2),
    ]


class IrParams(ctypes.Structure):
    _fields_ = [("storage", ctypes.c_int), ("inner_sweeps", ctypes.c_int),
                ("check_every", ctypes.c_int), ("engine", ctypes.c_int),
                ("temporal", ctypes.c_int), ("tile_x", ctypes.c_int), ("tile_y", ctypes.c_int),
                ("reserved", ctypes.c_int), ("tol", ctypes.c_double)]


class IrResult(ctypes.Structure):
    _fields_ = [("sweeps", ctypes.c_int), ("outer_steps", ctypes.c_int),
                ("rel_residual", ctypes.c_double), ("engine", ctypes.c_int),
                ("kernel_launches", ctypes.c_int), ("temporal", ctypes.c_int),
                ("tile_x", ctypes.c_int), ("tile_y", ctypes.c_int)]


class SolveResult(ctypes.Structure):
    _fields_ = [("sweeps", ctypes.c_int), ("checks", ctypes.c_int),
                ("rel_residual", ctypes.c_double), ("d_result", ctypes.c_void_p)]


STORAGE_FP32, STORAGE_BF16, STORAGE_FP16 = 0, 1, 2
IR_ENGINE_AUTO, IR_ENGINE_LAUNCHES, IR_ENGINE_PERSISTENT_2D = 0, 1, 2
IR_ENGINE_NAMES = {"auto": IR_ENGINE_AUTO, "launches": IR_ENGINE_LAUNCHES,
                   "persistent2d": IR_ENGINE_PERSISTENT_2D}


class StencilParams(ctypes.Structure):
    _fields_ = [
        ("dims", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("nz", ctypes.c_int), ("radius", ctypes.c_int), ("iterations", ctypes.c_int),
        ("mode", ctypes.c_int), ("variant", ctypes.c_int), ("block_x", ctypes.c_int),
        ("block_y", ctypes.c_int), ("block_z", ctypes.c_int), ("coarsen_x", ctypes.c_int),
        ("temporal", ctypes.c_int), ("reserved", ctypes.c_int * 4),
    ]


_lib = None


def load() -> ctypes.CDLL:
    """Loads the in-tree library (raises if it is absent: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libstencil_gb300.so is not built (run __graft_entry__.build())")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER(StencilParams)
    vp, i, sz, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t, ctypes.c_uint64
    sig = {
        "stencil_params_init": (i, [P]),
        "stencil_params_check": (i, [P]),
        "stencil_dispatch_ex": (i, [P, vp, vp, vp, ctypes.POINTER(vp)]),
        "stencil_run_host": (i, [P, vp, vp, ctypes.POINTER(ctypes.c_float)]),
        "stencil_last_dispatch": (i, [ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_longlong)]),
        "stencil_heuristic_block": (i, [P, i, ctypes.POINTER(i), ctypes.POINTER(i),
                                        ctypes.POINTER(i)]),
        "stencil_heuristic_geometry": (i, [P, ctypes.POINTER(i), ctypes.POINTER(i),
                                           ctypes.POINTER(i), ctypes.POINTER(i)]),
        "stencil_run_host_timed": (i, [P, vp, vp, ctypes.POINTER(ctypes.c_float),
                                       ctypes.POINTER(ctypes.c_float)]),
        "stencil_init_reference": (i, [P, vp, vp]),
        "stencil_init_uniform": (i, [vp, sz, u64, vp]),
        "stencil_copy_border": (i, [P, vp, vp, vp]),
        "stencil_init_fourier": (i, [P, vp, u64, i, vp]),
        "stencil_init_laplace2d": (i, [P, vp, u64, vp]),
        "stencil_residual": (i, [P, vp, ctypes.POINTER(ctypes.c_double), vp]),
        "stencil_residual_noalloc": (i, [P, vp, ctypes.POINTER(ctypes.c_double), vp]),
        "stencil_solve": (i, [P, vp, vp, ctypes.c_double, i, vp, ctypes.POINTER(SolveResult)]),
        "stencil_selftest_div": (i, [i, ctypes.POINTER(ctypes.c_ulonglong),
                                     ctypes.POINTER(ctypes.c_uint)]),
        "stencil_selftest_wait": (i, [i, ctypes.POINTER(i), ctypes.POINTER(i)]),
        "stencil_batch_workspace_bytes": (i, [i, ctypes.POINTER(sz)]),
        "stencil_batch_workspace_bytes_for": (i, [ctypes.POINTER(BatchJob), i, ctypes.POINTER(sz)]),
        "stencil_batch_prepare": (i, [ctypes.POINTER(BatchJob), i, i, vp, sz, vp]),
        "stencil_batch_launch": (i, [vp, vp]),
        "stencil_batch_forget": (i, [vp]),
        "stencil_batch_plan": (i, [vp, ctypes.POINTER(i), ctypes.POINTER(i)]),
        "stencil_batch_side_by_side": (i, [vp, ctypes.POINTER(i), ctypes.POINTER(i)]),
        "stencil_batch_prepare_engine": (i, [ctypes.POINTER(BatchJob), i, i, i, vp, sz, vp]),
        "stencil_batch_launches": (i, [vp, ctypes.POINTER(i)]),
        "stencil_batch_teams": (i, [vp, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i), i]),
        "stencil_ir_workspace_bytes": (i, [P, ctypes.POINTER(IrParams), ctypes.POINTER(sz)]),
        "stencil_ir_solve": (i, [P, ctypes.POINTER(IrParams), vp, vp, sz, vp,
                                 ctypes.POINTER(IrResult)]),
        "stencil_tuning_set": (i, [P, P]),
        "stencil_tuning_get": (i, [P, P]),
        "stencil_tuning_clear": (i, []),
        "stencil_strerror": (ctypes.c_char_p, [i]),
        "stencil_last_error": (ctypes.c_char_p, []),
        "stencil_device_status": (i, [ctypes.POINTER(i)]),
        "stencil_release": (i, []),
        "stencil_version": (i, [ctypes.POINTER(i), ctypes.POINTER(i)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _strerror(status: int) -> str:
    try:
        return load().stencil_strerror(status).decode()
    except Exception:  # pragma: no cover - only when the library itself is missing
        return "status %d" % status


def check(status: int, where: str) -> None:
    if status != OK:
        raise StencilError(status, where, load().stencil_last_error().decode())


def declared_symbols() -> list[str]:
    """Every function include/*.h declares with STENCIL_API / UNET_API."""
    names = []
    for fn in sorted(os.listdir(HEADER_DIR)):
        if not fn.endswith(".h"):
            continue
        text = "\n".join(line for line in open(os.path.join(HEADER_DIR, fn))
                         if not line.lstrip().startswith("#"))
        names += re.findall(r"\b(?:STENCIL_API|UNET_API)\s+[\w\s\*]*?\b(\w+)\s*\(", text)
    return names


def make_params(shape, radius: int, iterations: int, mode: int = MODE_LEGACY,
                variant: int = VARIANT_AUTO, block=(0, 0, 0), coarsen_x: int = 0,
                temporal: int = 0) -> StencilParams:
    """shape is numpy/torch order: (ny, nx) for 2-D, (nz, ny, nx) for 3-D."""
    p = StencilParams()
    check(load().stencil_params_init(ctypes.byref(p)), "stencil_params_init")
    if len(shape) == 2:
        p.dims, p.ny, p.nx, p.nz = 2, shape[0], shape[1], 1
    elif len(shape) == 3:
        p.dims, p.nz, p.ny, p.nx = 3, shape[0], shape[1], shape[2]
    else:
        raise ValueError("grid must be 2-D or 3-D")
    p.radius, p.iterations, p.mode = radius, iterations, mode
    p.variant = VARIANT_NAMES[variant] if isinstance(variant, str) else variant
    p.block_x, p.block_y, p.block_z = block
    p.coarsen_x, p.temporal = coarsen_x, temporal
    return p
