"""Runs the reference's own GPU kernels (TEST INFRASTRUCTURE ONLY).

The cubins come from oracle/build.py's ``build_ref_gpu`` (the reference's
src/stencil_kernel_{base,smem,smem_padded,smem_register}.cu compiled
unchanged for sm_103a, one cubin per compile-time configuration).  This
module loads them with the CUDA driver API and launches them with the
reference's dispatch geometry, restated from src/stencil_dispatch.cu:
  * kernel by variant and COARSEN_X (get_kernel, :14-42);
  * block (BLOCK_X, BLOCK_Y, BLOCK_Z); grid ((1 + (NX-1)/bx) / COARSEN_X,
    1 + (NY-1)/by, 1 + (NZ-1)/bz) (:147-150);
  * dynamic shared memory by set_smem (:46-66);
  * arguments (d_u1, d_u2, 0, NZ-1), pointers swapped after every sweep
    (:151-156).
Only tests use it: to show that the reference kernels reproduce the oracle and
the golden fixtures on this GPU, and to time them beside this library's.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

VARIANTS = ("base", "smem", "smem_padded", "smem_register")


def kernel_name(variant: str, dims: int, coarsen_x: int) -> str:
    """Itanium-ABI name of void <name>(float*, float*, unsigned, unsigned)."""
    base = variant + ("_unroll" if coarsen_x > 1 else "") + "_%dd" % dims
    return "_Z%d%sPfS_jj" % (len(base), base)


def smem_bytes(variant: str, dims: int, radius: int, bx: int, by: int, bz: int, cf: int) -> int:
    """set_smem (src/stencil_dispatch.cu:46-66)."""
    if variant == "base":
        return 0
    sx = bx * cf
    px, py, pz = sx + 2 * radius, by + 2 * radius, bz + 2 * radius
    if dims == 3:
        if variant == "smem_padded":
            return px * py * pz * 4
        if variant == "smem_register":
            return px * py * bz * 4
        return sx * by * bz * 4
    if variant == "smem_padded":
        return px * py * 4
    if variant == "smem_register":
        return px * by * 4
    return sx * by * 4


def valid(variant: str, dims: int, radius: int, bx: int, by: int, bz: int) -> bool:
    """The reference's own launch check (check_early_exit,
    include/stencil_utils.h:113-124): shapes it refuses are not run."""
    if variant == "smem_padded":
        return bx >= radius and by >= radius and (dims != 3 or bz >= radius)
    if variant == "smem_register":
        return bx >= radius and (dims != 3 or by >= radius)
    return True


class RefKernels:
    """One cubin (one compile-time configuration) loaded into the current
    CUDA context (the one torch uses)."""

    def __init__(self, cfg):
        self.cfg = tuple(cfg)
        self.dims, self.dim, self.radius, self.bx, self.by, self.bz, self.cf = self.cfg
        path = _build.ref_cubin(self.cfg)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0), "cuInit")
        ctx = ctypes.c_void_p()
        self._check(self.cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context (initialise torch.cuda first)")
        self.mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(self.mod), path.encode()), "cuModuleLoad")
        self.fns = {}

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError("%s failed with CUresult %d" % (what, rc))

    def function(self, variant):
        if variant not in self.fns:
            if not valid(variant, self.dims, self.radius, self.bx, self.by, self.bz):
                raise ValueError("the reference refuses %s with block %dx%dx%d at R=%d"
                                 % (variant, self.bx, self.by, self.bz, self.radius))
            fn = ctypes.c_void_p()
            name = kernel_name(variant, self.dims, self.cf).encode()
            self._check(self.cu.cuModuleGetFunction(ctypes.byref(fn), self.mod, name),
                        "cuModuleGetFunction(%s)" % name.decode())
            smem = smem_bytes(variant, self.dims, self.radius, self.bx, self.by, self.bz, self.cf)
            if smem > 48 * 1024:
                # CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES = 8
                self._check(self.cu.cuFuncSetAttribute(fn, 8, smem), "cuFuncSetAttribute")
            self.fns[variant] = (fn, smem)
        return self.fns[variant]

    def heuristic_geometry(self, variant, heuristic_block):
        """The reference's HEURISTIC geometry for this cubin's kernel
        (src/stencil_dispatch.cu:138-146): cuOccupancyMaxPotentialBlockSize
        -- the driver form of the runtime call the reference makes at :143 --
        with calculate_smem (:103-112: set_smem of the block that
        set_max_occupancy_block_dimensions, :89-101, shapes from the thread
        count) as the shared-memory function; heuristic_block(threads) is that
        shaping rule.  Returns (threads, bx, by, bz)."""
        fn = ctypes.c_void_p()
        name = kernel_name(variant, self.dims, self.cf).encode()
        self._check(self.cu.cuModuleGetFunction(ctypes.byref(fn), self.mod, name), "cuModuleGetFunction")
        # CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES = 8, as large as the device allows
        self.cu.cuFuncSetAttribute(fn, 8, 200 * 1024)

        def smem_of(threads):
            bx, by, bz = heuristic_block(threads)
            return smem_bytes(variant, self.dims, self.radius, bx, by, bz, self.cf)

        CB = ctypes.CFUNCTYPE(ctypes.c_size_t, ctypes.c_int)
        cb = CB(smem_of)
        min_grid, block = ctypes.c_int(), ctypes.c_int()
        self.cu.cuOccupancyMaxPotentialBlockSize.argtypes = [
            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.c_void_p, CB,
            ctypes.c_size_t, ctypes.c_int]
        self._check(self.cu.cuOccupancyMaxPotentialBlockSize(ctypes.byref(min_grid), ctypes.byref(block),
                                                             fn, cb, 0, 0),
                    "cuOccupancyMaxPotentialBlockSize")
        t = block.value
        return (t,) + tuple(heuristic_block(t))

    def grid(self):
        n = self.dim
        gx = (1 + (n - 1) // self.bx) // self.cf
        gy = 1 + (n - 1) // self.by if self.dims > 1 else 1
        gz = 1 + (n - 1) // self.bz if self.dims > 2 else 1
        return gx, gy, gz

    def sweeps(self, variant, d_u1: int, d_u2: int, iterations: int, stream: int = 0):
        """`iterations` launches with the reference's pointer swap; returns the
        device pointer holding the last sweep's result."""
        fn, smem = self.function(variant)
        gx, gy, gz = self.grid()
        kstart, kend = ctypes.c_uint(0), ctypes.c_uint(self.dim - 1)
        a, b = ctypes.c_void_p(d_u1), ctypes.c_void_p(d_u2)
        for _ in range(iterations):
            args = (ctypes.c_void_p * 4)(ctypes.cast(ctypes.pointer(a), ctypes.c_void_p),
                                         ctypes.cast(ctypes.pointer(b), ctypes.c_void_p),
                                         ctypes.cast(ctypes.pointer(kstart), ctypes.c_void_p),
                                         ctypes.cast(ctypes.pointer(kend), ctypes.c_void_p))
            self._check(self.cu.cuLaunchKernel(fn, gx, gy, gz, self.bx, self.by, self.bz, smem,
                                               ctypes.c_void_p(stream), args, None),
                        "cuLaunchKernel")
            a, b = b, a
        return a.value

    def close(self):
        if self.mod:
            self.cu.cuModuleUnload(self.mod)
            self.mod = None


def available(cfg) -> bool:
    return os.path.exists(_build.ref_cubin(cfg))
