"""Host-side interface of the sweep loop, mirroring the reference's dispatch.

The reference configures one binary per configuration with the compile-time
macros of include/constants.h and runs ``dispatch_kernels(d_u1, d_u2)``
(src/stencil_dispatch.cu:138-158).  ``StencilConfig`` keeps those macro names
as fields, and ``dispatch_kernels`` takes the same two device buffers; both go
straight to the C ABI (``stencil_dispatch_ex``).  Device memory is held in
torch CUDA tensors (plumbing only: every sweep runs in libstencil_gb300.so).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import lib as _lib


@dataclass
class StencilConfig:
    """Runtime form of include/constants.h (same names and defaults)."""
    DIMENSIONS: int = 3
    DIM: int = 256
    RADIUS: int = 1
    ITERATIONS: int = 64
    BLOCK_X: int = 32
    BLOCK_Y: int = 2
    BLOCK_Z: int = 2
    COARSEN_X: int = 4
    SMEM: bool = False
    PADDED: bool = False
    REGISTER: bool = False
    COOP: bool = False
    HEURISTIC: bool = False
    STENCIL_MODE: int = _lib.MODE_LEGACY
    TEMPORAL_T: int = 0

    @property
    def shape(self):
        return (self.DIM,) * self.DIMENSIONS

    def variant(self) -> int:
        """Variant selection of get_kernel() (src/stencil_dispatch.cu:14-42)."""
        if self.COOP:
            return _lib.VARIANT_COOP
        if self.SMEM and self.REGISTER:
            return _lib.VARIANT_SMEM_REGISTER
        if self.SMEM and self.PADDED:
            return _lib.VARIANT_SMEM_PADDED
        if self.SMEM:
            return _lib.VARIANT_SMEM
        return _lib.VARIANT_BASE

    def params(self) -> _lib.StencilParams:
        """HEURISTIC: False = the BLOCK_* shape; True (1) = the library's
        choice; 2 = the reference's occupancy-based shape
        (stencil_heuristic_geometry)."""
        block = (0, 0, 0) if self.HEURISTIC else (self.BLOCK_X, self.BLOCK_Y, self.BLOCK_Z)
        p = _lib.make_params(self.shape, self.RADIUS, self.ITERATIONS, self.STENCIL_MODE,
                             self.variant(), block, self.COARSEN_X, self.TEMPORAL_T)
        if self.HEURISTIC == 2 and not self.COOP:
            p.block_x = self.BLOCK_X
            t, bx, by, bz = heuristic_geometry(p)
            # the 3-D stream kernel (SMEM_REGISTER) takes x and y as its tile
            if p.variant == _lib.VARIANT_SMEM_REGISTER and p.dims == 3:
                bz = 0
            p.block_x, p.block_y, p.block_z = bx, by, bz
        return p


def heuristic_geometry(params: _lib.StencilParams):
    """(threads, bx, by, bz) of the reference's HEURISTIC selection for these
    parameters (stencil_heuristic_geometry)."""
    t, bx, by, bz = (ctypes.c_int() for _ in range(4))
    _lib.check(_lib.load().stencil_heuristic_geometry(ctypes.byref(params), ctypes.byref(t),
                                                      ctypes.byref(bx), ctypes.byref(by),
                                                      ctypes.byref(bz)),
               "stencil_heuristic_geometry")
    return t.value, bx.value, by.value, bz.value


def _stream_handle(stream):
    import torch
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _check_tensor(t, shape=None):
    import torch
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError("device buffers must be CUDA tensors")
    if t.dtype != torch.float32 or not t.is_contiguous():
        raise TypeError("device buffers must be contiguous float32")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError("buffer shape %s does not match %s" % (tuple(t.shape), tuple(shape)))


def dispatch(params: _lib.StencilParams, d_u1, d_u2, stream=None):
    """Runs params.iterations sweeps; returns whichever of d_u1 / d_u2 holds the result."""
    _check_tensor(d_u1)
    _check_tensor(d_u2, d_u1.shape)
    res = ctypes.c_void_p()
    _lib.check(_lib.load().stencil_dispatch_ex(ctypes.byref(params), ctypes.c_void_p(d_u1.data_ptr()),
                                               ctypes.c_void_p(d_u2.data_ptr()),
                                               _stream_handle(stream), ctypes.byref(res)),
               "stencil_dispatch_ex")
    return d_u1 if res.value == d_u1.data_ptr() else d_u2


def dispatch_kernels(d_u1, d_u2, cfg: StencilConfig | None = None, stream=None):
    """Same role as the reference's dispatch_kernels(d_u1, d_u2); returns the result buffer."""
    cfg = cfg or StencilConfig()
    return dispatch(cfg.params(), d_u1, d_u2, stream)


def sweep(d_u1, d_u2, radius: int, iterations: int, mode: int = _lib.MODE_JACOBI,
          variant="auto", block=(0, 0, 0), coarsen_x: int = 0, temporal: int = 0, stream=None):
    p = _lib.make_params(tuple(d_u1.shape), radius, iterations, mode, variant, block,
                         coarsen_x, temporal)
    return dispatch(p, d_u1, d_u2, stream)


def init_reference(shape, device="cuda", stream=None):
    import torch
    u = torch.empty(shape, dtype=torch.float32, device=device)
    p = _lib.make_params(shape, 1, 0)
    _lib.check(_lib.load().stencil_init_reference(ctypes.byref(p), ctypes.c_void_p(u.data_ptr()),
                                                  _stream_handle(stream)), "stencil_init_reference")
    return u


def init_uniform(shape, seed: int, device="cuda", stream=None):
    import torch
    u = torch.empty(shape, dtype=torch.float32, device=device)
    _lib.check(_lib.load().stencil_init_uniform(ctypes.c_void_p(u.data_ptr()), u.numel(),
                                                seed, _stream_handle(stream)),
               "stencil_init_uniform")
    return u


def init_fourier(shape, seed: int, radius: int, modes: int = 8, device="cuda", stream=None):
    """Smooth Fourier-mode border band + uniform [0,1) interior (stencil_init_fourier)."""
    import torch
    u = torch.empty(shape, dtype=torch.float32, device=device)
    p = _lib.make_params(shape, radius, 0)
    _lib.check(_lib.load().stencil_init_fourier(ctypes.byref(p), ctypes.c_void_p(u.data_ptr()),
                                                seed, modes, _stream_handle(stream)),
               "stencil_init_fourier")
    return u


def init_laplace2d(shape, seed: int, device="cuda", stream=None):
    """2-D Laplace Dirichlet border (continuous, Fourier modes per edge), zero interior."""
    import torch
    u = torch.empty(shape, dtype=torch.float32, device=device)
    p = _lib.make_params(shape, 1, 0)
    _lib.check(_lib.load().stencil_init_laplace2d(ctypes.byref(p), ctypes.c_void_p(u.data_ptr()),
                                                  seed, _stream_handle(stream)),
               "stencil_init_laplace2d")
    return u


def copy_border(src, dst, radius: int, stream=None):
    _check_tensor(src)
    _check_tensor(dst, src.shape)
    p = _lib.make_params(tuple(src.shape), radius, 0)
    _lib.check(_lib.load().stencil_copy_border(ctypes.byref(p), ctypes.c_void_p(src.data_ptr()),
                                               ctypes.c_void_p(dst.data_ptr()),
                                               _stream_handle(stream)), "stencil_copy_border")


def residual(u, radius: int, stream=None) -> float:
    _check_tensor(u)
    p = _lib.make_params(tuple(u.shape), radius, 0)
    out = ctypes.c_double()
    _lib.check(_lib.load().stencil_residual(ctypes.byref(p), ctypes.c_void_p(u.data_ptr()),
                                            ctypes.byref(out), _stream_handle(stream)),
               "stencil_residual")
    return out.value


def solve(d_u1, d_u2, radius: int, max_sweeps: int, tol: float, check_every: int = 500,
          variant="auto", stream=None):
    """Plain JACOBI sweeps from d_u1 to relative residual tol, checked every
    check_every sweeps (stencil_solve).  Returns (sweeps, rel_residual,
    buffer holding the result)."""
    _check_tensor(d_u1)
    _check_tensor(d_u2, d_u1.shape)
    p = _lib.make_params(tuple(d_u1.shape), radius, max_sweeps, _lib.MODE_JACOBI, variant)
    r = _lib.SolveResult()
    _lib.check(_lib.load().stencil_solve(ctypes.byref(p), ctypes.c_void_p(d_u1.data_ptr()),
                                         ctypes.c_void_p(d_u2.data_ptr()), tol, check_every,
                                         _stream_handle(stream), ctypes.byref(r)), "stencil_solve")
    return r.sweeps, r.rel_residual, (d_u1 if r.d_result == d_u1.data_ptr() else d_u2)


def run_host(h_in: np.ndarray, radius: int, iterations: int, mode: int = _lib.MODE_JACOBI,
             variant="auto", block=(0, 0, 0), coarsen_x: int = 0, temporal: int = 0,
             out: np.ndarray | None = None, sweeps_ms: bool = False):
    """End to end from host memory (stencil_run_host_timed); returns (result,
    ms) with ms the upload + sweeps + download time, or (result, ms, ms_sweeps)
    when sweeps_ms is set (ms_sweeps = the sweeps alone, the figure the
    reference's binary prints)."""
    h_in = np.ascontiguousarray(h_in, dtype=np.float32)
    if out is None:
        out = np.empty_like(h_in)
    p = _lib.make_params(h_in.shape, radius, iterations, mode, variant, block, coarsen_x,
                         temporal)
    ms, ms_sw = ctypes.c_float(), ctypes.c_float()
    _lib.check(_lib.load().stencil_run_host_timed(ctypes.byref(p), ctypes.c_void_p(h_in.ctypes.data),
                                                  ctypes.c_void_p(out.ctypes.data), ctypes.byref(ms),
                                                  ctypes.byref(ms_sw)),
               "stencil_run_host_timed")
    return (out, ms.value, ms_sw.value) if sweeps_ms else (out, ms.value)


def last_dispatch():
    """(engine, kernel launches) of this thread's last dispatch."""
    eng, n = ctypes.c_char_p(), ctypes.c_longlong()
    _lib.check(_lib.load().stencil_last_dispatch(ctypes.byref(eng), ctypes.byref(n)),
               "stencil_last_dispatch")
    return (eng.value or b"").decode(), n.value


def device_status() -> int:
    st = ctypes.c_int()
    _lib.check(_lib.load().stencil_device_status(ctypes.byref(st)), "stencil_device_status")
    return st.value


class Batch:
    """Many grids of uneven sizes and sweep counts in persistent launches
    (stencil_batch_prepare_engine / stencil_batch_launch).

    engine: "one_launch" (every job in ONE cooperative launch, teams of CTAs
    taking grids from device queues), "phased" (a cluster launch, then
    whole-GPU launches and lanes) or "auto" (the library's choice).

    jobs: list of (d_u1, d_u2, radius, iterations, mode[, hints]) with CUDA
    float32 tensors of shape (ny, nx) or (nz, ny, nx); hints (optional dict)
    sets the job's tuning fields "temporal" and "tile" (tile_x, tile_y; the
    phased engine's) and "team" (the one-launch engine's CTAs for the grid).
    hints_for(shape) -> dict, when given, supplies hints for jobs without
    their own (e.g. autotune.batch_hints of a tuning database).  After
    ``launch`` each job's result is in d_u1 for an even sweep count, else in
    d_u2 (``result(i)``).
    """

    ENGINES = {"auto": 0, "phased": 1, "one_launch": 2}

    def __init__(self, jobs, cluster_size: int = 0, stream=None, hints_for=None, engine: str = "auto"):
        import torch
        self.jobs = [tuple(j[:5]) for j in jobs]
        hints = [j[5] if len(j) > 5 else None for j in jobs]
        arr = (_lib.BatchJob * max(1, len(self.jobs)))()
        for k, (u1, u2, radius, iters, mode) in enumerate(self.jobs):
            h = hints[k] if hints[k] is not None else (hints_for(tuple(u1.shape)) if hints_for else None)
            if h:
                arr[k].temporal = int(h.get("temporal", 0))
                arr[k].tile_x, arr[k].tile_y = (int(v) for v in h.get("tile", (0, 0)))
                arr[k].team = int(h.get("team", 0))
            _check_tensor(u1)
            _check_tensor(u2, u1.shape)
            j = arr[k]
            j.d_u1, j.d_u2 = u1.data_ptr(), u2.data_ptr()
            if u1.dim() == 2:
                j.dims, j.ny, j.nx, j.nz = 2, u1.shape[0], u1.shape[1], 1
            else:
                j.dims, j.nz, j.ny, j.nx = 3, u1.shape[0], u1.shape[1], u1.shape[2]
            j.radius, j.iterations, j.mode = radius, iters, mode
        L = _lib.load()
        nbytes = ctypes.c_size_t()
        _lib.check(L.stencil_batch_workspace_bytes_for(arr, len(self.jobs), ctypes.byref(nbytes)),
                   "stencil_batch_workspace_bytes_for")
        dev = self.jobs[0][0].device if self.jobs else torch.device("cuda")
        self.workspace = torch.empty(nbytes.value + 256, dtype=torch.uint8, device=dev)
        base = self.workspace.data_ptr()
        self.ws = ctypes.c_void_p((base + 255) & ~255)
        _lib.check(L.stencil_batch_prepare_engine(arr, len(self.jobs), self.ENGINES[engine], cluster_size,
                                                  self.ws, nbytes.value, _stream_handle(stream)),
                   "stencil_batch_prepare_engine")

    def launch(self, stream=None):
        _lib.check(_lib.load().stencil_batch_launch(self.ws, _stream_handle(stream)),
                   "stencil_batch_launch")

    def plan(self):
        """(jobs in the cluster launch, jobs with a whole-GPU launch of their own)."""
        c, w = ctypes.c_int(), ctypes.c_int()
        _lib.check(_lib.load().stencil_batch_plan(self.ws, ctypes.byref(c), ctypes.byref(w)),
                   "stencil_batch_plan")
        return c.value, w.value

    def side_by_side(self):
        """(sets of lanes that run side by side, each lane a queue of jobs on
        a share of the GPU; jobs in them)."""
        g, n = ctypes.c_int(), ctypes.c_int()
        _lib.check(_lib.load().stencil_batch_side_by_side(self.ws, ctypes.byref(g), ctypes.byref(n)),
                   "stencil_batch_side_by_side")
        return g.value, n.value

    def kernel_launches(self):
        """Kernel launches of one ``launch`` (one replay of its CUDA graph):
        1 for the one-launch engine; for the phased one the cluster launch,
        one per whole-GPU job, and the two copy kernels of jobs whose nx is
        not a multiple of 4."""
        n = ctypes.c_int()
        _lib.check(_lib.load().stencil_batch_launches(self.ws, ctypes.byref(n)), "stencil_batch_launches")
        return n.value

    def teams(self):
        """The one-launch engine's tiers as [(nominal team size, jobs)], largest
        teams first ([] for the phased engine)."""
        n = ctypes.c_int()
        sizes, counts = (ctypes.c_int * 16)(), (ctypes.c_int * 16)()
        _lib.check(_lib.load().stencil_batch_teams(self.ws, ctypes.byref(n), sizes, counts, 16),
                   "stencil_batch_teams")
        return [(sizes[t], counts[t]) for t in range(min(n.value, 16))]

    def result(self, k):
        u1, u2, _, iters, _ = self.jobs[k]
        return u1 if iters % 2 == 0 else u2

    def close(self):
        if self.ws is not None:
            _lib.load().stencil_batch_forget(self.ws)
            self.ws = None


def ir_workspace(shape, radius: int, storage: str = "bf16", device="cuda"):
    """A device workspace for ir_solve on grids of this shape (reusable)."""
    import torch
    p = _lib.make_params(tuple(shape), radius, 0, _lib.MODE_JACOBI)
    ir = _lib.IrParams()
    ir.storage = {"bf16": _lib.STORAGE_BF16, "fp16": _lib.STORAGE_FP16}[storage]
    nbytes = ctypes.c_size_t()
    _lib.check(_lib.load().stencil_ir_workspace_bytes(ctypes.byref(p), ctypes.byref(ir),
                                                      ctypes.byref(nbytes)),
               "stencil_ir_workspace_bytes")
    return torch.empty(nbytes.value + 256, dtype=torch.uint8, device=device)


def ir_solve_ex(d_u, radius: int, iterations: int, storage: str = "bf16", inner_sweeps: int = 0,
                tol: float = 0.0, check_every: int = 1, engine="auto", temporal: int = 0,
                tile=(0, 0), workspace=None, stream=None) -> dict:
    """Mixed-precision iterative refinement in place on the FP32 master d_u
    (stencil_ir_solve).  Returns the stencil_ir_result fields as a dict."""
    import torch
    _check_tensor(d_u)
    p = _lib.make_params(tuple(d_u.shape), radius, iterations, _lib.MODE_JACOBI)
    ir = _lib.IrParams()
    ir.storage = {"bf16": _lib.STORAGE_BF16, "fp16": _lib.STORAGE_FP16}[storage]
    ir.inner_sweeps, ir.check_every, ir.tol = inner_sweeps, check_every, tol
    ir.engine = _lib.IR_ENGINE_NAMES[engine] if isinstance(engine, str) else engine
    ir.temporal, ir.tile_x, ir.tile_y = temporal, tile[0], tile[1]
    L = _lib.load()
    nbytes = ctypes.c_size_t()
    _lib.check(L.stencil_ir_workspace_bytes(ctypes.byref(p), ctypes.byref(ir), ctypes.byref(nbytes)),
               "stencil_ir_workspace_bytes")
    if workspace is None or workspace.numel() < nbytes.value + 256:
        workspace = torch.empty(nbytes.value + 256, dtype=torch.uint8, device=d_u.device)
    ws = (workspace.data_ptr() + 255) & ~255
    res = _lib.IrResult()
    _lib.check(L.stencil_ir_solve(ctypes.byref(p), ctypes.byref(ir), ctypes.c_void_p(d_u.data_ptr()),
                                  ctypes.c_void_p(ws), nbytes.value, _stream_handle(stream),
                                  ctypes.byref(res)), "stencil_ir_solve")
    names = {_lib.IR_ENGINE_LAUNCHES: "launches", _lib.IR_ENGINE_PERSISTENT_2D: "persistent2d"}
    return {"sweeps": res.sweeps, "outer_steps": res.outer_steps,
            "rel_residual": res.rel_residual, "engine": names.get(res.engine, str(res.engine)),
            "kernel_launches": res.kernel_launches, "temporal": res.temporal,
            "tile": (res.tile_x, res.tile_y)}


def ir_solve(d_u, radius: int, iterations: int, storage: str = "bf16", inner_sweeps: int = 0,
             tol: float = 0.0, check_every: int = 1, workspace=None, stream=None, engine="auto"):
    """Mixed-precision iterative refinement in place on the FP32 master d_u
    (stencil_ir_solve).  Returns (sweeps, outer_steps, rel_residual)."""
    r = ir_solve_ex(d_u, radius, iterations, storage, inner_sweeps, tol, check_every, engine,
                    workspace=workspace, stream=stream)
    return r["sweeps"], r["outer_steps"], r["rel_residual"]
