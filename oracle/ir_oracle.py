"""CPU restatement of the mixed-precision iterative refinement (TEST
INFRASTRUCTURE ONLY: the checker of stencil_ir_solve on 2-D grids).

Only tests/ import this module.  It restates, in numpy FP32 arithmetic with
the 16-bit roundings emulated bit for bit, the outer step that the library's
two engines implement (thesis_gb300/csrc/k_ir.cu k_ir_resid / k_lp_sweep /
k_ir_update, and the persistent form thesis_gb300/csrc/k_ir2d.cu):

  r   = (sum of the 2DR axis neighbours of u, from +0, axis i offsets
         -R..-1, +1..+R, then axis j) / (2DR) - u          (FP32, IEEE)
  s   = 2^ex with max|r| = f 2^ex, f in [0.5, 1)  (max over the update region)
  rhs = E(r * (1/s))                                      (E = BF16 or FP16)
  e_1 = rhs;  e_{k+1} = E(sum(e_k) / (2DR) + rhs), the sum started from its
        first term, same axis and offset order
  u  += s * e_m                                           (one rounding)

The refinement extends the reference's plain sweep (src/stencil_cpu.cu:32-35
with the per-cell update of src/stencils.cu:8-19); it has no counterpart in
the reference, so this restatement is pinned by the library's own
definition, and checked here against the plain FP32 loop of the C oracle
(same sweep count, agreement to the 16-bit storage precision).
"""
from __future__ import annotations

import numpy as np

F32 = np.float32


def round_bf16(x: np.ndarray) -> np.ndarray:
    """FP32 -> BF16 -> FP32, round to nearest even (finite inputs)."""
    b = np.ascontiguousarray(x, F32).view(np.uint32)
    r = (b + np.uint32(0x7FFF) + ((b >> np.uint32(16)) & np.uint32(1))) & np.uint32(0xFFFF0000)
    return r.view(F32)


def round_fp16(x: np.ndarray) -> np.ndarray:
    """FP32 -> FP16 -> FP32, round to nearest even (IEEE binary16)."""
    return np.asarray(x, F32).astype(np.float16).astype(F32)


ROUND = {"bf16": round_bf16, "fp16": round_fp16}


def _shift(a: np.ndarray, R: int, axis: int, o: int) -> np.ndarray:
    """Neighbours at offset o along axis (x = -1, y = -2) of every update-region cell."""
    ny, nx = a.shape
    if axis == -1:
        return a[R:ny - R, R + o:nx - R + o]
    return a[R + o:ny - R + o, R:nx - R]


def _offsets(R):
    return [o for o in range(-R, R + 1) if o]


def residual_scaled(u: np.ndarray, R: int, storage: str):
    """(rhs grid in E, scale s): the first two lines of the outer step."""
    C = F32(4 * R)
    acc = np.zeros((u.shape[0] - 2 * R, u.shape[1] - 2 * R), F32)
    for axis in (-1, -2):
        for o in _offsets(R):
            acc = acc + _shift(u, R, axis, o)
    r = acc / C - _shift(u, R, -1, 0)
    mx = F32(np.abs(r).max()) if r.size else F32(0)
    ex = int(np.frexp(mx)[1]) if mx > 0 else 0
    s = F32(np.ldexp(F32(1), ex))
    inv = F32(1) / s
    rhs = np.zeros_like(u)
    rhs[R:-R, R:-R] = ROUND[storage](r * inv)
    return rhs, s


def correction_sweep(e: np.ndarray, rhs: np.ndarray, R: int, storage: str) -> np.ndarray:
    C = F32(4 * R)
    terms = [(axis, o) for axis in (-1, -2) for o in _offsets(R)]
    acc = _shift(e, R, *terms[0]).copy()
    for axis, o in terms[1:]:
        acc = acc + _shift(e, R, axis, o)
    out = np.zeros_like(e)
    out[R:-R, R:-R] = ROUND[storage](acc / C + rhs[R:-R, R:-R])
    return out


def outer_step(u: np.ndarray, R: int, m: int, storage: str) -> np.ndarray:
    """u after one outer step of m correction sweeps (a new array)."""
    rhs, s = residual_scaled(u, R, storage)
    e = rhs.copy()
    for _ in range(m - 1):
        e = correction_sweep(e, rhs, R, storage)
    out = u.copy()
    out[R:-R, R:-R] = (s * e[R:-R, R:-R]).astype(F32) + u[R:-R, R:-R]
    return out


def ir_solve(u: np.ndarray, R: int, iterations: int, inner: int, storage: str):
    """FP32 master grid after `iterations` sweeps in outer steps of `inner`
    (the last one shorter): returns (u, outer steps)."""
    u = np.ascontiguousarray(u, F32).copy()
    assert u.ndim == 2 and min(u.shape) > 2 * R
    done = outer = 0
    while done < iterations:
        m = min(inner, iterations - done)
        u = outer_step(u, R, m, storage)
        done += m
        outer += 1
    return u, outer
