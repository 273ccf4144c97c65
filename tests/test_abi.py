"""CPU tests of the C ABI: the library builds, loads, exports every declared
symbol, and validates parameters without touching a device."""
import ctypes
import os
import subprocess
import tempfile

import pytest

from thesis_gb300 import lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_every_declared_symbol_is_exported(stencil_lib):
    names = L.declared_symbols()
    assert "stencil_dispatch_ex" in names and "stencil_run_host" in names
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert getattr(stencil_lib, n) is not None


def test_version(stencil_lib):
    abi, sm = ctypes.c_int(), ctypes.c_int()
    assert stencil_lib.stencil_version(ctypes.byref(abi), ctypes.byref(sm)) == 0
    assert abi.value == 1 and sm.value == 103


def test_params_defaults_match_reference_constants(stencil_lib):
    p = L.StencilParams()
    assert stencil_lib.stencil_params_init(ctypes.byref(p)) == 0
    # include/constants.h defaults of the reference: 3-D, DIM 256, R 1, 64 sweeps
    assert (p.dims, p.nx, p.ny, p.nz, p.radius, p.iterations) == (3, 256, 256, 256, 1, 64)
    assert p.mode == L.MODE_LEGACY and p.variant == L.VARIANT_AUTO


@pytest.mark.parametrize("field,value", [
    ("dims", 1), ("dims", 4), ("radius", 0), ("nx", 2), ("iterations", -1), ("mode", 7),
    ("variant", 99), ("block_x", -1), ("coarsen_x", -2),
])
def test_params_check_rejects(stencil_lib, field, value):
    p = L.make_params((16, 16, 16), 1, 4)
    setattr(p, field, value)
    assert stencil_lib.stencil_params_check(ctypes.byref(p)) == L.EINVAL
    assert stencil_lib.stencil_last_error().decode()


def test_params_check_rejects_oversized_block_and_reserved(stencil_lib):
    p = L.make_params((16, 16, 16), 1, 4, block=(64, 32, 1))
    assert stencil_lib.stencil_params_check(ctypes.byref(p)) == L.EINVAL
    p = L.make_params((16, 16, 16), 1, 4)
    p.reserved[2] = 1
    assert stencil_lib.stencil_params_check(ctypes.byref(p)) == L.EINVAL
    p = L.make_params((9, 9, 9), 4, 4)  # 2R+1 = 9: smallest legal extent
    assert stencil_lib.stencil_params_check(ctypes.byref(p)) == 0
    p = L.make_params((8, 9, 9), 4, 4)
    assert stencil_lib.stencil_params_check(ctypes.byref(p)) == L.EINVAL


def test_dispatch_rejects_bad_pointers_without_device(stencil_lib):
    p = L.make_params((16, 16), 1, 4)
    res = ctypes.c_void_p()
    assert stencil_lib.stencil_dispatch_ex(ctypes.byref(p), None, None, None,
                                           ctypes.byref(res)) == L.EINVAL
    assert stencil_lib.stencil_dispatch_ex(ctypes.byref(p), ctypes.c_void_p(4096),
                                           ctypes.c_void_p(4096), None, None) == L.EINVAL
    assert stencil_lib.stencil_dispatch_ex(ctypes.byref(p), ctypes.c_void_p(4100),
                                           ctypes.c_void_p(8192), None, None) == L.EINVAL


def test_strerror(stencil_lib):
    for code in (L.OK, L.EINVAL, L.ENOMEM, L.ECUDA, L.ETIMEOUT, L.EUNSUPPORTED, L.ENODEVICE):
        assert stencil_lib.stencil_strerror(code)
    assert b"unknown" in stencil_lib.stencil_strerror(12345)


DROPIN = r"""
#include <stdio.h>
#include "constants.h"
#include "stencil_dispatch.h"
int main(void) {
    stencil_params p;
    if (stencil_params_from_constants(&p)) return 1;
    printf("%d %d %d %d %d %d %d %d %d %d %d\n", p.dims, p.nx, p.ny, p.nz, p.radius,
           p.iterations, p.mode, p.variant, p.block_x, p.coarsen_x, stencil_params_check(&p));
    return 0;
}
"""


@pytest.mark.parametrize("flags,expect", [
    ([], "3 256 256 256 1 64 0 1 32 4 0"),
    (["-DDIMENSIONS=2", "-DDIM=512", "-DRADIUS=4", "-DITERATIONS=8", "-DSMEM=true",
      "-DPADDED=true"], "2 512 512 1 4 8 0 3 32 4 0"),
    (["-DDIM=128", "-DSMEM=true", "-DREGISTER=true", "-DCOARSEN_X=8"],
     "3 128 128 128 1 64 0 4 32 8 0"),
    (["-DCOOP=true", "-DSTENCIL_MODE=STENCIL_MODE_JACOBI", "-DHEURISTIC=true"],
     "3 256 256 256 1 64 1 5 0 4 0"),
])
def test_constants_h_dropin(stencil_lib, flags, expect):
    """A C caller configured with the reference's -D macros gets the same configuration."""
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "m.c")
        exe = os.path.join(tmp, "m")
        open(src, "w").write(DROPIN)
        subprocess.run(["gcc", "-std=c99", "-o", exe, src, "-I", os.path.join(ROOT, "include"),
                        L.LIB_PATH, "-Wl,-rpath," + os.path.dirname(L.LIB_PATH)] + flags,
                       check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.strip()
    assert out == expect


def test_ngpus_must_be_one():
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "m.c")
        open(src, "w").write('#include "constants.h"\nint main(void){return 0;}\n')
        r = subprocess.run(["gcc", "-DNGPUS=2", "-I", os.path.join(ROOT, "include"), "-c", src,
                            "-o", os.path.join(tmp, "m.o")], capture_output=True, text=True)
        assert r.returncode != 0 and "NGPUS" in r.stderr


@pytest.mark.parametrize("dims,variant,radius,block_x,threads,want", [
    # 3-D: b0 = BLOCK_X, b1 = min(max(2, R), 8), b2 = threads / (b0 * b1), sorted descending
    (3, "base", 1, 32, 1024, (32, 16, 2)),
    (3, "base", 4, 32, 1024, (32, 8, 4)),
    (3, "smem", 16, 32, 512, (32, 8, 2)),
    (3, "base", 2, 8, 256, (16, 8, 2)),
    # padded smem halves b0 while threads / (b0 * R * R) == 0
    (3, "smem_padded", 8, 32, 1024, (16, 8, 8)),
    (3, "smem_padded", 16, 64, 1024, (32, 8, 4)),
    # 2-D: (BLOCK_X, threads / BLOCK_X, 1)
    (2, "base", 1, 32, 1024, (32, 32, 1)),
    (2, "smem_padded", 4, 64, 768, (64, 12, 1)),
])
def test_reference_heuristic_block(stencil_lib, dims, variant, radius, block_x, threads, want):
    """stencil_heuristic_block restates src/stencil_dispatch.cu:89-101."""
    from thesis_gb300 import lib
    p = lib.make_params((64,) * dims, radius, 1, lib.MODE_JACOBI, variant, (block_x, 0, 0))
    bx, by, bz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    assert stencil_lib.stencil_heuristic_block(ctypes.byref(p), threads, ctypes.byref(bx),
                                               ctypes.byref(by), ctypes.byref(bz)) == 0
    assert (bx.value, by.value, bz.value) == want
    assert stencil_lib.stencil_heuristic_block(ctypes.byref(p), 0, ctypes.byref(bx),
                                               ctypes.byref(by), ctypes.byref(bz)) != 0


def test_batch_engine_choice_is_validated_without_device(stencil_lib):
    """An unknown batch engine is refused before anything reaches a device,
    and the workspace size covers either engine (job table, tensor maps,
    team counters, pitched copies)."""
    ws = ctypes.c_void_p(4096)
    for engine in (-1, 3):
        rc = stencil_lib.stencil_batch_prepare_engine(None, 0, engine, 0, ws, 1 << 20, None)
        assert rc == L.EINVAL
        assert b"engine" in stencil_lib.stencil_last_error()
    small, big = ctypes.c_size_t(), ctypes.c_size_t()
    assert stencil_lib.stencil_batch_workspace_bytes(1, ctypes.byref(small)) == L.OK
    assert stencil_lib.stencil_batch_workspace_bytes(100, ctypes.byref(big)) == L.OK
    assert big.value > small.value > 0
    jobs = (L.BatchJob * 2)()
    for j, (nx, ny, nz, d) in zip(jobs, [(66, 70, 1, 2), (41, 37, 43, 3)]):
        j.dims, j.nx, j.ny, j.nz, j.radius, j.iterations = d, nx, ny, nz, 1, 1
    need = ctypes.c_size_t()
    assert stencil_lib.stencil_batch_workspace_bytes_for(jobs, 2, ctypes.byref(need)) == L.OK
    # two pitched copies of each ragged grid at least
    assert need.value >= 2 * 4 * (68 * 70 + 44 * 37 * 43)


def test_one_launch_batch_jobs_are_checked_without_device(stencil_lib):
    """The one-launch engine checks every job before it touches a device: a
    negative team field, a nonzero reserved field, bad buffers or an odd tile
    are refused with STENCIL_EINVAL; unknown workspaces are refused by the
    queries."""
    def job(**kw):
        j = L.BatchJob()
        j.d_u1, j.d_u2 = 4096, 8192
        j.dims, j.nx, j.ny, j.nz, j.radius, j.iterations, j.mode = 2, 64, 64, 1, 1, 3, 1
        for k, v in kw.items():
            if k == "reserved":
                j.reserved[0] = v
            else:
                setattr(j, k, v)
        return j
    ws = ctypes.c_void_p(1 << 20)
    for bad, word in [(dict(team=-1), b"team"), (dict(reserved=1), b"reserved"),
                      (dict(d_u2=4096), b"buffers"), (dict(tile_x=6), b"tile_x"),
                      (dict(radius=5), b"radius")]:
        jobs = (L.BatchJob * 2)(job(), job(**bad))
        rc = stencil_lib.stencil_batch_prepare_engine(jobs, 2, 2, 0, ws, 1 << 30, None)
        assert rc in (L.EINVAL, L.EUNSUPPORTED), bad
        assert word in stencil_lib.stencil_last_error() and b"job 1" in stencil_lib.stencil_last_error(), bad
    n = ctypes.c_int()
    assert stencil_lib.stencil_batch_launches(ws, ctypes.byref(n)) == L.EINVAL
    assert stencil_lib.stencil_batch_teams(ws, ctypes.byref(n), None, None, 0) == L.OK and n.value == 0
