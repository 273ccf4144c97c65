"""CPU tests of the oracle itself: pinned against the reference's golden output."""
import glob
import os
import tempfile

import numpy as np
import pytest

from oracle import build as obuild
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "legacy_*.npz")))


def load_fixture(path):
    z = np.load(path)
    return (z["grid"], int(z["dims"]), int(z["dim"]), int(z["radius"]), int(z["iterations"]))


def test_fixtures_present():
    assert len(FIXTURES) >= 10


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_oracle_matches_reference_golden(path):
    """LEGACY restatement == the reference's own stencil_cpu output, bit for bit."""
    grid, dims, dim, radius, iters = load_fixture(path)
    a = O.init_reference(grid.shape)
    b = np.zeros_like(a)  # the reference's second buffer is a fresh malloc
    res = O.run(a, b, radius, O.LEGACY, iters, threads=1)
    assert np.isfinite(grid).all()
    assert np.array_equal(res.view(np.uint32), grid.view(np.uint32))


@pytest.mark.skipif(not obuild.reference_available(), reason="reference sources absent")
def test_oracle_matches_reference_binary_fresh():
    """Rebuilds one reference binary from its sources and compares a fresh run."""
    cfg = (3, 24, 2, 6)
    exe = obuild.build_ref([cfg])[0]
    with tempfile.TemporaryDirectory() as tmp:
        path, _ = obuild.run_ref(exe, tmp)
        ref = np.fromfile(path, dtype=np.float32).reshape((24,) * 3)
    a = O.init_reference(ref.shape)
    res = O.run(a, np.zeros_like(a), 2, O.LEGACY, 6)
    assert np.array_equal(res.view(np.uint32), ref.view(np.uint32))


def test_threads_do_not_change_results():
    u = O.uniform((20, 33, 37), seed=5)
    a1, b1 = u.copy(), u.copy()
    a4, b4 = u.copy(), u.copy()
    r1 = O.run(a1, b1, 2, O.JACOBI, 5, threads=1)
    r4 = O.run(a4, b4, 2, O.JACOBI, 5, threads=4)
    assert np.array_equal(r1.view(np.uint32), r4.view(np.uint32))


def test_uniform_generator_known_values():
    # SplitMix64-derived values; fixed forever (CPU and GPU must agree).
    vals = [O.uniform01(0, i) for i in range(4)] + [O.uniform01(12345, 7)]
    u = O.uniform((1000,), 99)
    assert all(0.0 <= v < 1.0 for v in vals)
    assert np.all((u >= 0) & (u < 1)) and abs(float(u.mean()) - 0.5) < 0.05
    assert len(set(vals)) == 5
    np.testing.assert_array_equal(O.uniform((8,), 0), np.array(vals[:4] + [O.uniform01(0, i) for i in range(4, 8)], np.float32))
    # value = top 24 bits of the mixed word times 2^-24: an exact multiple of 2^-24
    assert all(float(v) * 2 ** 24 == int(float(v) * 2 ** 24) for v in vals)


def test_jacobi_constant_is_fixed_point():
    u = np.full((16, 16, 16), 0.5, np.float32)
    res = O.run(u.copy(), u.copy(), 2, O.JACOBI, 3)
    assert np.all(res == 0.5)


def test_fp64_twin_close_to_fp32():
    u = O.uniform((40, 40), seed=11)
    r32 = O.run(u.copy(), u.copy(), 1, O.JACOBI, 200)
    u64 = u.astype(np.float64)
    r64 = O.run(u64.copy(), u64.copy(), 1, O.JACOBI, 200)
    err, bad = O.max_rel_err(r32, r64)
    assert bad == 0 and err < 1e-5


def test_border_band_untouched():
    u = O.uniform((12, 13, 14), seed=3)
    dst = np.full_like(u, -7.0)
    O.sweep(u, dst, 2, O.JACOBI)
    band = np.ones(u.shape, bool)
    band[2:-2, 2:-2, 2:-2] = False
    assert np.all(dst[band] == -7.0) and np.all(dst[~band] != -7.0)


def test_residual_decreases_under_jacobi():
    u = O.uniform((48, 48), seed=1)
    r0 = O.rel_residual(u, 1)
    res = O.run(u.copy(), u.copy(), 1, O.JACOBI, 500)
    assert O.rel_residual(res, 1) < 0.5 * r0


def test_legacy_reference_state_diverges_to_nan():
    """The reference update subtracts the centre and diverges (documented fact)."""
    a = O.init_reference((64, 64))
    res = O.run(a, np.zeros_like(a), 1, O.LEGACY, 1000)
    assert not np.isfinite(res[1:-1, 1:-1]).all()
    nan_err, bad = O.max_rel_err(res, res)
    assert bad > 0


def test_error_metrics():
    a = np.array([1.0, 2.0, np.nan], np.float32)
    b = np.array([1.0, 2.5, 1.0], np.float32)
    e, bad = O.max_rel_err(a, b)
    assert bad == 1 and abs(e - 0.2) < 1e-7
    assert O.sq_err(a[:2], b[:2]) == pytest.approx(0.25)
