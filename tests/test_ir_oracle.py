"""The CPU restatement of the mixed-precision refinement (oracle/ir_oracle.py):
its 16-bit roundings against torch's conversions, and its result against the
plain FP32 sweep loop of the C oracle at equal sweep counts (CPU only)."""
import numpy as np
import pytest

from oracle import ir_oracle as IRO
from oracle import oracle as O


def _samples():
    rng = np.random.default_rng(3)
    x = np.concatenate([
        rng.standard_normal(20000).astype(np.float32),
        (rng.standard_normal(5000) * 1e-6).astype(np.float32),
        (rng.standard_normal(5000) * 1e-40).astype(np.float32),  # FP32 subnormals
        np.array([0.0, -0.0, 1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 65504.0, 6e-8, -6e-8],
                 np.float32)])
    return x


@pytest.mark.parametrize("name", ["bf16", "fp16"])
def test_roundings_match_torch(name):
    torch = pytest.importorskip("torch")
    x = _samples()
    ref = torch.from_numpy(x).to(torch.bfloat16 if name == "bf16" else torch.float16).float().numpy()
    got = IRO.ROUND[name](x)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def _field(shape, seed):
    rng = np.random.default_rng(seed)
    u = rng.random(shape, dtype=np.float32)
    t = np.linspace(0, 1, shape[1], dtype=np.float32)
    u[0, :] = np.sin(3 * np.pi * t)
    u[-1, :] = np.cos(2 * np.pi * t)
    return u


# bounds: the unit roundoff of the storage format (BF16 2^-8, FP16 2^-11),
# relative to the largest value of the field
@pytest.mark.parametrize("storage,bound", [("bf16", 2 ** -8), ("fp16", 2 ** -11)])
@pytest.mark.parametrize("radius,inner", [(1, 50), (2, 7), (4, 1)])
def test_refinement_tracks_fp32_loop(storage, bound, radius, inner):
    shape, iters = (48, 64), 120
    u0 = _field(shape, radius)
    got, outer = IRO.ir_solve(u0, radius, iters, inner, storage)
    assert outer == -(-iters // inner)
    fp32 = O.run(u0.copy(), u0.copy(), radius, O.JACOBI, iters)
    err = float(np.abs(got - fp32).max() / np.abs(fp32).max())
    assert err < bound
    band = np.ones(shape, bool)
    band[radius:-radius, radius:-radius] = False
    assert np.array_equal(got[band], u0[band])
    # equal accuracy at equal sweep counts
    assert O.rel_residual(got, radius) == pytest.approx(O.rel_residual(fp32, radius), rel=0.05)


def test_one_sweep_per_step_is_a_plain_sweep_to_storage_precision():
    u0 = _field((32, 40), 9)
    got, _ = IRO.ir_solve(u0, 1, 1, 1, "fp16")
    want = O.run(u0.copy(), u0.copy(), 1, O.JACOBI, 1)
    rhs, s = IRO.residual_scaled(u0, 1, "fp16")
    # u + s * E(r / s): the only rounding beyond FP32 is that of r to FP16
    assert float(np.abs(got - want).max()) <= float(s) * 2 ** -11 + 1e-6
