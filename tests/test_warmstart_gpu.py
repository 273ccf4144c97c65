"""Learned warm start, small scale: solver-generated pairs, training with the
library's own kernels, the ablation (sweeps to tolerance with and without the
trained network), and the combined method -- the network's prediction
followed by the mixed-precision refinement -- against plain FP32 Jacobi from
zero, each solve timed and checked against the FP64 steady state."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained(cuda):
    from thesis_gb300 import warmstart as W
    from thesis_gb300.unet import UNet
    fields, sols = W.generate_pairs(512, size=64, seed0=5000, sweeps=6000)
    # the generated solutions are converged
    assert max(W.S.residual(sols[k], 1) for k in range(0, 512, 64)) < 1e-5
    net = UNet(seed=1)
    losses, _ = W.train(net, fields, sols, epochs=4, batch=32, lr=2e-3)
    return net, losses


TRAIN = 64  # the test network's training size


def _solve_all(W, net, f, arm, ws, check=100):
    out = [W.solve_arm(net, f[k:k + 1], arm, 1e-5, ws, TRAIN, check) for k in range(f.shape[0])]
    return [o[0] for o in out], [o[1] for o in out], [o[2] for o in out], [o[4] for o in out]


def test_training_reduces_loss_and_network_beats_zero_init(trained):
    from thesis_gb300 import warmstart as W
    net, losses = trained
    assert losses[-1] < 0.5 * losses[0]
    f = W.borders(list(range(777000, 777008)), 128)
    ws = {st: W.S.ir_workspace((128, 128), 1, st) for st in ("fp16", "bf16")}
    sw = {}
    for arm in ("zero_fp32", "learned_fp32", "coons_fp32"):
        sweeps, res, secs, _ = _solve_all(W, net, f, arm, ws)
        assert max(res) < 1e-5 and min(secs) > 0
        sw[arm] = np.mean(sweeps)
    print("sweeps", sw)
    assert sw["learned_fp32"] < sw["zero_fp32"]
    # ablation: the same pipeline without the network (its Coons base field)
    assert sw["learned_fp32"] < sw["coons_fp32"]


def test_learned_plus_refinement_reaches_tolerance_faster(trained):
    """The combined arm on 128^2 problems: every solve ends below the
    tolerance, takes fewer sweeps and less time than plain FP32 from zero,
    and its final field is as close to the FP64 steady state as the plain
    solve's (both limited by the same residual tolerance)."""
    from thesis_gb300 import warmstart as W
    net, _ = trained
    f = W.borders(list(range(778000, 778006)), 128)
    ws = {st: W.S.ir_workspace((128, 128), 1, st) for st in ("fp16", "bf16")}
    for arm in ("zero_fp32", "learned_ir_fp16"):  # warm-up (kernels, buffers)
        W.solve_arm(net, f[:1], arm, 1e-3, ws, TRAIN)
    zs, zr, zt, zu = _solve_all(W, net, f, "zero_fp32", ws)
    ls, lr, lt, lu = _solve_all(W, net, f, "learned_ir_fp16", ws)
    assert max(zr) < 1e-5 and max(lr) < 1e-5
    print("zero %.0f sweeps %.2f ms, learned+fp16 %.0f sweeps %.2f ms"
          % (np.mean(zs), 1e3 * np.mean(zt), np.mean(ls), 1e3 * np.mean(lt)))
    assert np.mean(ls) < np.mean(zs)
    assert np.mean(lt) < np.mean(zt)
    for k in range(f.shape[0]):
        ex = W.exact_steady_state(f[k].cpu().numpy())
        ez = np.abs(zu[k].cpu().numpy() - ex).max() / np.abs(ex).max()
        el = np.abs(lu[k].cpu().numpy() - ex).max() / np.abs(ex).max()
        # equal accuracy: the refinement's error within a small factor of the
        # plain solve's, both far below the field's scale
        assert el < max(3 * ez, 1e-4) and ez < 1e-2


def test_refinement_engine_runs_persistent_on_the_learned_path(trained):
    from thesis_gb300 import warmstart as W
    net, _ = trained
    f = W.borders([779000], 128)
    u0, used = W.warm_init(net, f, train_size=TRAIN)
    assert used
    r = W.S.ir_solve_ex(u0.clone(), 1, 200000, "fp16", inner_sweeps=500, tol=1e-5)
    assert r["engine"] == "persistent2d" and r["rel_residual"] < 1e-5
    assert W.S.device_status() == 0


def test_inference_kernels_match_torch(cuda):
    """Border resampling, bilinear upsampling and the Coons fill (library
    kernels on the learned path) against torch on the same inputs."""
    import torch
    from thesis_gb300 import unet as U, warmstart as W
    f = W.borders([5, 6], 96)
    c = U.resample_border(f, 32, 32)
    idx = torch.round(torch.linspace(0, 95, 32, device=f.device)).long()
    ref = f[:, idx][:, :, idx]
    band = torch.ones(32, 32, dtype=torch.bool, device=f.device)
    band[1:-1, 1:-1] = False
    assert torch.equal(c[:, band], ref[:, band]) and torch.all(c[:, ~band] == 0)
    up = U.upsample_bilinear(c, f)
    ref_up = torch.nn.functional.interpolate(c[:, None], size=(96, 96), mode="bilinear",
                                             align_corners=True)[:, 0]
    inner = (slice(None), slice(1, -1), slice(1, -1))
    assert torch.allclose(up[inner], ref_up[inner], atol=1e-5, rtol=1e-5)
    assert torch.equal(up[:, 0], f[:, 0]) and torch.equal(up[:, :, -1], f[:, :, -1])
    cf = U.coons_fill(f)
    n, h, w = f.shape
    s = torch.linspace(0, 1, w, device=f.device)[None, None, :]
    t = torch.linspace(0, 1, h, device=f.device)[None, :, None]
    B, T, L, R = f[:, :1, :], f[:, -1:, :], f[:, :, :1], f[:, :, -1:]
    cp = ((1 - t) * B + t * T + (1 - s) * L + s * R -
          ((1 - s) * (1 - t) * f[:, :1, :1] + s * (1 - t) * f[:, :1, -1:] + (1 - s) * t * f[:, -1:, :1]
           + s * t * f[:, -1:, -1:]))
    assert torch.allclose(cf[inner], cp[inner], atol=1e-5)
    assert torch.equal(cf[:, 0], f[:, 0])
