"""Learned warm start, small scale: solver-generated pairs, training with the
library's own kernels, and the ablation -- sweeps to tolerance with and
without the trained network."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_training_reduces_loss_and_network_beats_zero_init(cuda):
    import torch
    from thesis_gb300 import warmstart as W
    from thesis_gb300.unet import UNet
    fields, sols = W.generate_pairs(512, size=64, seed0=5000, sweeps=6000)
    # the generated solutions are converged
    assert max(W.S.residual(sols[k], 1) for k in range(0, 512, 64)) < 1e-5
    net = UNet(seed=1)
    losses, _ = W.train(net, fields, sols, epochs=4, batch=32, lr=2e-3)
    assert losses[-1] < 0.5 * losses[0]
    seeds = list(range(777000, 777008))
    f = W.borders(seeds, 128)
    zero = list(f.clone())
    pred = W.predict(net, f, "coarse", train_size=64)
    r_zero = W.residuals(zero)
    sw_zero, _ = W.sweeps_to_tol(zero, 1e-5, chunk=500)
    sw_net, _ = W.sweeps_to_tol(list(pred), 1e-5, chunk=500)
    # ablation: the same pipeline without the network (its Coons base field)
    sw_coons, _ = W.sweeps_to_tol(list(W.coons_fill(f)), 1e-5, chunk=500)
    print("sweeps zero %s coons %s net %s" % (np.mean(sw_zero), np.mean(sw_coons), np.mean(sw_net)))
    assert np.mean(sw_net) < np.mean(sw_zero)
    assert np.mean(sw_net) < np.mean(sw_coons)
    # fallback rule inputs are well defined
    r_net = W.residuals(list(pred))
    assert all(np.isfinite(r_net)) and all(np.isfinite(r_zero))
