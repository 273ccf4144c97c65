"""The tcgen05 convolution engine (5th-generation tensor cores, accumulator
in tensor memory; TMA-fed operands where the 128-pixel tiles are whole image
rows or row runs, cp.async-fed otherwise) against the warp-level mma.sync
engine and a torch float64 reference, on the same BF16 inputs."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

SHAPES = [  # n, cin, cout, h, w, dilation
    (1, 32, 32, 10, 9, 1), (2, 32, 64, 16, 24, 1), (2, 64, 128, 16, 16, 2), (1, 384, 128, 8, 16, 1),
    (2, 256, 256, 16, 12, 4), (3, 96, 32, 12, 20, 1), (1, 32, 64, 1, 200, 1),
    # shapes whose 128-pixel tiles are whole rows or row runs: TMA-fed operands
    (2, 32, 32, 128, 128, 1), (1, 96, 32, 64, 64, 1), (2, 128, 128, 32, 32, 1), (1, 32, 64, 4, 256, 1),
    (1, 256, 256, 16, 16, 4), (3, 192, 64, 8, 64, 1)]


def run_engines(n, cin, cout, h, w, dil, relu, engines=(1, 2)):
    import torch
    from thesis_gb300 import unet as U
    L = U._L()
    g = torch.Generator().manual_seed(cin * 7 + cout + dil)
    x = torch.randn(n, h, w, cin, generator=g).to(torch.bfloat16)
    wt = (torch.randn(cout, 9, cin, generator=g) * 0.1).to(torch.bfloat16)
    b = torch.randn(cout, generator=g).float()
    xd, wd, bd = x.cuda(), wt.cuda(), b.cuda()
    outs = {}
    for engine in engines:
        y = torch.full((n, h, w, cout), float("nan"), dtype=torch.bfloat16, device="cuda")
        U._chk(L.unet_conv3x3_fwd_engine(ctypes.byref(U.view(xd)), U._p(wd), U._p(bd),
                                         ctypes.byref(U.view(y)), relu, dil, engine, None),
               "engine %d" % engine)
        torch.cuda.synchronize()
        outs[engine] = y.cpu().double()
    X = x.double().permute(0, 3, 1, 2)
    W = wt.double().reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
    ref = torch.nn.functional.conv2d(X, W, b.double(), padding=dil, dilation=dil).permute(0, 2, 3, 1)
    if relu:
        ref = torch.relu(ref)
    return outs, ref


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("relu", [0, 1])
def test_tcgen05_conv_matches_mma_and_float64(cuda, shape, relu):
    import torch
    outs, ref = run_engines(*shape, relu)
    scale = ref.abs().max().item()
    for engine in (1, 2):
        assert torch.isfinite(outs[engine]).all(), engine
        assert (outs[engine] - ref).abs().max().item() / scale < 1e-2, engine
    # the engines differ only by the FP32 summation order before the BF16 rounding
    assert (outs[1] - outs[2]).abs().max().item() / scale < 1e-2


WG_SHAPES = [  # n, cin, cout, h, w, dilation
    (2, 32, 32, 16, 32, 1), (1, 96, 32, 8, 64, 1), (2, 64, 128, 8, 32, 1), (1, 384, 128, 4, 32, 1),
    (2, 256, 256, 8, 32, 4), (1, 128, 256, 16, 32, 2), (3, 32, 64, 5, 96, 1)]


@pytest.mark.parametrize("shape", WG_SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_tcgen05_weight_gradient_matches_mma_and_float64(cuda, shape):
    import torch
    from thesis_gb300 import unet as U
    n, cin, cout, h, w, dil = shape
    L = U._L()
    g = torch.Generator().manual_seed(cin + 3 * cout + dil)
    x = torch.randn(n, h, w, cin, generator=g).to(torch.bfloat16)
    dy = torch.randn(n, h, w, cout, generator=g).to(torch.bfloat16)
    xd, dyd = x.cuda(), dy.cuda()
    need = ctypes.c_size_t()
    U._chk(L.unet_wgrad_workspace_bytes(ctypes.byref(U.view(xd)), ctypes.byref(U.view(dyd)),
                                        ctypes.byref(need)), "ws")
    ws = torch.empty(need.value, dtype=torch.uint8, device="cuda")
    outs = {}
    for engine in (1, 2):
        dw = torch.zeros(cout, 9, cin, device="cuda")
        db = torch.zeros(cout, device="cuda")
        for _ in range(2):  # accumulates: two calls give twice the gradient
            U._chk(L.unet_conv3x3_wgrad_engine(ctypes.byref(U.view(xd)), ctypes.byref(U.view(dyd)),
                                               U._p(dw), U._p(db), dil, engine, U._p(ws), need.value,
                                               None), "wgrad %d" % engine)
        torch.cuda.synchronize()
        outs[engine] = (dw.cpu().double() / 2, db.cpu().double() / 2)
    X = x.double().permute(0, 3, 1, 2).requires_grad_(True)
    W = torch.zeros(cout, cin, 3, 3, dtype=torch.float64, requires_grad=True)
    out = torch.nn.functional.conv2d(X, W, None, padding=dil, dilation=dil)
    out.backward(dy.double().permute(0, 3, 1, 2))
    ref = W.grad.permute(0, 2, 3, 1).reshape(cout, 9, cin)
    refb = dy.double().sum((0, 1, 2))
    for engine in (1, 2):
        gw, gb = outs[engine]
        assert (gw - ref).abs().max().item() / ref.abs().max().item() < 1e-4, engine
        assert (gb - refb).abs().max().item() / refb.abs().max().item() < 1e-4, engine
