"""CPU reference of the warm-start U-Net (TEST INFRASTRUCTURE ONLY).

The network of thesis_gb300/unet.py restated with torch CPU operators in
float64 (autograd supplies the reference gradients); the input features and
the masked MSE restate the library's unet_features / unet_mse.  Used only by
tests/ to check the CUDA kernels' forward pass and gradients.  The U-Net has no
counterpart in the reference project.
"""
from __future__ import annotations

import numpy as np

DILATION = {"ba": 2, "bb": 4}
LAYERS = [
    ("e0a", 32, 32), ("e0b", 32, 32), ("e1a", 32, 64), ("e1b", 64, 64),
    ("e2a", 64, 128), ("e2b", 128, 128), ("ba", 128, 256), ("bb", 256, 256),
    ("d2a", 384, 128), ("d2b", 128, 128), ("d1a", 192, 64), ("d1b", 64, 64),
    ("d0a", 96, 32), ("d0b", 32, 32),
]


def features(fields: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """fields [n, h, w] -> (x [n, 32, h, w], coons [n, h, w]) in float64."""
    f = fields.astype(np.float64)
    n, h, w = f.shape
    s = np.arange(w) / (w - 1)
    t = np.arange(h) / (h - 1)
    S, T = np.meshgrid(s, t)
    B = f[:, 0, :][:, None, :]
    Tp = f[:, -1, :][:, None, :]
    L = f[:, :, 0][:, :, None]
    R = f[:, :, -1][:, :, None]
    c00, c10 = f[:, 0, 0][:, None, None], f[:, 0, -1][:, None, None]
    c01, c11 = f[:, -1, 0][:, None, None], f[:, -1, -1][:, None, None]
    coons = ((1 - T) * B + T * Tp + (1 - S) * L + S * R -
             ((1 - S) * (1 - T) * c00 + S * (1 - T) * c10 + (1 - S) * T * c01 + S * T * c11))
    mask = np.zeros((h, w))
    mask[0, :] = mask[-1, :] = mask[:, 0] = mask[:, -1] = 1.0
    coons = np.where(mask > 0, f, coons)
    x = np.zeros((n, 32, h, w))
    x[:, 0] = f * mask
    x[:, 1] = mask
    x[:, 2] = coons
    return x, coons


def forward(torch, params: dict, x, head_w, head_b):
    """params: name -> (w [cout, 9, cin], b [cout]) torch tensors; x NCHW."""
    F = torch.nn.functional

    def conv(name, t):
        w, b = params[name]
        cout, _, cin = w.shape
        wk = w.reshape(cout, 3, 3, cin).permute(0, 3, 1, 2)
        d = DILATION.get(name, 1)
        return F.relu(F.conv2d(t, wk, b, padding=d, dilation=d))

    e0 = conv("e0b", conv("e0a", x))
    e1 = conv("e1b", conv("e1a", F.max_pool2d(e0, 2)))
    e2 = conv("e2b", conv("e2a", F.max_pool2d(e1, 2)))
    bt = conv("bb", conv("ba", F.max_pool2d(e2, 2)))
    up = lambda t: F.interpolate(t, scale_factor=2, mode="nearest")
    d2 = conv("d2b", conv("d2a", torch.cat([up(bt), e2], 1)))
    d1 = conv("d1b", conv("d1a", torch.cat([up(d2), e1], 1)))
    d0 = conv("d0b", conv("d0a", torch.cat([up(d1), e0], 1)))
    return (d0 * head_w[None, :, None, None]).sum(1) + head_b


def masked_mse(torch, out, coons, target):
    n, h, w = out.shape
    d = (coons + out - target)[:, 1:-1, 1:-1]
    return (d * d).sum() / (n * (h - 2) * (w - 2))
