"""CPU oracle of the learned warm-start network (test infrastructure only).

The same encoder-decoder as the GPU library's (tg_cnn.cu), written with
PyTorch CPU ops in float64 so that autograd gives the reference gradient:
tensors are (1, C, nz, nx, ny) for a node grid stored ((z*nx)+x)*ny+y with
channels last; a layer's weights W[27][cin][cout] (tap k = (dz+1)*9 +
(dx+1)*3 + (dy+1)) map to torch's [cout][cin][dz][dx][dy] cross-correlation
kernel.  Pooling averages the present children of each coarse node (ceil
mode), upsampling repeats each coarse node to its children and crops.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

SPEC = [(7, 16), (16, 32), (32, 64), (64, 32), (32, 16), (16, 3)]


def unpack(params):
    p = torch.as_tensor(np.asarray(params, dtype=np.float64))
    out, off = [], 0
    for cin, cout in SPEC:
        w = p[off:off + 27 * cin * cout].reshape(3, 3, 3, cin, cout).permute(4, 3, 0, 1, 2)
        off += 27 * cin * cout
        b = p[off:off + cout]
        off += cout
        out.append((w.contiguous(), b.contiguous()))
    assert off == p.numel()
    return out


def _pool(x):
    nz, nx, ny = x.shape[2:]
    pad = (0, ny % 2, 0, nx % 2, 0, nz % 2)
    s = F.avg_pool3d(F.pad(x, pad), 2, 2) * 8.0
    ones = torch.ones((1, 1, nz, nx, ny), dtype=x.dtype)
    c = F.avg_pool3d(F.pad(ones, pad), 2, 2) * 8.0
    return s / c


def _up(x, shape):
    y = x.repeat_interleave(2, 2).repeat_interleave(2, 3).repeat_interleave(2, 4)
    return y[:, :, :shape[0], :shape[1], :shape[2]]


def forward(layers, x0):
    """x0: (1, 7, nz, nx, ny) -> y: (1, 3, nz, nx, ny)"""
    conv = lambda x, i: F.conv3d(x, layers[i][0], layers[i][1], padding=1)
    e1 = F.relu(conv(x0, 0))
    e2 = F.relu(conv(_pool(e1), 1))
    e3 = F.relu(conv(_pool(e2), 2))
    d2 = F.relu(conv(_up(e3, e2.shape[2:]), 3) + e2)
    d1 = F.relu(conv(_up(d2, e1.shape[2:]), 4) + e1)
    return conv(d1, 5)


def to_torch(a, grid, c):
    """channels-last node array [n][c] -> (1, c, nz, nx, ny)"""
    nx, ny, nz = grid
    t = torch.as_tensor(np.asarray(a, dtype=np.float64)).reshape(nz, nx, ny, c)
    return t.permute(3, 0, 1, 2).unsqueeze(0).contiguous()


def from_torch(t):
    return t[0].permute(1, 2, 3, 0).reshape(-1, t.shape[1]).detach().numpy()


def loss_and_grad(params, x0, target, grid):
    """MSE loss mean((y - t)^2) and its gradient w.r.t. the flat parameters."""
    p = torch.tensor(np.asarray(params, dtype=np.float64), requires_grad=True)
    out, off = [], 0
    for cin, cout in SPEC:
        w = p[off:off + 27 * cin * cout].reshape(3, 3, 3, cin, cout).permute(4, 3, 0, 1, 2)
        off += 27 * cin * cout
        b = p[off:off + cout]
        off += cout
        out.append((w, b))
    y = forward(out, to_torch(x0, grid, 7))
    t = to_torch(target, grid, 3)
    loss = ((y - t) ** 2).mean()
    loss.backward()
    return float(loss), p.grad.numpy().copy(), from_torch(y)


def adam_steps(params, grads, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """Parameters after len(grads) Adam steps from params with zero moments
    (Kingma & Ba, bias-corrected), in FP32 like the network's optimiser:
    m = b1 m + (1-b1) g, v = b2 v + (1-b2) g^2,
    w -= lr (m / (1-b1^t)) / (sqrt(v / (1-b2^t)) + eps)."""
    f = np.float32
    w = np.asarray(params, dtype=f).copy()
    m = np.zeros_like(w)
    v = np.zeros_like(w)
    for t, g in enumerate(grads, start=1):
        g = np.asarray(g, dtype=f)
        m = f(b1) * m + f(1 - b1) * g
        v = f(b2) * v + f(1 - b2) * g * g
        c1, c2 = f(1 - b1 ** t), f(1 - b2 ** t)
        w = w - f(lr) * (m / c1) / (np.sqrt(v / c2) + f(eps))
    return w
