"""Oracle (test infrastructure only): the warm-start U-Net in PyTorch on the
CPU in FP32, rounding to BF16 at the points where the GPU stores BF16 (the
normalised input, each convolution's weights and GELU output (the tanh form
of GELU, as the GPU computes it) except the
last one, which feeds the FP32 head directly, pooled and upsampled
activations, and the gradient of every convolution's pre-activation).  Used to check the GPU forward pass, the loss gradients and
the Adam update (Kingma & Ba 2015).

Parameter vector layout (shared with libff): per convolution W[27][cin][cout]
with tap = (dz+1) 9 + (dy+1) 3 + (dx+1), then bias[cout], in the order
enc0a enc0b enc1a enc1b bot_a bot_b dec1a dec1b dec0a dec0b, then the 1x1
head's 16 weights and bias.
"""
import math

import numpy as np
import torch
import torch.nn.functional as F

SPEC = [(3, 16), (16, 16), (16, 32), (32, 32), (32, 64), (64, 64), (96, 32), (32, 32), (48, 16), (16, 16)]


def param_count():
    return sum(27 * ci * co + co for ci, co in SPEC) + 17


def bf16(x):
    return x.to(torch.bfloat16).to(torch.float32)


class _RoundGrad(torch.autograd.Function):
    """Identity forward; the backward gradient rounded to BF16."""

    @staticmethod
    def forward(ctx, x):
        return x.view_as(x)

    @staticmethod
    def backward(ctx, g):
        return bf16(g)


def split(params):
    params = torch.as_tensor(np.asarray(params, np.float32))
    convs, off = [], 0
    for ci, co in SPEC:
        w = params[off:off + 27 * ci * co].reshape(3, 3, 3, ci, co)   # [dz][dy][dx][ci][co]
        off += 27 * ci * co
        b = params[off:off + co]
        off += co
        convs.append((w, b))
    head = params[off:off + 17]
    return convs, head


def scales(b, p_prev, h, shape):
    n = b.size
    sb = math.sqrt(float(np.sum(np.asarray(b, np.float64) ** 2)) / n)
    sp = math.sqrt(float(np.sum(np.asarray(p_prev, np.float64) ** 2)) / n) if p_prev is not None else 0.0
    L = h * min(shape)
    if not sp > 0:
        sp = sb * L * L / (4.0 * math.pi * math.pi)
    return np.float32(sb if sb > 0 else 1.0), np.float32(sp if sp > 0 else 1.0)


def forward(params, b, mask, p_prev, h, shape, requires_grad=False):
    """Returns (raw output in normalised units, scales, parameter tensors)."""
    nx, ny, nz = shape
    sb, sp = scales(b, p_prev, h, shape)
    x = np.zeros((1, 3, nz, ny, nx), np.float32)
    x[0, 0] = (np.asarray(b, np.float32) * np.float32(1.0 / sb)).reshape(nz, ny, nx)
    if mask is not None:
        x[0, 1] = np.asarray(mask, np.float32).reshape(nz, ny, nx)
    if p_prev is not None:
        x[0, 2] = (np.asarray(p_prev, np.float32) * np.float32(1.0 / sp)).reshape(nz, ny, nx)
    x = bf16(torch.from_numpy(x))
    convs, head = split(params)
    tw = []
    for w, bb in convs:
        w = w.clone().requires_grad_(requires_grad)
        bb = bb.clone().requires_grad_(requires_grad)
        tw.append((w, bb))
    head = head.clone().requires_grad_(requires_grad)

    def conv(i, inp, store_bf16=True):
        w, bb = tw[i]
        wt = bf16(w).permute(4, 3, 0, 1, 2)   # [co][ci][dz][dy][dx]
        z = F.conv3d(inp, wt, padding=1) + bb.view(1, -1, 1, 1, 1)
        z = _RoundGrad.apply(z)
        y = F.gelu(z, approximate="tanh")
        return bf16(y) if store_bf16 else y

    e0 = conv(1, conv(0, x))
    e1 = conv(3, conv(2, bf16(F.avg_pool3d(e0, 2))))
    bt = conv(5, conv(4, bf16(F.avg_pool3d(e1, 2))))
    d1 = conv(7, conv(6, torch.cat([F.interpolate(bt, scale_factor=2, mode="nearest"), e1], 1)))
    # the last convolution's output feeds the FP32 head without BF16 rounding
    d0 = conv(9, conv(8, torch.cat([F.interpolate(d1, scale_factor=2, mode="nearest"), e0], 1)), store_bf16=False)
    raw = (d0 * head[:16].view(1, -1, 1, 1, 1)).sum(1)[0] + head[16]
    return raw, (sb, sp), tw, head


def predict(params, b, mask, p_prev, h, shape):
    raw, (sb, sp), _, _ = forward(params, b, mask, p_prev, h, shape)
    return (raw.detach().numpy().ravel() * sp).astype(np.float32)


LAP_W = 0.25


def graph_laplacian(d):
    """7-point graph Laplacian of a (nz, ny, nx) grid: sum over the existing
    face neighbours of d_nbr - d_v (edge-replicated padding gives 0 across
    the domain edge)."""
    p = F.pad(d[None, None], (1, 1, 1, 1, 1, 1), mode="replicate")[0, 0]
    c = p[1:-1, 1:-1, 1:-1]
    return (p[1:-1, 1:-1, :-2] + p[1:-1, 1:-1, 2:] + p[1:-1, :-2, 1:-1] + p[1:-1, 2:, 1:-1] +
            p[:-2, 1:-1, 1:-1] + p[2:, 1:-1, 1:-1] - 6.0 * c)


def loss_and_grads(params, b, mask, p_prev, target, h, shape):
    """Loss mean(d^2) + LAP_W mean((D d)^2) with d = raw - target / sp and D
    the grid's graph Laplacian (the GPU's k_loss_* kernels)."""
    raw, (sb, sp), tw, head = forward(params, b, mask, p_prev, h, shape, requires_grad=True)
    t = torch.from_numpy((np.asarray(target, np.float32) * np.float32(1.0 / sp)).reshape(raw.shape))
    d = raw - t
    loss = (d ** 2).mean() + LAP_W * (graph_laplacian(d.reshape(shape[2], shape[1], shape[0])) ** 2).mean()
    loss.backward()
    grads = []
    for w, bb in tw:
        grads.append(w.grad.reshape(-1))
        grads.append(bb.grad.reshape(-1))
    grads.append(head.grad.reshape(-1))
    return float(loss.detach()), torch.cat(grads).numpy()


def adam(params, grads, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step on float32 arrays; returns (params, m, v)."""
    m = b1 * m + (1 - b1) * grads
    v = b2 * v + (1 - b2) * grads * grads
    c1, c2 = 1 - b1 ** t, 1 - b2 ** t
    return params - lr * (m / c1) / (np.sqrt(v / c2) + eps), m, v
