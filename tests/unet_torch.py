"""CPU restatement of the learned preconditioner's U-Net in PyTorch (autograd),
used as the oracle for the CUDA forward and backward kernels.

It mirrors csrc/unet.cu layer for layer and rounds every stored activation to
BF16 as the kernels do (a straight-through rounding, so gradients flow in
FP32 like the kernels' FP32 activation gradients).  Weights are rounded to
BF16 too; products accumulate in FP32.
"""
import numpy as np
import torch
import torch.nn.functional as F


def _bf16(x):
    return x + (x.to(torch.bfloat16).float() - x).detach()


def split_params(params, shapes):
    out, off = [], 0
    for co, ci, k in shapes:
        n = co * ci * k * k
        out.append(torch.as_tensor(np.asarray(params[off:off + n]), dtype=torch.float32).reshape(co, ci, k, k))
        off += n
    return out


def forward(weights, x):
    """weights: 12 tensors (autograd leaves allowed); x: [B, ny, nx] FP32."""
    w = [_bf16(t) for t in weights]
    h = _bf16(x[:, None])
    enc = []
    for l in range(4):
        a = _bf16(F.relu(F.conv2d(h, w[2 * l], padding=1)))
        e = _bf16(F.relu(F.conv2d(a, w[2 * l + 1], padding=1)))
        enc.append(e)
        if l < 3:
            h = _bf16(F.avg_pool2d(e, 2))
    d = enc[3]
    for l, li in ((2, 8), (1, 9), (0, 10)):
        u = F.interpolate(d, scale_factor=2, mode="nearest")
        d = _bf16(F.relu(F.conv2d(torch.cat([u, enc[l]], dim=1), w[li], padding=1)))
    return F.conv2d(d, w[11])[:, 0]
