"""CPU oracle for the learned-preconditioner CNN (TEST INFRASTRUCTURE ONLY).

The network has no counterpart in the reference, so this oracle restates the
mathematics directly with torch's CPU convolution in float64:

* ``conv3d``       y[v, co] = sum_{t, ci} w[t, co, ci] x[v + off(t), ci],
                   zero padding 1, tap t = (kd*3 + kh)*3 + kw reading offset
                   (kd-1, kh-1, kw-1) (a cross-correlation, as
                   ``torch.nn.functional.conv3d``).
* ``conv3d_dgrad`` d/dx of the above (``torch.nn.grad.conv3d_input``).
* ``conv3d_wgrad`` d/dw of the above (``torch.nn.grad.conv3d_weight``).
* ``expand``       the preconditioner's four layer weights from its free
                   parameters (two layers and their transposes).
* ``network``      the preconditioner z = |r| N^T N (r/|r|) + skip r with the
                   same bfloat16 rounding points as the GPU path (packed input
                   and every hidden activation), differentiable by autograd.

Activations are channels-last [D, H, W, C]; weights [27, Cout, Cin].
"""

from __future__ import annotations

import torch
import torch.nn.functional as F

__all__ = ["to_torch_weight", "conv3d", "conv3d_dgrad", "conv3d_wgrad", "bf16_round", "expand", "network",
           "network_loss"]


def to_torch_weight(w: torch.Tensor) -> torch.Tensor:
    """[27, co, ci] -> torch's [co, ci, 3, 3, 3]."""
    co, ci = w.shape[1], w.shape[2]
    return w.reshape(3, 3, 3, co, ci).permute(3, 4, 0, 1, 2)


def _nc(x):  # [D, H, W, C] -> [1, C, D, H, W]
    return x.permute(3, 0, 1, 2).unsqueeze(0)


def _cl(y):  # [1, C, D, H, W] -> [D, H, W, C]
    return y[0].permute(1, 2, 3, 0)


def conv3d(x: torch.Tensor, w: torch.Tensor) -> torch.Tensor:
    x, w = x.double(), w.double()
    return _cl(F.conv3d(_nc(x), to_torch_weight(w), padding=1))


def conv3d_dgrad(gy: torch.Tensor, w: torch.Tensor) -> torch.Tensor:
    gy, w = gy.double(), w.double()
    D, H, W, _ = gy.shape
    gx = torch.nn.grad.conv3d_input((1, w.shape[2], D, H, W), to_torch_weight(w), _nc(gy), padding=1)
    return _cl(gx)


def conv3d_wgrad(x: torch.Tensor, gy: torch.Tensor) -> torch.Tensor:
    x, gy = x.double(), gy.double()
    co, ci = gy.shape[-1], x.shape[-1]
    gw = torch.nn.grad.conv3d_weight(_nc(x), (co, ci, 3, 3, 3), _nc(gy), padding=1)  # [co, ci, 3, 3, 3]
    return gw.permute(2, 3, 4, 0, 1).reshape(27, co, ci)


class _RoundBF16(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        return x.to(torch.bfloat16).to(x.dtype)

    @staticmethod
    def backward(ctx, g):
        return g


def bf16_round(x: torch.Tensor) -> torch.Tensor:
    """Round to bfloat16 and back (straight-through for autograd)."""
    return _RoundBF16.apply(x)


def expand(v1: torch.Tensor, v2: torch.Tensor):
    """The preconditioner's four layers from v1 [27, 8] and v2 [27, 8, 8]:
    layer 1 maps each real component (bf16 value in channel 0 / 1 and its
    remainder in 2 / 3, same weights) to 8 features (channels 0-7 / 8-15),
    layer 2 mixes the 8 features of each component, layers 3 and 4 are the
    transposes of 2 and 1 (taps reversed, channels swapped)."""
    taps = v1.shape[0]
    w1 = v1.new_zeros(taps, 16, 16)
    w2 = v1.new_zeros(taps, 16, 16)
    for c in (0, 1):
        w1[:, 8 * c:8 * c + 8, c] = v1
        w1[:, 8 * c:8 * c + 8, c + 2] = v1
        w2[:, 8 * c:8 * c + 8, 8 * c:8 * c + 8] = v2
    t = lambda w: w.flip(0).transpose(1, 2)
    return [w1, w2, t(w2), t(w1)]


def network(r: torch.Tensor, v1: torch.Tensor, v2: torch.Tensor, skip) -> torch.Tensor:
    """z = |r| N^T N (r / |r|) + skip r for a [D, H, W] complex residual
    (float64): the input as a two-term bfloat16 split, the hidden activations
    rounded to bfloat16, the last layer in float32."""
    nrm = torch.linalg.vector_norm(r)
    rh = r / nrm
    v = torch.stack([rh.real, rh.imag], dim=-1).float()
    hi = v.to(torch.bfloat16).float()
    lo = (v - hi).to(torch.bfloat16).float()
    x = torch.cat([hi.double(), lo.double(), torch.zeros(*r.shape, 12, dtype=torch.float64)], dim=-1)
    ws = expand(bf16_round(v1.double()), bf16_round(v2.double()))
    for i, w in enumerate(ws):
        y = _cl(F.conv3d(_nc(x), to_torch_weight(w), padding=1))
        x = bf16_round(y) if i < len(ws) - 1 else y
    return nrm * torch.complex(x[..., 0], x[..., 1]) + skip * r


def network_loss(r: torch.Tensor, e: torch.Tensor, v1, v2, skip) -> torch.Tensor:
    """|z - e|^2 / |e|^2 (the "mse" loss of the GPU trainer)."""
    z = network(r, v1, v2, skip)
    return (torch.linalg.vector_norm(z - e) ** 2) / (torch.linalg.vector_norm(e) ** 2)
