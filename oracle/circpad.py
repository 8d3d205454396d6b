"""CPU restatement of the reference circular padding (TEST INFRASTRUCTURE ONLY).

* ``circular_pad``         <- ``functional/_interp/_circ_pad.py:10-83``: the
  last ``len(padding) // 2`` dims padded circularly, ``padding`` in
  ``torch.nn.functional.pad`` order (pairs from the last dim backwards).
  Restated as one modular ``index_select`` per dim (the same copies).
* ``circular_pad_adjoint`` <- ``:119-134`` (autograd through the pad there):
  per dim, ``index_add_`` of the padded slices onto their sources.
* ``conv_circular``        <- ``linops/convolution.py:120-130,140-150``: the
  Convolution linop's circular forward and adjoint with torch's conv.
"""

from __future__ import annotations

import torch
import torch.nn.functional as F

__all__ = ["circular_pad", "circular_pad_adjoint", "conv_circular"]


def _pairs(padding):
    padding = [int(p) for p in padding]
    return [(padding[2 * i], padding[2 * i + 1]) for i in range(len(padding) // 2)][::-1]


def circular_pad(t: torch.Tensor, padding) -> torch.Tensor:
    pairs = _pairs(padding)
    nd = len(pairs)
    out = t
    for e, (lo, hi) in enumerate(pairs):
        dim = t.ndim - nd + e
        n = t.shape[dim]
        out = out.index_select(dim, torch.remainder(torch.arange(-lo, n + hi), n))
    return out


def circular_pad_adjoint(t: torch.Tensor, padding) -> torch.Tensor:
    pairs = _pairs(padding)
    nd = len(pairs)
    out = t
    for e, (lo, hi) in enumerate(pairs):
        dim = t.ndim - nd + e
        n = t.shape[dim] - lo - hi
        shape = list(out.shape)
        shape[dim] = n
        acc = torch.zeros(shape, dtype=t.dtype)
        acc.index_add_(dim, torch.remainder(torch.arange(-lo, n + hi), n), out)
        out = acc
    return out


def conv_circular(kernel: torch.Tensor, x: torch.Tensor, adjoint: bool = False) -> torch.Tensor:
    ndim = kernel.dim()
    pad = []
    for s in reversed(kernel.shape):
        pad += [0, 0 if s % 2 else 1]
    kernel = F.pad(kernel, pad)
    half = [(s // 2, s // 2) for s in kernel.shape]
    cpad = [v for pair in reversed(half) for v in pair]
    w = torch.flip(kernel, dims=tuple(range(ndim)))[None, None]
    if adjoint:
        w = torch.flip(w, dims=tuple(range(-ndim, 0))).conj()
    lead = x.shape[: x.ndim - ndim]
    xf = x.reshape(-1, 1, *x.shape[x.ndim - ndim:])
    y = (F.conv1d, F.conv2d, F.conv3d)[ndim - 1](circular_pad(xf, cpad), w, padding=0)
    return y.reshape(*lead, *y.shape[2:])
