"""CPU restatement of the reference unfold / fold path (TEST INFRASTRUCTURE ONLY).

* ``get_nblocks`` <- ``src/torchlinops/functional/_unfold/nblocks.py:6-33``:
  ``(im - block) // stride + 1`` per dimension.
* ``unfold``      <- ``_unfold_torch`` + ``unfold`` (unfold.py:31-69,531-561):
  block ``b`` of the last ``ndim`` dims copied into ``out[..., b, :]``; the
  mask is applied after the full unfold as ``y[..., mask]`` (unfold.py:68).
  Restated with ``Tensor.unfold`` (same elements, bit-exact).
* ``fold``        <- ``_fold_torch`` + ``fold`` (fold.py:32-63,489-517,520-537):
  overlapping blocks summed into a zero array in ascending block order
  (``itertools.product`` over the block grid); with a mask the blocks are
  first scattered into a zero ``[..., *nblocks, *block]`` buffer.
"""

from __future__ import annotations

from itertools import product
from math import prod

import torch

__all__ = ["get_nblocks", "unfold", "fold", "norm_weights"]


def get_nblocks(im_size, block_size, stride=None):
    stride = stride if stride is not None else (1,) * len(block_size)
    return tuple((i - b) // s + 1 for i, b, s in zip(im_size, block_size, stride))


def unfold(x: torch.Tensor, block_size, stride=None, mask=None) -> torch.Tensor:
    ndim = len(block_size)
    stride = tuple(stride) if stride is not None else (1,) * ndim
    nb = get_nblocks(x.shape[-ndim:], block_size, stride)
    if any(b <= 0 for b in nb):
        raise ValueError(f"Found 0 in nblocks: {nb}")
    y = x
    first = x.ndim - ndim
    for e in range(ndim):
        # each Tensor.unfold appends the window dim at the end, so after the
        # loop the layout is [..., *nblocks, *block] as in the reference
        y = y.unfold(first + e, block_size[e], stride[e])
    y = y.contiguous()
    if mask is not None:
        y = y[..., mask]
    return y


def fold(y: torch.Tensor, im_size, block_size, stride=None, mask=None) -> torch.Tensor:
    ndim = len(block_size)
    stride = tuple(stride) if stride is not None else (1,) * ndim
    nb = get_nblocks(im_size, block_size, stride)
    if mask is not None:
        batch = y.shape[: y.ndim - (ndim + 1)]
        tmp = torch.zeros(*batch, *nb, *block_size, dtype=y.dtype)
        tmp[..., mask] = y
        y = tmp
    batch = y.shape[: y.ndim - 2 * ndim]
    out = torch.zeros(*batch, *im_size, dtype=y.dtype)
    lead = (slice(None),) * len(batch)
    for b in product(*(range(n) for n in nb)):
        slc = tuple(slice(i * s, i * s + k) for i, s, k in zip(b, stride, block_size))
        out[lead + slc] += y[lead + tuple(b)]
    return out


def norm_weights(im_size, block_size, stride=None, mask=None) -> torch.Tensor:
    """fold(unfold(ones)) as in get_norm_weights (array_to_blocks.py:125-140)."""
    x = torch.ones(tuple(im_size))
    return fold(unfold(x, block_size, stride, mask), im_size, block_size, stride, mask)
