"""ArrayToBlocks / BlocksToArray (unfold / fold) and their autograd wrappers.

Same names, arguments, shapes and errors as the reference functional API
(torchlinops 0.7.4):

* ``get_nblocks``       <- functional/_unfold/nblocks.py:6-33
* ``unfold``            <- functional/_unfold/unfold.py:31-131
* ``fold``              <- functional/_unfold/fold.py:32-118
* ``array_to_blocks``   <- functional/_unfold/array_to_blocks.py:59-67
* ``blocks_to_array``   <- functional/_unfold/array_to_blocks.py:113-122
* ``get_norm_weights``  <- functional/_unfold/array_to_blocks.py:125-140

The copies and sums run in the tlgb CUDA library. A mask is fused into the
kernels (the reference unfolds everything and then indexes ``y[..., mask]``).
"""

from __future__ import annotations

import ctypes
from math import prod
from typing import Optional

import torch
from torch import Tensor
from torch.autograd import Function

from . import _ext

__all__ = [
    "get_nblocks",
    "unfold",
    "fold",
    "array_to_blocks",
    "blocks_to_array",
    "get_norm_weights",
]


def get_nblocks(im_size, block_size, block_stride=None) -> tuple[int, ...]:
    """Number of valid (possibly overlapping) blocks per dimension.

    >>> get_nblocks((5, 5), (3, 3), (2, 2))
    (2, 2)
    """
    assert len(im_size) == len(block_size), f"im_size {im_size} and block_size {block_size} don't match"
    block_stride = block_stride if block_stride is not None else (1,) * len(block_size)
    return tuple((im - bl) // st + 1 for im, bl, st in zip(im_size, block_size, block_stride))


def _dtype_code(t: Tensor) -> int:
    code = _ext.BLOCK_DTYPES.get(t.dtype)
    if code is None:
        raise TypeError(f"unfold / fold support float32, float64, complex64, complex128; got {t.dtype}")
    return code


def _mask_tables(mask: Tensor, block_size, device):
    m = mask.detach().to("cpu", torch.bool)
    if tuple(m.shape) != tuple(block_size):
        raise ValueError(f"mask shape {tuple(m.shape)} must equal the block size {tuple(block_size)}")
    flat = m.reshape(-1)
    idx = torch.nonzero(flat).reshape(-1).to(torch.int32)
    inv = torch.full((flat.numel(),), -1, dtype=torch.int32)
    inv[idx.long()] = torch.arange(idx.numel(), dtype=torch.int32)
    return idx.to(device, non_blocking=True), inv.to(device, non_blocking=True), int(idx.numel())


def _desc(ndim, dtype_code, nbatch, im_size, block_size, stride, nnz, idx=None, inv=None) -> _ext.BlocksDesc:
    d = _ext.BlocksDesc()
    d.ndim = ndim
    d.dtype = dtype_code
    d.nbatch = int(nbatch)
    for i in range(ndim):
        d.im_size[i] = int(im_size[i])
        d.block[i] = int(block_size[i])
        d.stride[i] = int(stride[i])
    d.nnz = int(nnz)
    d.mask_idx = idx.data_ptr() if idx is not None else None
    d.mask_inv = inv.data_ptr() if inv is not None else None
    return d


def _prep(block_size, stride, im_size):
    ndim = len(block_size)
    if ndim not in (1, 2, 3):
        raise ValueError(f"block dims must be 1, 2 or 3, got {ndim}")
    stride = tuple(stride) if stride is not None else (1,) * ndim
    nblocks = get_nblocks(tuple(im_size), tuple(block_size), stride)
    if any(b <= 0 for b in nblocks):
        raise ValueError(
            f"Found 0 in nblocks: {nblocks} with im_size {tuple(im_size)}, block_size {tuple(block_size)} and stride {stride} - make sure there is at least one block in each direction."
        )
    return ndim, stride, nblocks


def unfold(
    x: Tensor,
    block_size: tuple,
    stride: Optional[tuple] = None,
    mask: Optional[Tensor] = None,
    output: Optional[Tensor] = None,
) -> Tensor:
    """[B..., *im_size] -> [B..., *nblocks, *block_size] (or [..., nnz] with a mask)."""
    dev = _ext.check_cuda(x)
    ndim = len(block_size)
    im_size = tuple(x.shape[-ndim:])
    ndim, stride, nblocks = _prep(block_size, stride, im_size)
    if output is not None and output.dtype != x.dtype:
        raise ValueError(f"Output and input dtypes must match but got output {output.dtype} != input {x.dtype}")
    batch_shape = x.shape[:-ndim]
    nbatch = prod(batch_shape)
    code = _dtype_code(x)
    xc = x.resolve_conj().resolve_neg().contiguous()
    L = _ext.lib()
    if mask is not None and output is None:
        idx, inv, nnz = _mask_tables(mask, block_size, dev)
        y = torch.empty(*batch_shape, *nblocks, nnz, dtype=x.dtype, device=dev)
        d = _desc(ndim, code, nbatch, im_size, block_size, stride, nnz, idx, inv)
        with torch.cuda.device(dev):
            _ext.check(L.tlgb_unfold(ctypes.byref(d), _ext.ptr(xc), _ext.ptr(y), _ext.stream_ptr(dev)), "unfold")
        return y
    full = (*batch_shape, *nblocks, *block_size)
    if output is not None:
        if output.numel() != prod(full) or not output.is_contiguous():
            raise ValueError(f"output buffer must be contiguous with {prod(full)} elements")
        y = output.view(full)
    else:
        y = torch.empty(full, dtype=x.dtype, device=dev)
    d = _desc(ndim, code, nbatch, im_size, block_size, stride, prod(block_size))
    with torch.cuda.device(dev):
        _ext.check(L.tlgb_unfold(ctypes.byref(d), _ext.ptr(xc), _ext.ptr(y), _ext.stream_ptr(dev)), "unfold")
    if mask is not None:  # reference order: full unfold into the buffer, then index
        y = y[..., mask.to(dev)]
    return y


def fold(
    x: Tensor,
    im_size: tuple,
    block_size: tuple,
    stride: tuple,
    mask: Optional[Tensor] = None,
    output: Optional[Tensor] = None,
) -> Tensor:
    """[B..., *nblocks, *block_size] (or [..., nnz]) -> [B..., *im_size], overlaps summed."""
    dev = _ext.check_cuda(x)
    ndim, stride, nblocks = _prep(block_size, stride, im_size)
    if output is not None and output.dtype != x.dtype:
        raise ValueError(f"Output and input dtypes must match but got output {output.dtype} != input {x.dtype}")
    code = _dtype_code(x)
    L = _ext.lib()
    idx = inv = None
    if mask is not None:
        idx, inv, nnz = _mask_tables(mask, block_size, dev)
        tail = (*nblocks, nnz)
        nd_tail = ndim + 1
    else:
        nnz = prod(block_size)
        tail = (*nblocks, *block_size)
        nd_tail = 2 * ndim
    if tuple(x.shape[x.ndim - nd_tail:]) != tuple(tail):
        raise RuntimeError(f"Fold expected input with full size {tuple(tail)} but got {tuple(x.shape)}")
    batch_shape = x.shape[: x.ndim - nd_tail]
    nbatch = prod(batch_shape)
    out_shape = (*batch_shape, *im_size)
    if output is not None:
        if output.numel() != prod(out_shape) or not output.is_contiguous():
            raise ValueError(f"output buffer must be contiguous with {prod(out_shape)} elements")
        y = output.view(out_shape)
    else:
        y = torch.empty(out_shape, dtype=x.dtype, device=dev)
    xc = x.resolve_conj().resolve_neg().contiguous()
    d = _desc(ndim, code, nbatch, im_size, block_size, stride, nnz, idx, inv)
    with torch.cuda.device(dev):
        _ext.check(L.tlgb_fold(ctypes.byref(d), _ext.ptr(xc), _ext.ptr(y), _ext.stream_ptr(dev)), "fold")
    return y


class ArrayToBlocksFn(Function):
    """unfold with autograd (reference array_to_blocks.py:16-56)."""

    @staticmethod
    def forward(input, block_shape, stride, mask, out):
        output = unfold(input, block_shape, stride, mask, out)
        output.requires_grad_(input.requires_grad)
        return output

    @staticmethod
    def setup_context(ctx, inputs, output):
        input, block_shape, stride, mask, out = inputs
        ctx.im_size = tuple(input.shape[-len(block_shape):])
        ctx.block_shape = block_shape
        ctx.stride = stride
        ctx.save_for_backward(mask)

    @staticmethod
    def backward(ctx, grad_output):
        grad_input = None
        if ctx.needs_input_grad[0]:
            (mask,) = ctx.saved_tensors
            grad_input = fold(grad_output, ctx.im_size, ctx.block_shape, ctx.stride, mask)
        return grad_input, None, None, None, None


class BlocksToArrayFn(Function):
    """fold with autograd (reference array_to_blocks.py:70-110)."""

    @staticmethod
    def forward(input, im_size, block_shape, stride, mask, out):
        output = fold(input, im_size, block_shape, stride, mask, out)
        output.requires_grad_(input.requires_grad)
        return output

    @staticmethod
    def setup_context(ctx, inputs, output):
        input, im_size, block_shape, stride, mask, out = inputs
        ctx.block_shape = block_shape
        ctx.stride = stride
        ctx.save_for_backward(mask)

    @staticmethod
    def backward(ctx, grad_output):
        grad_input = None
        if ctx.needs_input_grad[0]:
            (mask,) = ctx.saved_tensors
            grad_input = unfold(grad_output, ctx.block_shape, ctx.stride, mask)
        return grad_input, None, None, None, None, None


def array_to_blocks(input, block_shape, stride=None, mask=None, out=None):
    return ArrayToBlocksFn.apply(input, block_shape, stride, mask, out)


def blocks_to_array(input, im_size, block_shape, stride=None, mask=None, out=None):
    return BlocksToArrayFn.apply(input, im_size, block_shape, stride, mask, out)


def get_norm_weights(im_size, block_shape, stride=None, mask=None, device="cpu"):
    """fold(unfold(ones)): 1/weights * fold(unfold(x)) == x where weights > 0
    (reference functional/_unfold/array_to_blocks.py:125-140, same arguments
    and default device). The unfold and fold run on the CUDA kernels: on the
    current CUDA device when ``device`` is not a CUDA device, and the weights
    are returned on ``device``."""
    device = torch.device(device)
    work = device if device.type == "cuda" else torch.device("cuda", torch.cuda.current_device())
    if mask is not None:
        mask = mask.to(work)
    x = torch.ones(tuple(im_size), device=work)
    w = blocks_to_array(array_to_blocks(x, block_shape, stride, mask), im_size, block_shape, stride, mask)
    return w.to(device)
