"""Circular padding of the trailing dims and its adjoint.

Same names, arguments, shapes and errors as the reference
(torchlinops 0.7.4, ``functional/_interp/_circ_pad.py``):

* ``circular_pad(t, padding)``          <- :10-83
* ``circular_pad_adjoint(t, padding)``  <- :119-134

``padding`` follows ``torch.nn.functional.pad``: pairs (left, right) from the
last dim backwards, one pair per padded dim. The ``Convolution`` linop pads
with it in its circular mode (``linops/convolution.py:120-130,148-150``).
The reference pads three dims at a time with torch's circular ``F.pad`` and
forms the adjoint by autograd through it; here each direction is one CUDA
pass over any number of dims (up to 8), and the adjoint sums the copies of
each element in a fixed order. Both are autograd functions whose backward is
the other.
"""

from __future__ import annotations

import ctypes
from math import prod

import torch
from torch import Tensor
from torch.autograd import Function

from . import _ext

__all__ = ["circular_pad", "circular_pad_adjoint"]

_ADJ_DTYPES = {
    torch.float32: 0,
    torch.float64: 1,
    torch.complex64: 2,
    torch.complex128: 3,
    torch.int32: _ext.TLGB_I32,
    torch.int64: _ext.TLGB_I64,
}
_RAW = {1: _ext.TLGB_RAW8, 2: _ext.TLGB_RAW16, 4: _ext.TLGB_I32, 8: _ext.TLGB_I64, 16: 3}


def _pairs(padding) -> list[tuple[int, int]]:
    """padding in F.pad order -> [(lo, hi)] for dims leading to trailing."""
    if isinstance(padding, int):
        raise TypeError("circular_pad takes padding as a tuple in torch.nn.functional.pad order, not an int")
    padding = tuple(int(p) for p in padding)
    if len(padding) % 2:
        raise ValueError(f"Padding must have even length but got {len(padding)}: {padding}")
    pairs = [(padding[2 * i], padding[2 * i + 1]) for i in range(len(padding) // 2)]
    return pairs[::-1]


def _desc(shape_unpadded, pairs, dtype_code) -> _ext.CircPadDesc:
    nd = len(pairs)
    if nd > _ext.CIRCPAD_MAX_DIM:
        raise NotImplementedError(f"circular padding of more than {_ext.CIRCPAD_MAX_DIM} dims")
    if nd > len(shape_unpadded):
        raise ValueError(f"padding {nd} dims of a tensor with {len(shape_unpadded)} dims")
    d = _ext.CircPadDesc()
    d.ndim = nd
    d.dtype = dtype_code
    d.nbatch = prod(shape_unpadded[: len(shape_unpadded) - nd])
    for e, (lo, hi) in enumerate(pairs):
        d.size[e] = int(shape_unpadded[len(shape_unpadded) - nd + e])
        d.pad_lo[e] = lo
        d.pad_hi[e] = hi
    return d


def _pad(t: Tensor, pairs) -> Tensor:
    dev = _ext.check_cuda(t)
    nd = len(pairs)
    lead = t.shape[: t.ndim - nd]
    out_shape = (*lead, *(s + lo + hi for s, (lo, hi) in zip(t.shape[t.ndim - nd:], pairs)))
    code = _ADJ_DTYPES[t.dtype] if t.dtype in _ADJ_DTYPES else _RAW[t.element_size()]
    d = _desc(tuple(t.shape), pairs, code)
    src = t.resolve_conj().resolve_neg().contiguous()
    out = torch.empty(out_shape, dtype=t.dtype, device=dev)
    with torch.cuda.device(dev):
        _ext.check(_ext.lib().tlgb_circular_pad(ctypes.byref(d), _ext.ptr(src), _ext.ptr(out), _ext.stream_ptr(dev)),
                   "circular_pad")
    return out


def _pad_adjoint(t: Tensor, pairs) -> Tensor:
    dev = _ext.check_cuda(t)
    nd = len(pairs)
    lead = t.shape[: t.ndim - nd]
    in_shape = (*lead, *(s - lo - hi for s, (lo, hi) in zip(t.shape[t.ndim - nd:], pairs)))
    code = _ADJ_DTYPES.get(t.dtype)
    if code is None:
        raise TypeError(f"circular_pad_adjoint supports float, complex, int32 and int64 tensors, got {t.dtype}")
    d = _desc(in_shape, pairs, code)
    src = t.resolve_conj().resolve_neg().contiguous()
    out = torch.empty(in_shape, dtype=t.dtype, device=dev)
    with torch.cuda.device(dev):
        _ext.check(
            _ext.lib().tlgb_circular_pad_adjoint(ctypes.byref(d), _ext.ptr(src), _ext.ptr(out), _ext.stream_ptr(dev)),
            "circular_pad_adjoint",
        )
    return out


class CircularPadFn(Function):
    @staticmethod
    def forward(t, pairs):
        return _pad(t, pairs)

    @staticmethod
    def setup_context(ctx, inputs, output):
        ctx.pairs = inputs[1]

    @staticmethod
    def backward(ctx, g):
        return (_pad_adjoint(g, ctx.pairs) if ctx.needs_input_grad[0] else None), None


class CircularPadAdjointFn(Function):
    @staticmethod
    def forward(t, pairs):
        return _pad_adjoint(t, pairs)

    @staticmethod
    def setup_context(ctx, inputs, output):
        ctx.pairs = inputs[1]

    @staticmethod
    def backward(ctx, g):
        return (_pad(g, ctx.pairs) if ctx.needs_input_grad[0] else None), None


def circular_pad(t: Tensor, padding) -> Tensor:
    """Circular padding of the last len(padding)//2 dims (reference _circ_pad.py:10)."""
    return CircularPadFn.apply(t, _pairs(padding))


def circular_pad_adjoint(t: Tensor, padding) -> Tensor:
    """Adjoint of ``circular_pad``: each element gathers the sum of its copies
    (reference _circ_pad.py:119)."""
    return CircularPadAdjointFn.apply(t, _pairs(padding))
