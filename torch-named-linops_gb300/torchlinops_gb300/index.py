"""Sampling at integer locations: ``index`` and ``index_adjoint``.

Same names, arguments, shapes and errors as the reference functional API
(torchlinops 0.7.4, ``functional/_index/index.py``):

* ``index(vals, idx, deterministic_backward=False)``  <- :17-49
* ``index_adjoint(vals, idx, grid_size)``             <- :75-100

They are the forward and adjoint of the ``Sampling`` linop
(``linops/sampling.py:95-101``), which the NUFFT uses in its "sampling" mode.
The reference's adjoint is ``index_add_`` (``multi_grid``, :141-184): float
atomics on a GPU, so not deterministic there. Here both directions run in the
tlgb CUDA library from a plan (the raveled cell of each sample and the
samples sorted by cell), built once per index set and cached like the
interpolation plans. The adjoint sums each cell's samples in ascending sample
order starting from zero, the order of a sequential ``index_add_``: it is
bit-identical to the reference's CPU result and to itself run to run,
whatever ``deterministic_backward`` says.
"""

from __future__ import annotations

import ctypes
from collections import OrderedDict
from math import prod

import torch
from torch import Tensor
from torch.autograd import Function

from . import _ext
from .interp import remember

__all__ = ["index", "index_adjoint", "IndexPlan", "get_index_plan"]

_DTYPES = {
    torch.float32: 0,
    torch.float64: 1,
    torch.complex64: 2,
    torch.complex128: 3,
    torch.int32: _ext.TLGB_I32,
    torch.int64: _ext.TLGB_I64,
}
# element types the gather copies unchanged (by size)
_RAW = {1: _ext.TLGB_RAW8, 2: _ext.TLGB_RAW16, 4: _ext.TLGB_I32, 8: _ext.TLGB_I64, 16: 3}


def _fwd_dtype(t: Tensor) -> int:
    code = _DTYPES.get(t.dtype)
    if code is not None:
        return code
    return _RAW[t.element_size()]


def _adj_dtype(t: Tensor) -> int:
    code = _DTYPES.get(t.dtype)
    if code is None:
        raise TypeError(f"index_adjoint supports float, complex, int32 and int64 values, got {t.dtype}")
    return code


def _desc(grid_size, npts: int, nbatch: int, dtype: int) -> _ext.IndexDesc:
    if not 1 <= len(grid_size) <= _ext.INDEX_MAX_DIM:
        raise ValueError(f"index: 1 to {_ext.INDEX_MAX_DIM} indexed dimensions, got {len(grid_size)}")
    d = _ext.IndexDesc()
    d.ndim = len(grid_size)
    d.dtype = dtype
    d.nbatch = int(nbatch)
    for i, s in enumerate(grid_size):
        d.grid_size[i] = int(s)
    d.npts = int(npts)
    return d


class IndexPlan:
    """Device-resident plan of one index set on one grid: the cell of every
    sample and the samples sorted by cell, with per-cell offsets."""

    def __init__(self, stacked: Tensor, grid_size: tuple[int, ...]):
        dev = _ext.check_cuda(stacked)
        self.device = dev
        self.grid_size = tuple(int(s) for s in grid_size)
        self.npts = stacked.shape[1]
        d = _desc(self.grid_size, self.npts, 1, 0)
        L = _ext.lib()
        pb, tb = ctypes.c_size_t(0), ctypes.c_size_t(0)
        _ext.check(L.tlgb_index_plan_size(ctypes.byref(d), ctypes.byref(pb), ctypes.byref(tb)), "index plan size")
        self.buffer = torch.empty(max(pb.value, 1), dtype=torch.uint8, device=dev)
        tmp = torch.empty(max(tb.value, 1), dtype=torch.uint8, device=dev)
        self.info = _ext.IndexPlanInfo()
        with torch.cuda.device(dev):
            st = L.tlgb_index_plan_build(ctypes.byref(d), _ext.ptr(stacked), _ext.ptr(self.buffer), pb.value,
                                         _ext.ptr(tmp), tb.value, ctypes.byref(self.info), _ext.stream_ptr(dev))
            if st == _ext.TLGB_ERR_INVALID and b"Out-of-bounds" in L.tlgb_last_error():
                raise IndexError(L.tlgb_last_error().decode())
            _ext.check(st, "index plan")
            self.stream = torch.cuda.current_stream(dev)
            self.ready = torch.cuda.Event()
            self.ready.record(self.stream)
        del tmp

    def use_on_current_stream(self) -> None:
        cur = torch.cuda.current_stream(self.device)
        if cur.cuda_stream != self.stream.cuda_stream and not torch.cuda.is_current_stream_capturing():
            cur.wait_event(self.ready)
            self.buffer.record_stream(cur)


_PLAN_CACHE: "OrderedDict[tuple, tuple]" = OrderedDict()
_PLAN_CACHE_SIZE = 16


def _prepare(idx: tuple, grid_size: tuple[int, ...], broadcast: bool) -> tuple[Tensor, tuple[int, ...], tuple]:
    """Index tensors -> [D, M] int64 (contiguous, on the values' device), the
    sample shape I, and the cache key (the index tensors' identities)."""
    tensors = [torch.as_tensor(i) for i in idx]
    if broadcast:
        tensors = list(torch.broadcast_tensors(*tensors))
    elif len({tuple(t.shape) for t in tensors}) > 1:
        raise RuntimeError("stack expects each tensor to be equal size, but got index tensors of different shapes")
    shape = tuple(tensors[0].shape)
    key = tuple((id(t), t.data_ptr(), tuple(t.shape), tuple(t.stride()), t._version) for t in idx) + (grid_size,)
    return tensors, shape, key


def get_index_plan(idx: tuple, grid_size, broadcast: bool = True) -> tuple[IndexPlan, tuple[int, ...]]:
    """Cached plan for an index set (rebuilt when an index tensor changes in place)."""
    grid_size = tuple(int(s) for s in grid_size)
    tensors, shape, key = _prepare(idx, grid_size, broadcast)
    hit = _PLAN_CACHE.get(key)
    if hit is not None:
        ref, version, plan = hit
        if ref() is idx[0] and version == idx[0]._version:
            _PLAN_CACHE.move_to_end(key)
            plan.use_on_current_stream()
            return plan, shape
        del _PLAN_CACHE[key]
    dev = tensors[0].device
    stacked = torch.stack([t.reshape(-1).to(torch.int64) for t in tensors]).contiguous()
    plan = IndexPlan(stacked, grid_size)
    remember(_PLAN_CACHE, key, idx[0], plan, _PLAN_CACHE_SIZE)
    return plan, shape


def _slices_to_flat(idx: tuple, grid_size: tuple[int, ...], device) -> tuple[Tensor]:
    """An index with slices, as one raveled index tensor over the grid with
    torch's own advanced-indexing semantics (the reference indexes with
    ``vals[(..., *idx)]`` whenever a slice is present, index.py:36-45)."""
    cells = torch.arange(prod(grid_size), device=device).reshape(grid_size)
    return (cells[tuple(i.to(device) if isinstance(i, Tensor) else i for i in idx)],)


def _forward(vals: Tensor, idx: tuple, grid_size: tuple[int, ...], plan: IndexPlan, shape) -> Tensor:
    nb = len(grid_size)
    batch = vals.shape[: vals.ndim - nb]
    nbatch = prod(batch)
    v = vals.resolve_conj().resolve_neg().contiguous()
    out = torch.empty(*batch, *shape, dtype=vals.dtype, device=vals.device)
    d = _desc(plan.grid_size, plan.npts, nbatch, _fwd_dtype(vals))
    with torch.cuda.device(vals.device):
        _ext.check(
            _ext.lib().tlgb_index_forward(ctypes.byref(d), ctypes.byref(plan.info), _ext.ptr(plan.buffer), _ext.ptr(v),
                                          _ext.ptr(out), _ext.stream_ptr(vals.device)),
            "index",
        )
    return out


def _adjoint(vals: Tensor, plan: IndexPlan, shape, grid_size: tuple[int, ...]) -> Tensor:
    ns = len(shape)
    if tuple(vals.shape[vals.ndim - ns:]) != tuple(shape):
        raise ValueError(
            f"x and idx should correspond in last {ns} dimensions but got x: {vals.shape} and idx: {torch.Size(shape)}"
        )
    batch = vals.shape[: vals.ndim - ns]
    nbatch = prod(batch)
    v = vals.resolve_conj().resolve_neg().contiguous()
    out = torch.empty(*batch, *grid_size, dtype=vals.dtype, device=vals.device)
    d = _desc(plan.grid_size, plan.npts, nbatch, _adj_dtype(vals))
    with torch.cuda.device(vals.device):
        _ext.check(
            _ext.lib().tlgb_index_adjoint(ctypes.byref(d), ctypes.byref(plan.info), _ext.ptr(plan.buffer),
                                          _ext.ptr(v), _ext.ptr(out), _ext.stream_ptr(vals.device)),
            "index_adjoint",
        )
    return out


class IndexFn(Function):
    @staticmethod
    def forward(vals, idx, grid_size, plan, shape):
        return _forward(vals, idx, grid_size, plan, shape)

    @staticmethod
    def setup_context(ctx, inputs, output):
        vals, idx, grid_size, plan, shape = inputs
        ctx.plan, ctx.shape, ctx.grid_size = plan, shape, grid_size

    @staticmethod
    def backward(ctx, grad_output):
        g = None
        if ctx.needs_input_grad[0]:
            g = _adjoint(grad_output, ctx.plan, ctx.shape, ctx.grid_size)
        return g, None, None, None, None


class IndexAdjointFn(Function):
    @staticmethod
    def forward(vals, plan, shape, grid_size):
        return _adjoint(vals, plan, shape, grid_size)

    @staticmethod
    def setup_context(ctx, inputs, output):
        vals, plan, shape, grid_size = inputs
        ctx.plan, ctx.shape, ctx.grid_size = plan, shape, grid_size

    @staticmethod
    def backward(ctx, grad_output):
        g = None
        if ctx.needs_input_grad[0]:
            g = _forward(grad_output, None, ctx.grid_size, ctx.plan, ctx.shape)
        return g, None, None, None


def index(vals: Tensor, idx: tuple, deterministic_backward: bool = False) -> Tensor:
    """vals[..., idx]: gather the samples at integer locations (reference
    index.py:17). Negative indices count from the end. The backward pass is
    the deterministic ``index_adjoint`` either way."""
    if len(vals.shape) < len(idx):
        raise ValueError(
            f"Input value with shape {vals.shape} cannot be indexed with index tensors of length {len(idx)}"
        )
    _ext.check_cuda(vals)
    grid_size = tuple(vals.shape[vals.ndim - len(idx):])
    if any(isinstance(i, slice) for i in idx):
        flat = _slices_to_flat(idx, grid_size, vals.device)
        plan, shape = get_index_plan(flat, (prod(grid_size),))
        v = vals.reshape(*vals.shape[: vals.ndim - len(idx)], prod(grid_size))
        return IndexFn.apply(v, flat, (prod(grid_size),), plan, shape)
    idx = tuple(i.to(vals.device) for i in idx)
    plan, shape = get_index_plan(idx, grid_size, broadcast=True)
    return IndexFn.apply(vals, idx, grid_size, plan, shape)


def index_adjoint(vals: Tensor, idx: tuple, grid_size: tuple[int, ...]) -> Tensor:
    """Scatter-add the samples into a zero grid (reference index.py:75):
    out[..., c] = sum of vals[..., m] over the samples m at cell c."""
    grid_size = tuple(int(s) for s in grid_size)
    _ext.check_cuda(vals)
    idx = tuple(torch.as_tensor(i).to(vals.device) for i in idx)
    if len(idx) != len(grid_size):
        raise ValueError(f"final_size should be of dimension {len(idx)} but got {grid_size}")
    plan, shape = get_index_plan(idx, grid_size, broadcast=False)
    return IndexAdjointFn.apply(vals, plan, shape, grid_size)
