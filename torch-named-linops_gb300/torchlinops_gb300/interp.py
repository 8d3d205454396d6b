"""Interpolation (ungrid), gridding (adjoint) and their autograd wrappers.

Same names, arguments, shapes and errors as the reference functional API
(torchlinops 0.7.4):

* ``ungrid``               <- functional/_interp/ungrid.py:37-67
* ``grid``                 <- functional/_interp/grid.py:37-72
* ``interpolate``          <- functional/_interp/interp.py:73-114
* ``interpolate_adjoint``  <- functional/_interp/interp.py:184-236

The work runs in the tlgb CUDA library. A *plan* (points binned by output
tile) is built once per trajectory and cached: it is keyed on the ``locs``
tensor object and its version counter, so an in-place change of ``locs``
(which bumps the version) rebuilds it. The gradient with respect to ``locs``
(the trajectory) is computed by a hand-written kernel; the reference returns
``None`` there (interp.py:46-70).
"""

from __future__ import annotations

import ctypes
import math
import weakref
from collections import OrderedDict
from math import prod
from typing import Literal

import torch
from torch import Tensor
from torch.autograd import Function

from . import _ext

__all__ = [
    "ungrid",
    "grid",
    "interpolate",
    "interpolate_adjoint",
    "InterpolatePlan",
    "get_plan",
    "clear_plan_cache",
    "kaiser_bessel_beta",
]

# Maximum kernel width per dimension handled by the CUDA kernels
MAX_WIDTH_1D_2D = 15.0
MAX_WIDTH_3D = 8.0


def kaiser_bessel_beta(width: float, oversamp: float) -> float:
    """Beta of the reference NUFFT (linops/nufft.py:337-346)."""
    return math.pi * (((width / oversamp) * (oversamp - 0.5)) ** 2 - 0.8) ** 0.5


def _apply_default_kernel_params(kernel: str, kernel_params: dict | None) -> dict:
    # reference kernels.py:245-252
    kernel_params = {} if kernel_params is None else dict(kernel_params)
    if kernel == "kaiser_bessel":
        kernel_params["beta"] = kernel_params.get("beta", 1.0)
    elif kernel == "spline":
        pass
    else:
        raise ValueError(f"Unrecognized kernel type: {kernel}")
    return kernel_params


def _width_tuple(width, ndim: int) -> tuple[float, ...]:
    # reference prep_ungrid_shapes / prep_grid_shapes (ungrid.py:600-606)
    if isinstance(width, (float, int)):
        return (float(width),) * ndim
    width = tuple(float(w) for w in width)
    if len(width) != ndim:
        raise ValueError(
            f"If width specified as tuple it must be same length as grid size but got len(width) = {len(width)} and len(grid_size) = {ndim}"
        )
    return width


def _desc(ndim, grid_size, width, kernel, norm, pad_mode, beta, is_complex, nbatch, npts) -> _ext.InterpDesc:
    if kernel not in _ext.KERNELS:
        raise ValueError(f"Unrecognized kernel type: {kernel}")
    if pad_mode not in _ext.PAD_MODES:
        raise ValueError(f"Unrecognized padding mode: {pad_mode}")
    if norm not in (1, 2):
        raise ValueError(f"Unexpected norm: {norm}.")
    d = _ext.InterpDesc()
    d.ndim = ndim
    d.kernel = _ext.KERNELS[kernel]
    d.norm = norm
    d.pad_mode = _ext.PAD_MODES[pad_mode]
    d.is_complex = 1 if is_complex else 0
    for i in range(ndim):
        d.grid_size[i] = int(grid_size[i])
        d.width[i] = float(width[i])
    d.beta = float(beta)
    d.nbatch = int(nbatch)
    d.npts = int(npts)
    return d


class InterpolatePlan:
    """Device-resident binning of one trajectory for one grid / kernel."""

    def __init__(self, locs: Tensor, grid_size, width, kernel: str, pad_mode: str, beta: float = 1.0, norm: int = 1):
        dev = _ext.check_cuda(locs)
        self.device = dev
        ndim = locs.shape[-1]
        self.ndim = ndim
        self.grid_size = tuple(int(g) for g in grid_size)
        self.width = _width_tuple(width, ndim)
        self.kernel = kernel
        self.pad_mode = pad_mode
        self.npts = prod(locs.shape[:-1])
        locs_c = locs.detach().reshape(-1, ndim).to(torch.float32).contiguous()
        self.beta, self.norm = float(beta), int(norm)
        # 2D and 3D plans also hold each point's tap weights, so they are built for one (kernel, norm, beta)
        d = _desc(ndim, self.grid_size, self.width, kernel, self.norm, pad_mode, self.beta, False, 1, self.npts)
        L = _ext.lib()
        pb, tb = ctypes.c_size_t(0), ctypes.c_size_t(0)
        _ext.check(L.tlgb_interp_plan_size(ctypes.byref(d), ctypes.byref(pb), ctypes.byref(tb)), "plan size")
        self.buffer = torch.empty(max(pb.value, 1), dtype=torch.uint8, device=dev)
        tmp = torch.empty(max(tb.value, 1), dtype=torch.uint8, device=dev)
        self.info = _ext.PlanInfo()
        with torch.cuda.device(dev):
            st = _ext.stream_ptr(dev)
            _ext.check(
                L.tlgb_interp_plan_build(
                    ctypes.byref(d), _ext.ptr(locs_c), _ext.ptr(self.buffer), pb.value, _ext.ptr(tmp), tb.value,
                    ctypes.byref(self.info), st,
                ),
                "interpolation plan",
            )
            # the build's last kernels are still in flight on this stream
            self.stream = torch.cuda.current_stream(dev)
            self.ready = torch.cuda.Event()
            self.ready.record(self.stream)
        del tmp

    def use_on_current_stream(self) -> None:
        """Plans are cached across streams: another stream waits for the
        build (no host synchronisation) and keeps the plan's memory from
        being reused while its own work may still read it. Under stream
        capture nothing is added (plans are built before capture: a build
        synchronises its stream)."""
        cur = torch.cuda.current_stream(self.device)
        if cur.cuda_stream != self.stream.cuda_stream and not torch.cuda.is_current_stream_capturing():
            cur.wait_event(self.ready)
            self.buffer.record_stream(cur)

    @property
    def n_entries(self) -> int:
        return int(self.info.n_entries)


_PLAN_CACHE: "OrderedDict[tuple, tuple]" = OrderedDict()
_PLAN_CACHE_SIZE = 16


def clear_plan_cache() -> None:
    _PLAN_CACHE.clear()


def remember(cache: "OrderedDict[tuple, tuple]", key: tuple, locs: Tensor, value, size: int) -> None:
    """cache[key] = (weak reference to locs, locs' version, value), most
    recent last. The entry is dropped when locs is freed (a plan holds device
    memory that a dead trajectory could never use again) and the oldest
    entries beyond ``size`` are evicted."""

    def drop(ref, cache=cache, key=key):
        hit = cache.get(key)
        if hit is not None and hit[0] is ref:
            del cache[key]

    cache[key] = (weakref.ref(locs, drop), locs._version, value)
    while len(cache) > size:
        cache.popitem(last=False)


def get_plan(locs: Tensor, grid_size, width, kernel: str, pad_mode: str, beta: float = 1.0,
             norm: int = 1) -> InterpolatePlan:
    """Cached plan for ``locs``: rebuilt when ``locs`` changes in place."""
    ndim = locs.shape[-1]
    key = (
        id(locs),
        locs.data_ptr(),
        tuple(locs.shape),
        locs.dtype,
        tuple(int(g) for g in grid_size),
        _width_tuple(width, ndim),
        kernel,
        pad_mode,
        float(beta),
        int(norm),
    )
    hit = _PLAN_CACHE.get(key)
    if hit is not None:
        ref, version, plan = hit
        if ref() is locs and version == locs._version:
            _PLAN_CACHE.move_to_end(key)
            plan.use_on_current_stream()
            return plan
        del _PLAN_CACHE[key]
    plan = InterpolatePlan(locs, grid_size, width, kernel, pad_mode, beta, norm)
    remember(_PLAN_CACHE, key, locs, plan, _PLAN_CACHE_SIZE)
    return plan


# batch entries per C-ABI call (TLGB_INTERP_MAX_BATCH in include/tlgb.h)
MAX_BATCH = 524280


def _batch_chunks(nbatch: int) -> list[tuple[int, int]]:
    """[begin, end) ranges of at most MAX_BATCH batch entries (one empty range
    for an empty batch); batch entries are independent."""
    return [(b, min(b + MAX_BATCH, nbatch)) for b in range(0, nbatch, MAX_BATCH)] or [(0, 0)]


def _check_values(vals: Tensor) -> bool:
    if vals.dtype == torch.complex64:
        return True
    if vals.dtype == torch.float32:
        return False
    raise TypeError(f"interpolation supports float32 and complex64 values, got {vals.dtype}")


def _as_f32_view(t: Tensor, is_complex: bool) -> Tensor:
    # autograd may hand over lazily conjugated / negated views: materialise them
    t = t.resolve_conj().resolve_neg().contiguous()
    return torch.view_as_real(t) if is_complex else t


def _locs_f32(locs: Tensor) -> Tensor:
    return locs.detach().to(torch.float32).contiguous()


def ungrid(
    vals: Tensor,
    locs: Tensor,
    width: float | tuple[float, ...],
    kernel: str = "kaiser_bessel",
    norm: int = 1,
    pad_mode: Literal["zero", "circular"] = "circular",
    kernel_params: dict = None,
) -> Tensor:
    """Interpolate from on-grid values to off-grid locations (reference ungrid.py:37)."""
    kernel_params = _apply_default_kernel_params(kernel, kernel_params)
    dev = _ext.check_cuda(vals, locs)
    ndim = locs.shape[-1]
    if ndim not in (1, 2, 3):
        raise ValueError(f"locs must have 1, 2 or 3 coordinates, got {ndim}")
    grid_size = tuple(vals.shape[-ndim:])
    batch_shape = vals.shape[:-ndim]
    nbatch = prod(batch_shape)
    locs_batch_shape = locs.shape[:-1]
    npts = prod(locs_batch_shape)
    width = _width_tuple(width, ndim)
    is_complex = _check_values(vals)
    beta = kernel_params["beta"] if kernel == "kaiser_bessel" else 1.0
    plan = get_plan(locs, grid_size, width, kernel, pad_mode, beta, norm)
    out = torch.empty(nbatch, npts, dtype=vals.dtype, device=dev)
    d = _desc(ndim, grid_size, width, kernel, norm, pad_mode, beta, is_complex, nbatch, npts)
    v = _as_f32_view(vals, is_complex)
    if nbatch > MAX_BATCH:
        v = v.reshape(nbatch, -1)
    lc = _locs_f32(locs)
    with torch.cuda.device(dev):
        for b0, b1 in _batch_chunks(nbatch):
            d.nbatch = b1 - b0
            _ext.check(
                _ext.lib().tlgb_interp_forward(
                    ctypes.byref(d), ctypes.byref(plan.info), _ext.ptr(plan.buffer), _ext.ptr(lc),
                    _ext.ptr(v[b0:b1] if nbatch > MAX_BATCH else v), _ext.ptr(out[b0:b1]), _ext.stream_ptr(dev),
                ),
                "ungrid",
            )
    return out.reshape(*batch_shape, *locs_batch_shape)


def grid(
    vals: Tensor,
    locs: Tensor,
    grid_size: tuple[int, ...],
    width: float | tuple[float, ...],
    kernel: str = "kaiser_bessel",
    norm: int = 1,
    pad_mode: Literal["zero", "circular"] = "circular",
    kernel_params: dict = None,
) -> Tensor:
    """Interpolate from off-grid values to on-grid locations (reference grid.py:37).

    Deterministic: the sum over points is taken in a fixed order, so repeated
    calls return bit-identical results.
    """
    kernel_params = _apply_default_kernel_params(kernel, kernel_params)
    dev = _ext.check_cuda(vals, locs)
    grid_size = tuple(int(g) for g in grid_size)
    ndim = len(grid_size)
    if locs.shape[-1] != ndim:
        raise ValueError(
            f"Expected last dim of locs: to equal ndim but got locs.shape[-1] {locs.shape[-1]} != ndim {ndim}"
        )
    if ndim not in (1, 2, 3):
        raise ValueError(f"grid must have 1, 2 or 3 dims, got {ndim}")
    locs_batch_shape = locs.shape[:-1]
    npts = prod(locs_batch_shape)
    nl = len(locs_batch_shape)
    if tuple(vals.shape[vals.ndim - nl:]) != tuple(locs_batch_shape):
        raise ValueError(f"vals shape {tuple(vals.shape)} does not end with the locs batch shape {tuple(locs_batch_shape)}")
    batch_shape = vals.shape[: vals.ndim - nl]
    nbatch = prod(batch_shape)
    width = _width_tuple(width, ndim)
    is_complex = _check_values(vals)
    beta = kernel_params["beta"] if kernel == "kaiser_bessel" else 1.0
    plan = get_plan(locs, grid_size, width, kernel, pad_mode, beta, norm)
    # the first batch range is the largest: its scratch serves every range
    d = _desc(ndim, grid_size, width, kernel, norm, pad_mode, beta, is_complex, min(nbatch, MAX_BATCH), npts)
    L = _ext.lib()
    sb = ctypes.c_size_t(0)
    _ext.check(L.tlgb_interp_adjoint_scratch_size(ctypes.byref(d), ctypes.byref(plan.info), ctypes.byref(sb)), "grid")
    out = torch.empty(nbatch, *grid_size, dtype=vals.dtype, device=dev)
    scratch = torch.empty(max(sb.value, 1), dtype=torch.uint8, device=dev)
    v = _as_f32_view(vals, is_complex)
    if nbatch > MAX_BATCH:
        v = v.reshape(nbatch, -1)
    lc = _locs_f32(locs)
    with torch.cuda.device(dev):
        for b0, b1 in _batch_chunks(nbatch):
            d.nbatch = b1 - b0
            _ext.check(
                L.tlgb_interp_adjoint(
                    ctypes.byref(d), ctypes.byref(plan.info), _ext.ptr(plan.buffer), _ext.ptr(lc),
                    _ext.ptr(v[b0:b1] if nbatch > MAX_BATCH else v), _ext.ptr(out[b0:b1]), _ext.ptr(scratch),
                    sb.value, _ext.stream_ptr(dev),
                ),
                "grid",
            )
    return out.reshape(*batch_shape, *grid_size)


def _grad_locs(gridvals: Tensor, a: Tensor, locs: Tensor, width, kernel, norm, pad_mode, kernel_params) -> Tensor:
    """sum_b Re(conj(a[b,p]) * sum_taps dw/dx * gridvals[b, tap]), shape of locs."""
    kernel_params = _apply_default_kernel_params(kernel, kernel_params)
    dev = _ext.check_cuda(gridvals, a, locs)
    ndim = locs.shape[-1]
    grid_size = tuple(gridvals.shape[-ndim:])
    nbatch = prod(gridvals.shape[:-ndim])
    npts = prod(locs.shape[:-1])
    width = _width_tuple(width, ndim)
    is_complex = gridvals.is_complex()
    if a.is_complex() != is_complex:
        a = a.to(gridvals.dtype)
    beta = kernel_params["beta"] if kernel == "kaiser_bessel" else 1.0
    plan = get_plan(locs, grid_size, width, kernel, pad_mode, beta, norm)
    d = _desc(ndim, grid_size, width, kernel, norm, pad_mode, beta, is_complex, min(nbatch, MAX_BATCH), npts)
    g = _as_f32_view(gridvals, is_complex)
    av = _as_f32_view(a.reshape(nbatch, npts), is_complex)
    chunks = _batch_chunks(nbatch)
    if len(chunks) > 1:
        g = g.reshape(nbatch, -1)
    out = torch.empty(npts, ndim, dtype=torch.float32, device=dev)
    part = torch.empty_like(out) if len(chunks) > 1 else out
    lc = _locs_f32(locs)
    L = _ext.lib()
    sb = ctypes.c_size_t(0)
    _ext.check(L.tlgb_interp_grad_scratch_size(ctypes.byref(d), ctypes.byref(plan.info), ctypes.byref(sb)),
               "trajectory gradient")
    scratch = torch.empty(max(sb.value, 1), dtype=torch.uint8, device=dev)
    with torch.cuda.device(dev):
        # the gradient sums over the batch: one call per batch range, the
        # ranges' results added in order
        for i, (b0, b1) in enumerate(chunks):
            d.nbatch = b1 - b0
            _ext.check(
                L.tlgb_interp_grad_locs(
                    ctypes.byref(d), ctypes.byref(plan.info), _ext.ptr(plan.buffer), _ext.ptr(lc),
                    _ext.ptr(g[b0:b1] if len(chunks) > 1 else g), _ext.ptr(av[b0:b1]),
                    _ext.ptr(out if i == 0 else part), _ext.ptr(scratch), sb.value, _ext.stream_ptr(dev),
                ),
                "trajectory gradient",
            )
            if i > 0:
                out += part
    return out.reshape(locs.shape).to(locs.dtype)


class InterpolateFn(Function):
    """ungrid with autograd (reference interp.py:13-70); adds d/dlocs."""

    @staticmethod
    def forward(vals, locs, width, kernel, norm, pad_mode, kernel_params):
        out = ungrid(vals, locs, width, kernel, norm, pad_mode, kernel_params)
        out.requires_grad_(vals.requires_grad or locs.requires_grad)
        return out

    @staticmethod
    def setup_context(ctx, inputs, output):
        vals, locs, width, kernel, norm, pad_mode, kernel_params = inputs
        ndim = locs.shape[-1]
        ctx.grid_size = tuple(vals.shape[-ndim:])
        ctx.params = (width, kernel, norm, pad_mode, kernel_params)
        # the grid image is needed only for the trajectory gradient
        ctx.save_for_backward(locs, vals if locs.requires_grad else None)

    @staticmethod
    def backward(ctx, grad_output):
        locs, vals = ctx.saved_tensors
        width, kernel, norm, pad_mode, kernel_params = ctx.params
        grad_vals = grad_locs = None
        if ctx.needs_input_grad[0]:
            grad_vals = grid(grad_output, locs, ctx.grid_size, width, kernel, norm, pad_mode, kernel_params)
        if ctx.needs_input_grad[1]:
            grad_locs = _grad_locs(vals, grad_output, locs, width, kernel, norm, pad_mode, kernel_params)
        return grad_vals, grad_locs, None, None, None, None, None


class InterpolateAdjointFn(Function):
    """grid with autograd (reference interp.py:117-181); adds d/dlocs."""

    @staticmethod
    def forward(vals, locs, grid_size, width, kernel, norm, pad_mode, kernel_params):
        out = grid(vals, locs, grid_size, width, kernel, norm, pad_mode, kernel_params)
        out.requires_grad_(vals.requires_grad or locs.requires_grad)
        return out

    @staticmethod
    def setup_context(ctx, inputs, output):
        vals, locs, grid_size, width, kernel, norm, pad_mode, kernel_params = inputs
        ctx.params = (width, kernel, norm, pad_mode, kernel_params)
        ctx.save_for_backward(locs, vals if locs.requires_grad else None)

    @staticmethod
    def backward(ctx, grad_output):
        locs, vals = ctx.saved_tensors
        width, kernel, norm, pad_mode, kernel_params = ctx.params
        grad_vals = grad_locs = None
        if ctx.needs_input_grad[0]:
            grad_vals = ungrid(grad_output, locs, width, kernel, norm, pad_mode, kernel_params)
        if ctx.needs_input_grad[1]:
            grad_locs = _grad_locs(grad_output, vals, locs, width, kernel, norm, pad_mode, kernel_params)
        return grad_vals, grad_locs, None, None, None, None, None, None


def interpolate(
    vals: Tensor,
    locs: Tensor,
    width: float | tuple[float, ...],
    kernel="kaiser_bessel",
    norm: int = 1,
    pad_mode: str = "circular",
    kernel_params: dict = None,
) -> Tensor:
    """Interpolate from a regular grid to scattered locations (reference interp.py:73)."""
    return InterpolateFn.apply(vals, locs, width, kernel, norm, pad_mode, kernel_params)


def interpolate_adjoint(
    vals: Tensor,
    locs: Tensor,
    grid_size: tuple[int, ...],
    width: float | tuple[float, ...],
    kernel: str = "kaiser_bessel",
    norm: int = 1,
    pad_mode: str = "circular",
    kernel_params: dict = None,
) -> Tensor:
    """Adjoint of interpolation (gridding) (reference interp.py:184)."""
    return InterpolateAdjointFn.apply(vals, locs, grid_size, width, kernel, norm, pad_mode, kernel_params)
