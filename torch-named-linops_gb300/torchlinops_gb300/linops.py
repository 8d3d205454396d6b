"""Operator layer around the GB300 kernels: Interpolate, ArrayToBlocks,
BlocksToArray and the NUFFT chain, with ``.H``, ``.N`` and composition.

This mirrors the operator interface of the reference's NamedLinop framework
(linops/namedlinop.py:34-661, chain.py:26-232) for the operators on the hot
path -- static ``fn`` / ``adj_fn`` / ``normal_fn`` taking the operator first,
``.H`` (adjoint), ``.N`` (normal), ``A @ B`` (chain, B applied first) -- so a
reference user's NUFFT / CG code runs against these kernels. The named-shape
arguments of the reference constructors are accepted and stored; the
named-dimension algebra, splitting across GPUs and streams are not part of
this package. The same kernels are reached from the reference's own linops by
re-pointing its functional calls (see the integration notes of this repo).

* ``Interpolate``    <- linops/interp.py:16-137
* ``ArrayToBlocks``  <- linops/array_to_blocks.py:16-110
* ``BlocksToArray``  <- linops/array_to_blocks.py:113-205
* ``NUFFT``          <- linops/nufft.py:34-392 (interpolate mode); its centred
  FFT's two shifts are folded into ``PadShift`` and the trajectory
* ``PadShift``, ``pad_shift``, ``crop_shift`` <- pad_last.py + utils/_fft.py
  (pad, ifftshift / fftshift, crop, apodization and coil maps in one pass)
* ``Diagonal``, ``Scalar``, ``Pad``, ``FFT`` <- linops/{diagonal,scalar,pad_last,fft}.py
* ``nufft`` / ``nufft_adjoint`` <- functional/_nufft.py:16-112
* ``ToeplitzNormal``, ``toeplitz_psf`` <- linops/nufft.py:226-239, 395-568
  (``NUFFT(..., toeplitz=True).normal(inner)``)
"""

from __future__ import annotations

import ctypes
import math
from collections import OrderedDict
from copy import copy
from math import prod
from typing import Optional

import torch
import torch.nn as nn
import torch.nn.functional as F
from torch import Tensor

from . import _ext
from . import blocks as B
from . import circpad as CP
from . import interp as I
from .index import index as _index_fwd
from .index import index_adjoint as _index_adj

__all__ = [
    "NamedLinop",
    "Chain",
    "Diagonal",
    "Scalar",
    "Pad",
    "FFT",
    "Interpolate",
    "ArrayToBlocks",
    "BlocksToArray",
    "Sampling",
    "Convolution",
    "NUFFT",
    "ToeplitzNormal",
    "toeplitz_psf",
    "nufft",
    "nufft_adjoint",
    "cfftn",
    "cifftn",
]


def cfftn(x, dim=None, norm="ortho"):
    """Centred n-D FFT (reference utils/_fft.py:7-32)."""
    x = torch.fft.ifftshift(x, dim=dim)
    x = torch.fft.fftn(x, dim=dim, norm=norm)
    return torch.fft.fftshift(x, dim=dim)


def cifftn(x, dim=None, norm="ortho"):
    """Centred n-D inverse FFT (reference utils/_fft.py:35-60)."""
    x = torch.fft.ifftshift(x, dim=dim)
    x = torch.fft.ifftn(x, dim=dim, norm=norm)
    return torch.fft.fftshift(x, dim=dim)


class NamedLinop(nn.Module):
    """Linear operator with static fn / adj_fn / normal_fn (namedlinop.py:88-450)."""

    def __init__(self):
        super().__init__()
        self._adjoint = None
        self._normal = None

    def forward(self, x: Tensor) -> Tensor:
        return self.fn(self, x)

    @staticmethod
    def fn(linop, x: Tensor, /) -> Tensor:
        raise NotImplementedError

    @staticmethod
    def adj_fn(linop, x: Tensor, /) -> Tensor:
        raise NotImplementedError

    @staticmethod
    def normal_fn(linop, x: Tensor, /) -> Tensor:
        return linop.adj_fn(linop, linop.fn(linop, x))

    def adjoint(self) -> "NamedLinop":
        adj = copy(self)
        adj._adjoint = None
        adj._normal = None
        adj.fn, adj.adj_fn = self.adj_fn, self.fn
        return adj

    @property
    def H(self) -> "NamedLinop":
        if self._adjoint is None:
            a = self.adjoint()
            a._adjoint = [self]
            self._adjoint = [a]
        return self._adjoint[0]

    def normal(self, inner: Optional["NamedLinop"] = None) -> "NamedLinop":
        if inner is not None:
            return Chain(self, inner, self.H)
        return _Normal(self)

    @property
    def N(self) -> "NamedLinop":
        if self._normal is None:
            self._normal = [self.normal()]
        return self._normal[0]

    def __matmul__(self, other: "NamedLinop") -> "NamedLinop":
        return Chain(other, self)

    def __copy__(self):
        new = type(self).__new__(type(self))
        new.__dict__ = self.__dict__.copy()
        new._parameters = self._parameters.copy()
        new._buffers = self._buffers.copy()
        new._modules = self._modules.copy()
        return new


class _Normal(NamedLinop):
    """A^H A as one operator: self-adjoint (namedlinop.py:565-600)."""

    def __init__(self, linop: NamedLinop):
        super().__init__()
        self.inner = linop

    @staticmethod
    def fn(n, x, /):
        return n.inner.normal_fn(n.inner, x)

    @staticmethod
    def adj_fn(n, x, /):
        return n.inner.normal_fn(n.inner, x)


class Chain(NamedLinop):
    """Composition applied left to right (chain.py:26-116)."""

    def __init__(self, *linops: NamedLinop, name: Optional[str] = None):
        super().__init__()
        flat = []
        for op in linops:
            flat.extend(op.linops if type(op) is Chain else [op])
        self.linops = nn.ModuleList(flat)
        self.name = name

    def __getitem__(self, i):
        return self.linops[i]

    @staticmethod
    def fn(chain, x, /):
        for op in chain.linops:
            x = op(x)
        return x

    @staticmethod
    def adj_fn(chain, x, /):
        for op in reversed(chain.linops):
            x = op.H(x)
        return x

    @staticmethod
    def normal_fn(chain, x, /):
        return chain.adj_fn(chain, chain.fn(chain, x))

    def adjoint(self):
        adj = copy(self)
        adj._adjoint = None
        adj._normal = None
        adj.linops = nn.ModuleList([op.H for op in reversed(self.linops)])
        return adj


class Diagonal(NamedLinop):
    """x -> w * x; adjoint conj(w) * x (diagonal.py)."""

    def __init__(self, weight: Tensor, ioshape=None, broadcast_dims=None):
        super().__init__()
        self.weight = nn.Parameter(weight, requires_grad=False)
        self.ioshape = ioshape

    @staticmethod
    def fn(d, x, /):
        return x * d.weight

    @staticmethod
    def adj_fn(d, x, /):
        return x * d.weight.conj()

    @staticmethod
    def normal_fn(d, x, /):
        return x * (d.weight.abs() ** 2)


class Scalar(Diagonal):
    """x -> alpha * x (scalar.py)."""

    def __init__(self, weight, ioshape=None):
        if not isinstance(weight, torch.Tensor):
            weight = torch.tensor(weight)
        super().__init__(weight, ioshape)


def pad_to_size(grid_size, padded_size):
    """Centred F.pad list (pad_last.py:137-178)."""
    if len(grid_size) != len(padded_size):
        raise ValueError(f"Dimension mismatch: cannot pad from size {grid_size} to size {padded_size}.")
    pad = []
    for i, p in zip(grid_size, padded_size):
        tp = p - i
        if tp % 2:
            left, right = (tp // 2 + 1, tp // 2) if i % 2 else (tp // 2, tp // 2 + 1)
        else:
            left = right = tp // 2
        pad.append([left, right])
    pad.reverse()
    return sum(pad, start=[])


def crop_slice_from_pad(pad):
    out = []
    for i in range(len(pad) // 2):
        start, stop = pad[2 * i], -pad[2 * i + 1]
        out.append(slice(start, stop if stop != 0 else None))
    out.reverse()
    return out


class Pad(NamedLinop):
    """Centred zero pad of the last dims; adjoint crops (pad_last.py:13-122)."""

    def __init__(self, pad_im_size, im_size, in_shape=None, out_shape=None, batch_shape=None):
        super().__init__()
        if len(pad_im_size) != len(im_size):
            raise ValueError(f"Padded and unpadded dims should be the same length. padded: {pad_im_size} unpadded: {im_size}")
        self.D = len(im_size)
        self.im_size = tuple(im_size)
        self.pad_im_size = tuple(pad_im_size)
        self.pad = pad_to_size(self.im_size, self.pad_im_size)
        self.crop_slice = crop_slice_from_pad(self.pad)

    @staticmethod
    def fn(p, x, /):
        if tuple(x.shape[-p.D:]) != p.im_size:
            raise ValueError(f"Mismatched shapes: expected {p.im_size} but got {x.shape[-p.D:]}")
        return F.pad(x, p.pad + [0, 0] * (x.ndim - p.D))

    @staticmethod
    def adj_fn(p, y, /):
        if tuple(y.shape[-p.D:]) != p.pad_im_size:
            raise ValueError(f"Mismatched shapes: expected {p.pad_im_size} but got {y.shape[-p.D:]}")
        return y[tuple([slice(None)] * (y.ndim - p.D) + p.crop_slice)]


def _i64(vals):
    arr = (ctypes.c_int64 * 3)()
    for i, v in enumerate(vals):
        arr[i] = int(v)
    return arr


def _pad_shift(x: Tensor, im_size, padded_size, maps: Optional[Tensor] = None, apod: Optional[Tensor] = None,
               modulate: bool = False) -> Tensor:
    nd = len(im_size)
    _ext.check_cuda(x, maps, apod)
    if x.dtype != torch.complex64:
        raise TypeError(f"pad_shift takes complex64, got {x.dtype}")
    if tuple(x.shape[-nd:]) != tuple(im_size):
        raise ValueError(f"Mismatched shapes: expected {tuple(im_size)} but got {tuple(x.shape[-nd:])}")
    pad = pad_to_size(im_size, padded_size)
    off = [pad[2 * (nd - 1 - i)] for i in range(nd)]
    shift = [p // 2 for p in padded_size]
    batch = x.shape[:-nd]
    xb = x.resolve_conj().resolve_neg().contiguous()
    nb = math.prod(batch)
    C = 1
    if maps is not None:
        maps = maps.resolve_conj().resolve_neg().to(torch.complex64).contiguous()
        C = maps.numel() // math.prod(im_size)
    out_batch = tuple(batch) + ((C,) if maps is not None else ())
    out = torch.empty(*out_batch, *padded_size, dtype=torch.complex64, device=x.device)
    ap = None if apod is None else apod.to(torch.float32).contiguous()
    _ext.check(_ext.lib().tlgb_pad_shift_c64(_ext.ptr(xb), nb, nd, _i64(im_size), _i64(padded_size), _i64(off),
                                             _i64(shift), int(bool(modulate)), _ext.ptr(ap), _ext.ptr(maps), C,
                                             _ext.ptr(out), _ext.stream_ptr(x.device)), "pad_shift")
    return out


def _crop_shift(z: Tensor, im_size, padded_size, maps: Optional[Tensor] = None, apod: Optional[Tensor] = None,
                alpha: float = 1.0, add: Optional[Tensor] = None, beta: float = 0.0, modulate: bool = False) -> Tensor:
    nd = len(im_size)
    _ext.check_cuda(z, maps, apod, add)
    if z.dtype != torch.complex64:
        raise TypeError(f"crop_shift takes complex64, got {z.dtype}")
    if tuple(z.shape[-nd:]) != tuple(padded_size):
        raise ValueError(f"Mismatched shapes: expected {tuple(padded_size)} but got {tuple(z.shape[-nd:])}")
    pad = pad_to_size(im_size, padded_size)
    off = [pad[2 * (nd - 1 - i)] for i in range(nd)]
    shift = [p // 2 for p in padded_size]
    zb = z.resolve_conj().resolve_neg().contiguous()
    C = 1
    batch = z.shape[:-nd]
    if maps is not None:
        maps = maps.resolve_conj().resolve_neg().to(torch.complex64).contiguous()
        C = maps.numel() // math.prod(im_size)
        batch = batch[:-1]
    nb = math.prod(batch)
    out = torch.empty(*batch, *im_size, dtype=torch.complex64, device=z.device)
    ap = None if apod is None else apod.to(torch.float32).contiguous()
    ad = None if add is None else add.resolve_conj().resolve_neg().to(torch.complex64).contiguous()
    _ext.check(_ext.lib().tlgb_crop_shift_c64(_ext.ptr(zb), nb, nd, _i64(im_size), _i64(padded_size), _i64(off),
                                              _i64(shift), int(bool(modulate)), _ext.ptr(ap), _ext.ptr(maps), C,
                                              ctypes.c_float(alpha), _ext.ptr(ad), ctypes.c_float(beta),
                                              _ext.ptr(out), _ext.stream_ptr(z.device)), "crop_shift")
    return out


class _PadShiftFn(torch.autograd.Function):
    """pad_shift is C-linear in x; its adjoint is crop_shift with the same
    maps and apodization, so the backward pass is one crop_shift. Maps and
    apodization are constants (no gradient)."""

    @staticmethod
    def forward(ctx, x, im_size, padded_size, maps, apod, modulate):
        ctx.args = (tuple(im_size), tuple(padded_size), maps, apod, modulate)
        return _pad_shift(x, im_size, padded_size, maps, apod, modulate)

    @staticmethod
    def backward(ctx, g):
        im_size, padded_size, maps, apod, modulate = ctx.args
        gx = None
        if ctx.needs_input_grad[0]:
            gx = _crop_shift(g.contiguous(), im_size, padded_size, maps, apod, modulate=modulate)
        return gx, None, None, None, None, None


class _CropShiftFn(torch.autograd.Function):
    """alpha * crop_shift(z) + beta * add: the backward pass is alpha *
    pad_shift(g) for z and beta * g for add."""

    @staticmethod
    def forward(ctx, z, add, im_size, padded_size, maps, apod, alpha, beta, modulate):
        ctx.args = (tuple(im_size), tuple(padded_size), maps, apod, alpha, beta, modulate)
        return _crop_shift(z, im_size, padded_size, maps, apod, alpha, add, beta, modulate)

    @staticmethod
    def backward(ctx, g):
        im_size, padded_size, maps, apod, alpha, beta, modulate = ctx.args
        gz = gadd = None
        if ctx.needs_input_grad[0]:
            gz = _pad_shift(g.contiguous(), im_size, padded_size, maps, apod, modulate)
            if alpha != 1.0:
                gz = gz * alpha
        if ctx.needs_input_grad[1]:
            gadd = g * beta
        return gz, gadd, None, None, None, None, None, None, None


def pad_shift(x: Tensor, im_size, padded_size, maps: Optional[Tensor] = None, apod: Optional[Tensor] = None,
              modulate: bool = False) -> Tensor:
    """ifftshift(pad(apod * x)) (or per coil map: ifftshift(pad(maps_c * apod * x)))
    over the last ``len(im_size)`` dims in one pass; complex64, CUDA.
    ``modulate`` multiplies by m[j] = prod_e exp(2 pi i j_e floor(Np_e/2) / Np_e)
    (the sign (-1)^j_e for even sizes), so that an uncentred fftn of the
    result is the centred cfftn of the padded image. Differentiable in ``x``."""
    if torch.is_grad_enabled() and x.requires_grad:
        return _PadShiftFn.apply(x, im_size, padded_size, maps, apod, modulate)
    return _pad_shift(x, im_size, padded_size, maps, apod, modulate)


def crop_shift(z: Tensor, im_size, padded_size, maps: Optional[Tensor] = None, apod: Optional[Tensor] = None,
               alpha: float = 1.0, add: Optional[Tensor] = None, beta: float = 0.0, modulate: bool = False) -> Tensor:
    """alpha * apod * crop(fftshift(z)) (with maps: summed over the coil dim of
    z after multiplying by conj(maps)) + beta * add, in one pass; with
    ``modulate``, z is first multiplied by conj(m[j]) (the adjoint of
    pad_shift's modulation). Differentiable in ``z`` and ``add``."""
    if torch.is_grad_enabled() and (z.requires_grad or (add is not None and add.requires_grad)):
        return _CropShiftFn.apply(z, add, im_size, padded_size, maps, apod, alpha, beta, modulate)
    return _crop_shift(z, im_size, padded_size, maps, apod, alpha, add, beta, modulate)


class PadShift(NamedLinop):
    """apod * x, centred zero pad, ifftshift and the k-space centring
    modulation in one pass; the adjoint is the conjugate modulation,
    fftshift, crop and apod in one pass. With an uncentred FFT after it, this
    is the reference's Apodize -> Pad -> cfftn (nufft.py:170-184) without
    the two shift passes per transform, and the interpolation after it reads
    the reference's own coordinates."""

    def __init__(self, padded_size, im_size, apod: Optional[Tensor] = None):
        super().__init__()
        self.im_size = tuple(im_size)
        self.pad_im_size = tuple(padded_size)
        self.apod = apod

    @staticmethod
    def fn(p, x, /):
        return pad_shift(x, p.im_size, p.pad_im_size, apod=p.apod, modulate=True)

    @staticmethod
    def adj_fn(p, y, /):
        return crop_shift(y, p.im_size, p.pad_im_size, apod=p.apod, modulate=True)


class FFT(NamedLinop):
    """Centred orthonormal FFT over the last ndim dims (fft.py)."""

    def __init__(self, ndim: int, centered: bool = True, norm: str = "ortho", batch_shape=None, grid_shapes=None):
        super().__init__()
        self.ndim = ndim
        self.centered = centered
        self.norm = norm
        self.dim = tuple(range(-ndim, 0))

    @staticmethod
    def fn(f, x, /):
        if f.centered:
            return cfftn(x, dim=f.dim, norm=f.norm)
        return torch.fft.fftn(x, dim=f.dim, norm=f.norm)

    @staticmethod
    def adj_fn(f, x, /):
        if f.centered:
            return cifftn(x, dim=f.dim, norm=f.norm)
        return torch.fft.ifftn(x, dim=f.dim, norm=f.norm)

    @staticmethod
    def normal_fn(f, x, /):
        return x


class Interpolate(NamedLinop):
    """Grid -> off-grid points (interp.py:16-137): (batch, grid) -> (batch, locs_batch)."""

    def __init__(
        self,
        locs: Tensor,
        grid_size: tuple[int, ...],
        batch_shape=None,
        locs_batch_shape=None,
        grid_shape=None,
        width: float = 4.0,
        kernel: str = "kaiser_bessel",
        norm: int = 1,
        pad_mode: str = "circular",
        kernel_params: Optional[dict] = None,
    ):
        super().__init__()
        if locs_batch_shape is not None and len(locs_batch_shape) > len(locs.shape) - 1:
            raise ValueError(
                f"locs_batch_shape has length longer than batch dim of locs. locs_batch_shape: {locs_batch_shape}, locs: {locs.shape}"
            )
        self.locs = nn.Parameter(locs, requires_grad=False)
        self.grid_size = tuple(grid_size)
        kp = dict(beta=1.0)
        if kernel_params:
            kp.update(kernel_params)
        self.interp_params = {
            "width": width,
            "kernel": kernel,
            "norm": norm,
            "pad_mode": pad_mode,
            "kernel_params": kp,
        }

    @staticmethod
    def fn(interp, x, /):
        return I.interpolate(x, interp.locs, **interp.interp_params)

    @staticmethod
    def adj_fn(interp, x, /):
        return I.interpolate_adjoint(x, interp.locs, interp.grid_size, **interp.interp_params)

    def size(self, dim):
        return None


class ArrayToBlocks(NamedLinop):
    """Sliding blocks of an array (array_to_blocks.py:16-110)."""

    def __init__(self, grid_size, block_size, stride, mask=None, batch_shape=None, array_shape=None, blocks_shape=None):
        super().__init__()
        self.grid_size = tuple(grid_size)
        self.ndim = len(self.grid_size)
        self.block_size = tuple(block_size)
        self.stride = tuple(stride)
        self.mask = nn.Parameter(mask, requires_grad=False) if mask is not None else None

    @staticmethod
    def fn(a, x, /):
        return B.array_to_blocks(x, a.block_size, a.stride, a.mask)

    @staticmethod
    def adj_fn(a, x, /):
        return B.blocks_to_array(x, a.grid_size, a.block_size, a.stride, a.mask)

    @staticmethod
    def normal_fn(a, x, /):
        return a.adj_fn(a, a.fn(a, x))

    def adjoint(self):
        return BlocksToArray(self.grid_size, self.block_size, self.stride, self.mask)


class BlocksToArray(NamedLinop):
    """Overlapping blocks summed into an array (array_to_blocks.py:113-205)."""

    def __init__(self, grid_size, block_size, stride, mask=None, batch_shape=None, blocks_shape=None, array_shape=None):
        super().__init__()
        self.grid_size = tuple(grid_size)
        self.ndim = len(self.grid_size)
        self.block_size = tuple(block_size)
        self.stride = tuple(stride)
        self.mask = nn.Parameter(mask, requires_grad=False) if mask is not None else None

    @staticmethod
    def fn(b, x, /):
        return B.blocks_to_array(x, b.grid_size, b.block_size, b.stride, b.mask)

    @staticmethod
    def adj_fn(b, x, /):
        if tuple(x.shape[-b.ndim:]) != b.grid_size:
            raise RuntimeError(f"BlocksToArray expected input with full size {b.grid_size} but got {x.shape}")
        return B.array_to_blocks(x, b.block_size, b.stride, b.mask)

    def adjoint(self):
        return ArrayToBlocks(self.grid_size, self.block_size, self.stride, self.mask)


class Sampling(NamedLinop):
    """Samples at integer locations (linops/sampling.py:16-101): (batch,
    grid) -> (batch, idx batch), forward ``index``, adjoint the deterministic
    ``index_adjoint``."""

    def __init__(self, idx: tuple[Tensor, ...], input_size: tuple[int, ...]):
        super().__init__()
        if len(idx) != len(input_size):
            raise ValueError(f"Input size {input_size} doesn't match index with length {len(idx)}.")
        for d, (t, s) in enumerate(zip(idx, input_size)):
            if (t < 0).any() or (t >= s).any():
                raise ValueError(
                    f"Sampling index must lie within range [0, {s - 1}] but got range [{t.min().item()}, {t.max().item()}] for dim {d}"
                )
        self.input_size = tuple(int(s) for s in input_size)
        self.idx = nn.ParameterList([nn.Parameter(i, requires_grad=False) for i in idx])

    @staticmethod
    def fn(s, x, /):
        return _index_fwd(x, tuple(s.idx))

    @staticmethod
    def adj_fn(s, x, /):
        return _index_adj(x, tuple(s.idx), s.input_size)


def _pad_to_odd(kernel: Tensor, ndim: int) -> Tensor:
    # reference linops/convolution.py:355-378: one trailing zero per even dim
    pad = []
    for s in reversed(kernel.shape[-ndim:]):
        pad += [0, 0 if s % 2 else 1]
    return F.pad(kernel, pad, value=0)


class _Fp32Conv:
    """cuDNN convolutions in full float32: torch lets cuDNN use TF32 (10-bit
    mantissas) by default, far coarser than this package's 1e-5 tolerance
    against the reference's CPU float32 convolution."""

    def __enter__(self):
        self.prev = torch.backends.cudnn.allow_tf32
        torch.backends.cudnn.allow_tf32 = False

    def __exit__(self, *exc):
        torch.backends.cudnn.allow_tf32 = self.prev


class Convolution(NamedLinop):
    """Convolution with one kernel broadcast over every leading dim
    (linops/convolution.py:19-164): 'zeros' or 'circular' padding, the kernel
    centred at kernel_size // 2 and flipped (a true convolution). The
    circular mode pads with this package's ``circular_pad`` and its adjoint
    convolves the padded input with the flipped, conjugated kernel, as the
    reference does; the convolutions themselves run in torch (cuDNN)."""

    def __init__(self, kernel: Tensor, padding_mode: str = "zeros"):
        super().__init__()
        ndim = kernel.dim()
        if ndim not in (1, 2, 3):
            raise ValueError(f"ndim must be 1, 2, or 3, got {ndim}")
        if padding_mode not in ("zeros", "circular"):
            raise ValueError(f"Unrecognized padding_mode: {padding_mode}")
        self.ndim = ndim
        self.padding_mode = padding_mode
        kernel = _pad_to_odd(kernel, ndim)
        half = [(s // 2, s // 2) for s in kernel.shape[-ndim:]]
        self._crop = tuple(slice(a, -b if b > 0 else None) for a, b in half)
        self._pad = tuple(v for pair in reversed(half) for v in pair)
        self.kernel = kernel
        w = torch.flip(kernel, dims=tuple(range(-ndim, 0)))[None, None]
        self._weight = nn.Parameter(w, requires_grad=False)

    def _flat(self, x):
        lead = x.shape[: x.ndim - self.ndim]
        return x.reshape(-1, 1, *x.shape[x.ndim - self.ndim:]), lead

    @staticmethod
    def fn(c, x, /):
        xf, lead = c._flat(x)
        conv = (F.conv1d, F.conv2d, F.conv3d)[c.ndim - 1]
        with _Fp32Conv():
            if c.padding_mode == "circular":
                y = conv(CP.circular_pad(xf, c._pad), c._weight, padding=0)
            else:
                y = conv(xf, c._weight, padding="same")
        return y.reshape(*lead, *y.shape[2:])

    @staticmethod
    def adj_fn(c, x, /):
        xf, lead = c._flat(x)
        with _Fp32Conv():
            if c.padding_mode == "circular":
                w = torch.flip(c._weight, dims=tuple(range(-c.ndim, 0))).conj()
                conv = (F.conv1d, F.conv2d, F.conv3d)[c.ndim - 1]
                y = conv(CP.circular_pad(xf, c._pad), w, padding=0)
            else:
                conv_t = (F.conv_transpose1d, F.conv_transpose2d, F.conv_transpose3d)[c.ndim - 1]
                y = conv_t(xf, c._weight.conj(), padding=0)[(slice(None), slice(None)) + c._crop]
        return y.reshape(*lead, *y.shape[2:])


def nufft_beta(width: float, oversamp: float) -> float:
    return I.kaiser_bessel_beta(width, oversamp)


def prep_locs_sampling(locs: Tensor, grid_size, padded_size, pad_mode="circular") -> Tensor:
    """Centred locs -> integer indices of the padded grid for the sampling
    mode (nufft.py:316-333): scale, shift, then clamp (zero padding) or round
    and wrap (circular), as int64."""
    if pad_mode not in ("zero", "circular"):
        raise ValueError(f"Unrecognized padding mode during prep: {pad_mode}")
    out = locs.clone()
    for i in range(-len(grid_size), 0):
        out[..., i] *= padded_size[i] / grid_size[i]
        out[..., i] += padded_size[i] // 2
        if pad_mode == "zero":
            out[..., i] = torch.clamp(out[..., i], 0, padded_size[i] - 1)
        else:
            out[..., i] = torch.round(out[..., i])
            out[..., i] = torch.remainder(out[..., i], padded_size[i])
    return out.to(torch.int64)


def prep_locs(locs: Tensor, grid_size, padded_size, pad_mode="circular") -> Tensor:
    """Scale centred locs in [-N/2, N/2] to the padded grid (nufft.py:242-334).

    The same float operations per coordinate as the reference (multiply by
    Np/N, add Np//2, then clamp or wrap), done on all dimensions at once when
    their sizes agree (one kernel per operation instead of several per
    dimension)."""
    if pad_mode not in ("zero", "circular"):
        raise ValueError(f"Unrecognized padding mode during prep: {pad_mode}")
    nd = len(grid_size)
    same = len(set(zip(grid_size, padded_size))) == 1
    if same and locs.shape[-1] == nd:
        n, p = grid_size[0], padded_size[0]
        out = locs * (p / n) + p // 2
        return torch.clamp(out, 0, p - 1) if pad_mode == "zero" else torch.remainder(out, p)
    out = locs.clone()
    for i in range(-nd, 0):
        out[..., i] *= padded_size[i] / grid_size[i]
        out[..., i] += padded_size[i] // 2
        if pad_mode == "zero":
            out[..., i] = torch.clamp(out[..., i], 0, padded_size[i] - 1)
        else:
            out[..., i] = torch.remainder(out[..., i], padded_size[i])
    return out


def apodize_weights(grid_size, padded_size, oversamp, width: float, beta: float) -> Tensor:
    """Separable KB apodization (nufft.py:349-365)."""
    gs = torch.tensor(grid_size)
    ps = torch.tensor(padded_size)
    g = torch.stack(torch.meshgrid(*(torch.arange(s) for s in grid_size), indexing="ij"), dim=-1)
    apod = (beta**2 - (torch.pi * width * (g - gs // 2) / ps) ** 2) ** 0.5
    apod = apod / torch.sinh(apod)
    return torch.prod(apod, dim=-1)


class NUFFT(Chain):
    """Apodize -> pad -> centred FFT -> Interpolate -> scale (nufft.py:34-215)."""

    def __init__(
        self,
        locs: Tensor,
        grid_size: tuple[int, ...],
        output_shape=None,
        input_shape=None,
        input_kshape=None,
        batch_shape=None,
        oversamp: float = 1.25,
        width: float = 4.0,
        mode: str = "interpolate",
        do_prep_locs: bool = True,
        apodize_weights: Optional[Tensor] = None,
        **options,
    ):
        if mode not in ("interpolate", "sampling"):
            raise ValueError(f"Unrecognized NUFFT mode: {mode}")
        device = locs.device
        ndim = len(grid_size)
        padded_size = tuple(int(i * oversamp) for i in grid_size)
        self.mode = mode
        if mode == "sampling":
            # pad -> centred FFT -> Sampling at rounded, wrapped k-space
            # indices; no apodization or scaling (nufft.py:185-200)
            locs_prepared = prep_locs_sampling(locs, grid_size, padded_size) if do_prep_locs else locs
            if locs_prepared.is_complex() or locs_prepared.is_floating_point():
                raise ValueError(f"Sampling linop requries integer-type locs but got {locs_prepared.dtype}")
            padshift = PadShift(padded_size, grid_size, None)
            fft = FFT(ndim=ndim, centered=False, norm="ortho")
            interp = Sampling(tuple(locs_prepared[..., d] for d in range(ndim)), padded_size)
            super().__init__(padshift, fft, interp, name="NUFFT")
            self.options = options
            self.apodize_weight = None
            self.scale_factor = 1.0
            self.padded_size = padded_size
            self.locs_prepared = locs_prepared
            self.locs = locs
            self.grid_size = tuple(grid_size)
            self.oversamp = oversamp
            self.width = width
            self.pad, self.fft, self.interp = padshift, fft, interp
            return
        beta = nufft_beta(width, oversamp)
        if apodize_weights is None:
            weight = globals()["apodize_weights"](grid_size, padded_size, oversamp, width, beta).to(device)
        else:
            weight = apodize_weights
        if weight.isnan().any() or weight.isinf().any():
            raise ValueError(f"Nan/Inf values detected in apodization weight (width={width}, oversamp={oversamp}).")
        # Apodize -> Pad -> cfftn, with both centring shifts folded into the
        # pad gather (no full-grid shift passes); same operator, same
        # interpolation coordinates as the reference
        padshift = PadShift(padded_size, grid_size, weight)
        fft = FFT(ndim=locs.shape[-1], centered=False, norm="ortho")
        locs_prepared = prep_locs(locs, grid_size, padded_size) if do_prep_locs else locs
        interp = Interpolate(
            locs_prepared, padded_size, width=width, kernel="kaiser_bessel", kernel_params=dict(beta=beta)
        )
        scale_factor = width**ndim * (prod(grid_size) / prod(padded_size)) ** 0.5
        scale = Scalar(torch.tensor(1.0 / scale_factor, device=device))
        super().__init__(padshift, fft, interp, scale, name="NUFFT")
        self.options = options
        self.apodize_weight = weight
        self.scale_factor = scale_factor
        self.padded_size = padded_size
        self.locs_prepared = locs_prepared
        self.locs = locs
        self.grid_size = tuple(grid_size)
        self.oversamp = oversamp
        self.width = width
        self.pad = padshift
        self.fft = fft
        self.interp = interp

    def normal(self, inner: Optional[NamedLinop] = None) -> NamedLinop:
        """With the ``toeplitz`` option, the Toeplitz embedding of
        ``self.H @ inner @ self`` (nufft.py:226-239) for ``inner`` None or a
        diagonal weighting of the points; otherwise (and for other ``inner``
        operators) the chain itself, forward then adjoint."""
        if self.options.get("toeplitz", False) and self.mode == "interpolate":
            weight = _point_weight(inner, self.locs_prepared.shape[:-1])
            if weight is not False:
                return ToeplitzNormal(self, weight, self.options.get("toeplitz_oversamp", 2.0),
                                      self.options.get("toeplitz_dtype"))
        return super().normal(inner)


def scale_int(t, scale_factor: float) -> tuple[int, ...]:
    return tuple(int(scale_factor * s) for s in t)


def rescale_locs(locs: Tensor, c0, w0, c1, w1) -> Tensor:
    """(loc - c0) * w1 / w0 + c1 per coordinate, with the reference's float
    operations in the locations' dtype (nufft.py:538-568)."""
    return torch.stack([(locs[..., d] - c0[d]) * w1[d] / w0[d] + c1[d] for d in range(locs.shape[-1])], dim=-1)


def _point_weight(inner: Optional[NamedLinop], points_shape):
    """The per-point weight of a diagonal ``inner`` (None for no inner), or
    False when ``inner`` is not a weighting of the points alone."""
    if inner is None:
        return None
    if isinstance(inner, Diagonal):
        w = inner.weight.detach()
        try:
            if torch.broadcast_shapes(w.shape, tuple(points_shape)) == tuple(points_shape):
                return w
        except RuntimeError:
            pass
    return False


@torch.no_grad()
def toeplitz_psf(nufft: NUFFT, weight: Optional[Tensor] = None, oversamp: float = 2.0,
                 dtype: Optional[torch.dtype] = None) -> Tensor:
    """The Toeplitz kernel of ``nufft.H @ diag(weight) @ nufft``: centred
    k-space on the ``oversamp`` x grid (nufft.py:395-494, the weight of its
    ``Dense``). It is the adjoint NUFFT of the weights (ones by default) on
    the larger grid, whose points are the prepared points rescaled from the
    padded grid Np to ``int(oversamp * Np)`` cells, through an unnormalised
    centred FFT, times ``oversamp^D / sqrt(prod(grid))``. As in the
    reference, the larger NUFFT pads its grid to ``int(1.25 * int(oversamp *
    N))`` cells, one more than the points' range when ``1.25 * N`` has a
    fractional part of at least 1/2."""
    dtype = torch.complex64 if dtype is None else dtype
    if dtype != torch.complex64:
        raise TypeError(f"Toeplitz kernels are complex64, got {dtype}")
    grid_size = nufft.grid_size
    ndim = len(grid_size)
    new_grid = scale_int(grid_size, oversamp)
    width = nufft.padded_size
    new_width = scale_int(width, oversamp)
    new_locs = rescale_locs(nufft.locs_prepared.detach(), tuple(w // 2 for w in width), width,
                            tuple(w // 2 for w in new_width), new_width)
    big = NUFFT(new_locs, new_grid, oversamp=nufft.oversamp, width=nufft.width, do_prep_locs=False)
    points = tuple(new_locs.shape[:-1])
    if weight is None:
        w = torch.ones(points, dtype=dtype, device=new_locs.device)
    else:
        w = torch.broadcast_to(weight.to(device=new_locs.device, dtype=dtype), points).contiguous()
    otf = big.H(w)
    dim = tuple(range(-ndim, 0))
    return cfftn(otf, dim=dim, norm=None) * (oversamp**ndim / prod(new_grid) ** 0.5)


class ToeplitzNormal(NamedLinop):
    """``nufft.H @ diag(weight) @ nufft`` by Toeplitz embedding
    (nufft.py:226-239): zero pad to the ``oversamp`` x grid, orthonormal
    centred FFT, multiply by the PSF kernel, inverse FFT, crop. Here the pad
    and ifftshift are one gather (``pad_shift``), the FFTs are uncentred
    cuFFT, the kernel is held in uncentred order, and fftshift and crop are
    one gather (``crop_shift``): no shift pass runs. Leading batch dims share
    the kernel."""

    def __init__(self, nufft: NUFFT, weight: Optional[Tensor] = None, oversamp: float = 2.0,
                 dtype: Optional[torch.dtype] = None):
        super().__init__()
        self.kernel = toeplitz_psf(nufft, weight, oversamp, dtype)
        ndim = len(nufft.grid_size)
        self.dim = tuple(range(-ndim, 0))
        self.im_size = tuple(nufft.grid_size)
        self.pad_im_size = scale_int(nufft.grid_size, oversamp)
        self.kernel_uncentred = torch.fft.ifftshift(self.kernel, dim=self.dim).contiguous()

    @staticmethod
    def _apply(t, x, k):
        z = pad_shift(x, t.im_size, t.pad_im_size)
        z = torch.fft.fftn(z, dim=t.dim, norm="ortho")
        z = torch.fft.ifftn(z * k, dim=t.dim, norm="ortho")
        return crop_shift(z, t.im_size, t.pad_im_size)

    @staticmethod
    def fn(t, x, /):
        return ToeplitzNormal._apply(t, x, t.kernel_uncentred)

    @staticmethod
    def adj_fn(t, x, /):
        return ToeplitzNormal._apply(t, x, t.kernel_uncentred.conj())


_APOD: "OrderedDict[tuple, Tensor]" = OrderedDict()


def _apod_on(device, grid_size, padded, oversamp: float, width: float, beta: float) -> Tensor:
    """The apodization weights on ``device``, computed once per sizes and
    kernel (the functional transforms would otherwise rebuild them on the
    host and copy them over on every call)."""
    key = (str(device), tuple(grid_size), tuple(padded), float(oversamp), float(width), float(beta))
    w = _APOD.get(key)
    if w is None:
        w = apodize_weights(grid_size, padded, oversamp, width, beta).to(device)
        _APOD[key] = w
        while len(_APOD) > 16:
            _APOD.popitem(last=False)
    else:
        _APOD.move_to_end(key)
    return w


_PREPARED_LOCS: "OrderedDict[tuple, tuple]" = OrderedDict()


def _prepared_locs(locs: Tensor, grid_size, padded) -> Tensor:
    """prep_locs for the functional transforms, memoised per locs tensor
    (object, version, weak reference) so that repeated calls on one
    trajectory reuse one interpolation plan. Locations that require a
    gradient are rescaled afresh (a trajectory being optimised changes every
    step, and the result carries the autograd graph)."""
    if locs.requires_grad and torch.is_grad_enabled():
        return prep_locs(locs, grid_size, padded)
    key = (id(locs), locs.data_ptr(), tuple(locs.shape), locs.dtype, tuple(grid_size), tuple(padded))
    hit = _PREPARED_LOCS.get(key)
    if hit is not None:
        ref, version, out = hit
        if ref() is locs and version == locs._version:
            _PREPARED_LOCS.move_to_end(key)
            return out
        del _PREPARED_LOCS[key]
    out = prep_locs(locs.detach(), grid_size, padded)
    I.remember(_PREPARED_LOCS, key, locs, out, 16)
    return out


def nufft(x: Tensor, locs: Tensor, oversamp: float = 1.25, width: float = 4.0) -> Tensor:
    """Functional NUFFT (functional/_nufft.py:16-62). Differentiable in ``x``
    and ``locs``."""
    grid_size = tuple(x.shape[-locs.shape[-1]:])
    ndim = locs.shape[-1]
    padded = tuple(int(s * oversamp) for s in grid_size)
    beta = nufft_beta(width, oversamp)
    x = pad_shift(x, grid_size, padded, apod=_apod_on(x.device, grid_size, padded, oversamp, width, beta), modulate=True)
    x = torch.fft.fftn(x, dim=tuple(range(-ndim, 0)), norm="ortho")
    x = I.interpolate(x, _prepared_locs(locs, grid_size, padded), width, kernel="kaiser_bessel",
                      kernel_params=dict(beta=beta))
    return x / (width**ndim * (prod(grid_size) / prod(padded)) ** 0.5)


def nufft_adjoint(x: Tensor, locs: Tensor, grid_size, oversamp: float = 1.25, width: float = 4.0) -> Tensor:
    """Functional adjoint NUFFT (functional/_nufft.py:65-112). Differentiable
    in ``x`` and ``locs``."""
    grid_size = tuple(grid_size)
    ndim = locs.shape[-1]
    padded = tuple(int(s * oversamp) for s in grid_size)
    beta = nufft_beta(width, oversamp)
    x = x / (width**ndim * (prod(grid_size) / prod(padded)) ** 0.5)
    x = I.interpolate_adjoint(x, _prepared_locs(locs, grid_size, padded), padded, width, kernel="kaiser_bessel",
                              kernel_params=dict(beta=beta))
    x = torch.fft.ifftn(x, dim=tuple(range(-ndim, 0)), norm="ortho")
    return crop_shift(x, grid_size, padded, apod=_apod_on(x.device, grid_size, padded, oversamp, width, beta),
                      modulate=True)
