"""CPU restatement of the reference's functional NUFFT, for the tests only.

Test infrastructure: this module is the checker; the product never imports
it. It follows ``functional/_nufft.py`` step by step:

* forward (``_nufft.py:16-62``): apodize, centred zero pad, centred
  orthonormal FFT, Kaiser-Bessel ungrid at the rescaled locations, divide by
  the scale factor;
* adjoint (``_nufft.py:65-112``): the same steps transposed;
* Toeplitz normal (``linops/nufft.py:226-239, 395-568``): the PSF kernel is
  the adjoint NUFFT, on a grid ``toep_oversamp`` times larger, of ones (or of
  the point weights of a diagonal ``inner``), through an unnormalised
  centred FFT; the normal operator pads, centred-FFTs, multiplies by the
  kernel, inverse-FFTs and crops.

``init_nufft`` (``_nufft.py:115-181``) supplies the oversampled size, beta
(``linops/nufft.py:337-346``), the apodization (``linops/nufft.py:349-365``),
the padding (``linops/pad_last.py:139-183``) and the location rescaling
(``linops/nufft.py:242-334``, circular mode). Arithmetic runs in ``dtype``
(float64 for the FP64 oracle); the interpolation is ``oracle.interp``.
"""

from __future__ import annotations

from math import prod

import torch

from . import interp as OI

__all__ = ["padded_size", "apodize_weights", "prep_locs", "kspace", "nufft", "nufft_adjoint", "scale_factor",
           "rescale_locs", "toeplitz_kernel", "toeplitz_normal"]


def padded_size(grid_size, oversamp: float):
    return tuple(int(s * oversamp) for s in grid_size)


def apodize_weights(grid_size, padded, oversamp: float, width: float, beta: float, dtype=torch.float64):
    """prod_e sqrt(beta^2 - (pi W (g_e - N_e//2) / Np_e)^2) / sinh(...)."""
    out = None
    for n, p in zip(grid_size, padded):
        g = torch.arange(n, dtype=dtype)
        a = (beta**2 - (torch.pi * width * (g - n // 2) / p) ** 2) ** 0.5
        a = a / torch.sinh(a)
        out = a if out is None else out[..., None] * a
    return out


def _pad_amounts(n: int, p: int):
    tp = p - n
    if tp % 2:
        return (tp // 2 + 1, tp // 2) if n % 2 else (tp // 2, tp // 2 + 1)
    return tp // 2, tp // 2


def _pad(x: torch.Tensor, grid_size, padded):
    spec = []
    for n, p in zip(reversed(grid_size), reversed(padded)):
        spec += list(_pad_amounts(n, p))
    return torch.nn.functional.pad(x, spec)


def _crop(x: torch.Tensor, grid_size, padded):
    sl = [slice(None)] * (x.ndim - len(grid_size))
    for n, p in zip(grid_size, padded):
        lo, _ = _pad_amounts(n, p)
        sl.append(slice(lo, lo + n))
    return x[tuple(sl)]


def _cfftn(x: torch.Tensor, dims, inverse: bool = False, norm: str | None = "ortho"):
    x = torch.fft.ifftshift(x, dim=dims)
    x = torch.fft.ifftn(x, dim=dims, norm=norm) if inverse else torch.fft.fftn(x, dim=dims, norm=norm)
    return torch.fft.fftshift(x, dim=dims)


def prep_locs(locs: torch.Tensor, grid_size, padded) -> torch.Tensor:
    """Scale [-N/2, N/2] locations to the padded grid and wrap (circular)."""
    out = locs.clone()
    for i in range(-len(grid_size), 0):
        out[..., i] = torch.remainder(out[..., i] * (padded[i] / grid_size[i]) + padded[i] // 2, padded[i])
    return out


def scale_factor(grid_size, padded, width: float) -> float:
    return width ** len(grid_size) * (prod(grid_size) / prod(padded)) ** 0.5


def kspace(x: torch.Tensor, ndim: int, oversamp: float = 1.25, width: float = 4.0, dtype=torch.float64):
    """cfftn(pad(apod * x)): the oversampled k-space grid the forward
    transform interpolates from."""
    cdt = torch.complex128 if dtype == torch.float64 else torch.complex64
    grid_size = tuple(x.shape[-ndim:])
    padded = padded_size(grid_size, oversamp)
    beta = OI.nufft_beta(width, oversamp)
    x = x.to(cdt) * apodize_weights(grid_size, padded, oversamp, width, beta, dtype)
    x = _pad(x, grid_size, padded)
    return _cfftn(x, tuple(range(-ndim, 0)))


def nufft(x: torch.Tensor, locs: torch.Tensor, oversamp: float = 1.25, width: float = 4.0, dtype=torch.float64):
    ndim = locs.shape[-1]
    grid_size = tuple(x.shape[-ndim:])
    padded = padded_size(grid_size, oversamp)
    beta = OI.nufft_beta(width, oversamp)
    k = kspace(x, ndim, oversamp, width, dtype)
    y = OI.ungrid(k, prep_locs(locs.to(dtype), grid_size, padded), width, beta=beta, dtype=dtype)
    return y / scale_factor(grid_size, padded, width)


def nufft_adjoint(y: torch.Tensor, locs: torch.Tensor, grid_size, oversamp: float = 1.25, width: float = 4.0,
                  dtype=torch.float64, prepared: bool = False):
    """``prepared``: ``locs`` are already in padded-grid units (the
    reference's ``do_prep_locs=False``)."""
    ndim = locs.shape[-1]
    grid_size = tuple(grid_size)
    padded = padded_size(grid_size, oversamp)
    beta = OI.nufft_beta(width, oversamp)
    cdt = torch.complex128 if dtype == torch.float64 else torch.complex64
    y = y.to(cdt) / scale_factor(grid_size, padded, width)
    gl = locs.to(dtype) if prepared else prep_locs(locs.to(dtype), grid_size, padded)
    g = OI.grid(y, gl, padded, width, beta=beta, dtype=dtype)
    x = _cfftn(g, tuple(range(-ndim, 0)), inverse=True)
    return _crop(x, grid_size, padded) * apodize_weights(grid_size, padded, oversamp, width, beta, dtype)


def rescale_locs(locs: torch.Tensor, c0, w0, c1, w1) -> torch.Tensor:
    """(loc - c0) * w1 / w0 + c1 per coordinate (``linops/nufft.py:538-568``)."""
    return torch.stack([(locs[..., d] - c0[d]) * w1[d] / w0[d] + c1[d] for d in range(locs.shape[-1])], dim=-1)


def toeplitz_kernel(locs: torch.Tensor, grid_size, oversamp: float = 1.25, width: float = 4.0,
                    toep_oversamp: float = 2.0, weight: torch.Tensor | None = None, dtype=torch.float64):
    """Centred k-space PSF kernel on the ``toep_oversamp`` x grid
    (``linops/nufft.py:395-494``). The points are prepared for the NUFFT's
    padded grid Np and then rescaled to ``int(toep_oversamp * Np)`` cells,
    while the larger NUFFT pads its grid ``int(toep_oversamp * N)`` to
    ``int(oversamp * int(toep_oversamp * N))`` cells; the two agree unless
    ``oversamp * N`` has a fractional part of at least 1/2 (then the
    reference's kernel is off, and so is this restatement)."""
    ndim = len(grid_size)
    grid_size = tuple(grid_size)
    padded = padded_size(grid_size, oversamp)
    new_grid = tuple(int(toep_oversamp * s) for s in grid_size)
    new_width = tuple(int(toep_oversamp * p) for p in padded)
    g = prep_locs(locs.to(dtype), grid_size, padded)
    g = rescale_locs(g, [p // 2 for p in padded], padded, [w // 2 for w in new_width], new_width)
    npts = locs.shape[:-1]
    cdt = torch.complex128 if dtype == torch.float64 else torch.complex64
    w = torch.ones(npts, dtype=cdt) if weight is None else weight.to(cdt).expand(npts)
    otf = nufft_adjoint(w, g, new_grid, oversamp, width, dtype, prepared=True)
    sf = toep_oversamp**ndim / prod(new_grid) ** 0.5
    return _cfftn(otf, tuple(range(-ndim, 0)), norm=None) * sf


def toeplitz_normal(x: torch.Tensor, kernel: torch.Tensor, grid_size, toep_oversamp: float = 2.0):
    """crop(cifftn(kernel * cfftn(pad(x)))) with orthonormal centred FFTs
    (``Pad.normal(FFT.normal(Dense(kernel)))``, ``linops/nufft.py:226-239``)."""
    ndim = len(grid_size)
    grid_size = tuple(grid_size)
    new_grid = tuple(int(toep_oversamp * s) for s in grid_size)
    dims = tuple(range(-ndim, 0))
    z = _cfftn(_pad(x.to(kernel.dtype), grid_size, new_grid), dims)
    return _crop(_cfftn(z * kernel, dims, inverse=True), grid_size, new_grid)
