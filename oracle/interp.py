"""CPU restatement of the reference interpolation path (TEST INFRASTRUCTURE ONLY).

Restates, in vectorised torch on the CPU, what the reference computes in
``src/torchlinops/functional/_interp/``:

* ``kaiser_bessel``  <- ``kaiser_bessel_torch`` (kernels.py:28-89): the
  Abramowitz & Stegun 9.8.1 / 9.8.2 polynomial approximation of I0 evaluated at
  ``beta * sqrt(1 - x**2)``; not normalised (KB(1) = 1, KB(0) = I0(beta)).
* ``spline``         <- ``spline_torch`` (kernels.py:92-94).
* ``axis_taps``      <- the tap window of ``ungrid_torch`` / ``grid_torch``
  (ungrid.py:655-661, grid.py:598-605): ``lower = ceil(x - W/2)``, taps
  ``lower + arange(W + 1)``, normalised offset ``(x - g) / (W/2)``, kept while
  ``|d| <= W/2`` (the reference's mask, kernels.py:136) and while the kernel
  value is finite (kernels.py:139 zeroes the NaN of KB beyond ``|d| = 1``).
* ``ungrid`` / ``grid`` <- ``ungrid_torch`` (ungrid.py:624-684) and
  ``grid_torch`` (grid.py:571-639), with ``prep_ungrid_shapes`` /
  ``prep_grid_shapes`` (ungrid.py:577, grid.py:522) for the batch flattening.

Deliberate differences, each because the reference path cannot be run as is:

* norm 2: ``weights_torch`` raises on the CPU (kernels.py:130-133 compares
  tensors of mismatched shape) and the Triton kernels return NaN for the
  corner taps (kernels.py:355-362 never masks ``rho > 1``). Here norm 2 is the
  radial weight ``K(rho)`` with ``rho = sqrt(sum_e d_e**2)`` kept while
  ``rho <= 1`` and every ``|d_e| <= W_e/2``; the CUDA kernels implement the
  same definition.
* the masked weights are formed with ``torch.where`` on clamped arguments
  instead of the in-place ``weights[~isfinite] = 0`` (kernels.py:139), so that
  autograd through the float64 restatement gives the trajectory gradient
  (the reference's own autograd raises on that in-place write).

``dtype=torch.float32`` mirrors the reference arithmetic op for op;
``dtype=torch.float64`` is the FP64 oracle (the same A&S formula in double).
"""

from __future__ import annotations

import math
from math import prod

import torch

__all__ = [
    "kaiser_bessel",
    "spline",
    "kernel_fn",
    "axis_taps",
    "ungrid",
    "grid",
    "grad_locs_interp",
    "grad_locs_adjoint",
    "nufft_beta",
]

# Abramowitz & Stegun, Handbook of Mathematical Functions, 9.8.1 (|z| < 3.75):
# I0(z) ~ sum_k A[k] * (z/3.75)**(2k)
_AS_SMALL = (1.0, 3.5156229, 3.0899424, 1.2067492, 0.2659732, 0.0360768, 0.0045813)
# A&S 9.8.2 (z >= 3.75): I0(z) ~ exp(z) / sqrt(z) * sum_k B[k] * (3.75/z)**k
_AS_BIG = (
    0.39894228,
    0.01328592,
    0.00225319,
    -0.00157565,
    0.00916281,
    -0.02057706,
    0.02635537,
    -0.01647633,
    0.00392377,
)


def nufft_beta(width: float, oversamp: float) -> float:
    """KB shape parameter used by the reference NUFFT (linops/nufft.py:337-346)."""
    return math.pi * (((width / oversamp) * (oversamp - 0.5)) ** 2 - 0.8) ** 0.5


def kaiser_bessel(x: torch.Tensor, beta: float) -> torch.Tensor:
    """KB(x) = I0(beta*sqrt(1-x^2)) by the A&S polynomials (kernels.py:50-89).

    Arguments with ``|x| > 1`` give NaN exactly like the reference; callers
    mask them. Evaluated in ``x.dtype`` in the reference's operation order.
    """
    z = beta * torch.sqrt(1 - x * x)
    small = z < 3.75
    # Clamp each branch's argument so that the unused branch stays finite
    # (keeps autograd through torch.where NaN-free); values are unchanged.
    zs = torch.where(small, z, torch.zeros_like(z))
    zb = torch.where(small, torch.full_like(z, 3.75), z)
    t = zs / 3.75
    t2 = t * t
    t4 = t2 * t2
    t6 = t4 * t2
    t8 = t4 * t4
    t10 = t6 * t4
    t12 = t6 * t6
    a = _AS_SMALL
    s = 1 + a[1] * t2 + a[2] * t4 + a[3] * t6 + a[4] * t8 + a[5] * t10 + a[6] * t12
    u = zb / 3.75
    u2 = u * u
    u3 = u2 * u
    u4 = u2 * u2
    u5 = u3 * u2
    u6 = u4 * u2
    u7 = u5 * u2
    u8 = u4 * u4
    b = _AS_BIG
    poly = (
        b[0]
        + b[1] / u
        + b[2] / u2
        + b[3] / u3
        + b[4] / u4
        + b[5] / u5
        + b[6] / u6
        + b[7] / u7
        + b[8] / u8
    )
    big = torch.exp(zb) / torch.sqrt(zb) * poly
    return torch.where(small, s, big)


def spline(x: torch.Tensor) -> torch.Tensor:
    """Linear spline max(1 - |x|, 0) (kernels.py:92-94)."""
    return torch.clamp(1.0 - torch.abs(x), min=0.0)


def kernel_fn(kernel: str, beta: float):
    if kernel == "kaiser_bessel":
        return lambda x: kaiser_bessel(x, beta)
    if kernel == "spline":
        return spline
    raise ValueError(f"Unrecognized kernel {kernel}")


def _radius(width: float, dtype: torch.dtype) -> torch.Tensor:
    # reference: radius = torch.tensor(width) / 2  (a float32 tensor)
    r = torch.tensor(float(width), dtype=torch.float32) / 2
    return r.to(dtype)


def axis_taps(x: torch.Tensor, width: float, kernel: str, dtype: torch.dtype):
    """Tap window of one axis.

    Returns ``(g, d, valid)``: integer tap coordinates ``g`` [P, NT] (unwrapped),
    normalised offsets ``d = (x - g) / r`` [P, NT] and the validity mask
    ``|d| <= r`` (and ``|d| <= 1`` for Kaiser-Bessel, where the reference's
    kernel value is NaN and zeroed).
    """
    x = x.to(dtype)
    r = _radius(width, dtype)
    lower = torch.ceil(x - r)
    nt = math.ceil(float(width) + 1)
    k = torch.arange(nt, dtype=dtype)
    g = lower[:, None] + k[None, :]
    d = (x[:, None] - g) / r
    valid = torch.abs(d) <= r
    if kernel == "kaiser_bessel":
        valid = valid & (torch.abs(d) <= 1)
    return g.to(torch.int64), d, valid


def _tap_weights(locs, width, kernel, norm, beta, dtype, grid_size, pad_mode):
    """Weights [P, G] and flat grid indices [P, G] for all taps of all points."""
    P, D = locs.shape
    K = kernel_fn(kernel, beta)
    gs, ds, vs = [], [], []
    for e in range(D):
        g, d, v = axis_taps(locs[:, e], width[e], kernel, dtype)
        gs.append(g)
        ds.append(d)
        vs.append(v)
    nts = [g.shape[1] for g in gs]

    def outer(tensors, op):
        out = None
        for e, t in enumerate(tensors):
            shape = [P] + [1] * D
            shape[1 + e] = nts[e]
            te = t.reshape(shape)
            out = te if out is None else op(out, te)
        return out

    valid = outer(vs, torch.logical_and)
    if norm == 1:
        ws = [K(torch.where(v, d, torch.zeros_like(d))) for d, v in zip(ds, vs)]
        w = outer(ws, torch.mul)
        w = torch.where(valid, w, torch.zeros_like(w))
    elif norm == 2:
        rho2 = outer([d * d for d in ds], torch.add)
        rho = torch.sqrt(rho2)
        ok = valid & (rho <= 1)
        w = K(torch.where(ok, rho, torch.zeros_like(rho)))
        w = torch.where(ok, w, torch.zeros_like(w))
    else:
        raise ValueError(f"Unexpected norm: {norm}.")

    # Edge behaviour (kernels.py:141-146)
    in_range = [(g >= 0) & (g < n) for g, n in zip(gs, grid_size)]
    if pad_mode == "zero":
        w = torch.where(outer(in_range, torch.logical_and), w, torch.zeros_like(w))
    elif pad_mode != "circular":
        raise ValueError(f"Unrecognized pad_mode {pad_mode}")
    wrapped = [torch.remainder(g, n) for g, n in zip(gs, grid_size)]
    flat = None
    for e in range(D):
        shape = [P] + [1] * D
        shape[1 + e] = nts[e]
        term = wrapped[e].reshape(shape)
        flat = term if flat is None else flat * grid_size[e] + term
    flat = flat.expand(w.shape)
    return w.reshape(P, -1), flat.reshape(P, -1)


def _prep_width(width, ndim):
    if isinstance(width, (int, float)):
        return (float(width),) * ndim
    width = tuple(float(w) for w in width)
    if len(width) != ndim:
        raise ValueError("width tuple must have one entry per grid dimension")
    return width


def _cplx(dtype: torch.dtype) -> torch.dtype:
    return torch.complex128 if dtype == torch.float64 else torch.complex64


def ungrid(
    vals: torch.Tensor,
    locs: torch.Tensor,
    width,
    kernel: str = "kaiser_bessel",
    norm: int = 1,
    pad_mode: str = "circular",
    beta: float = 1.0,
    dtype: torch.dtype = torch.float32,
    chunk: int = 1 << 15,
) -> torch.Tensor:
    """Forward interpolation (grid -> points), reference ungrid.py:37-67,624-684."""
    ndim = locs.shape[-1]
    grid_size = tuple(vals.shape[-ndim:])
    batch_shape = vals.shape[:-ndim]
    width = _prep_width(width, ndim)
    locs_batch_shape = locs.shape[:-1]
    npts = prod(locs_batch_shape)
    is_complex = vals.is_complex()
    vdt = _cplx(dtype) if is_complex else dtype
    v = vals.reshape(-1, prod(grid_size)).to(vdt)
    L = locs.reshape(npts, ndim)
    out = torch.zeros(v.shape[0], npts, dtype=vdt)
    for p0 in range(0, npts, chunk):
        p1 = min(npts, p0 + chunk)
        w, idx = _tap_weights(L[p0:p1], width, kernel, norm, beta, dtype, grid_size, pad_mode)
        gathered = v[:, idx]  # [B, P, G]
        out[:, p0:p1] = (w.to(vdt)[None] * gathered).sum(-1)
    return out.reshape(*batch_shape, *locs_batch_shape)


def grid(
    vals: torch.Tensor,
    locs: torch.Tensor,
    grid_size,
    width,
    kernel: str = "kaiser_bessel",
    norm: int = 1,
    pad_mode: str = "circular",
    beta: float = 1.0,
    dtype: torch.dtype = torch.float32,
    chunk: int = 1 << 15,
) -> torch.Tensor:
    """Adjoint interpolation (points -> grid), reference grid.py:37-72,571-639."""
    grid_size = tuple(int(s) for s in grid_size)
    ndim = len(grid_size)
    if locs.shape[-1] != ndim:
        raise ValueError(
            f"Expected last dim of locs: to equal ndim but got locs.shape[-1] {locs.shape[-1]} != ndim {ndim}"
        )
    width = _prep_width(width, ndim)
    locs_batch_shape = locs.shape[:-1]
    npts = prod(locs_batch_shape)
    batch_shape = vals.shape[: vals.ndim - len(locs_batch_shape)]
    is_complex = vals.is_complex()
    vdt = _cplx(dtype) if is_complex else dtype
    v = vals.reshape(-1, npts).to(vdt)
    L = locs.reshape(npts, ndim)
    out = torch.zeros(v.shape[0], prod(grid_size), dtype=vdt)
    for p0 in range(0, npts, chunk):
        p1 = min(npts, p0 + chunk)
        w, idx = _tap_weights(L[p0:p1], width, kernel, norm, beta, dtype, grid_size, pad_mode)
        contrib = w.to(vdt)[None] * v[:, p0:p1, None]  # [B, P, G]
        out.index_add_(1, idx.reshape(-1), contrib.reshape(v.shape[0], -1))
    return out.reshape(*batch_shape, *grid_size)


def grad_locs_interp(img, a, locs, width, kernel="kaiser_bessel", norm=1, pad_mode="circular", beta=1.0):
    """d/dlocs of sum Re(conj(a) * ungrid(img, locs)), by autograd in float64."""
    L = locs.detach().to(torch.float64).clone().requires_grad_(True)
    out = ungrid(img.detach(), L, width, kernel, norm, pad_mode, beta, dtype=torch.float64)
    a64 = a.detach().to(out.dtype)
    loss = (a64.conj() * out).real.sum() if out.is_complex() else (a64 * out).sum()
    (g,) = torch.autograd.grad(loss, L)
    return g


def grad_locs_adjoint(vals, b, locs, grid_size, width, kernel="kaiser_bessel", norm=1, pad_mode="circular", beta=1.0):
    """d/dlocs of sum Re(conj(b) * grid(vals, locs)), by autograd in float64."""
    L = locs.detach().to(torch.float64).clone().requires_grad_(True)
    out = grid(vals.detach(), L, grid_size, width, kernel, norm, pad_mode, beta, dtype=torch.float64)
    b64 = b.detach().to(out.dtype)
    loss = (b64.conj() * out).real.sum() if out.is_complex() else (b64 * out).sum()
    (g,) = torch.autograd.grad(loss, L)
    return g
