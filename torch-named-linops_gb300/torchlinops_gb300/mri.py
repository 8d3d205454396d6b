"""3D SENSE reconstruction pieces for the learned-preconditioner CG workload.

Seeded synthetic inputs in the spirit of the reference's MRI tutorial
(``tutorials/mri_reconstruction.py``: Gaussian coil maps, power-method
normalisation, CG on the normal equations), lifted to 3D:

* :func:`radial_trajectory_3d` - 3D radial spokes on Fibonacci-sphere
  directions, readouts spanning [-N/2, N/2);
* :func:`gaussian_coil_maps_3d` - smooth complex sensitivities, normalised;
* :func:`ellipsoid_phantom_3d` - sums of random ellipsoids;
* :class:`SenseNormal` - ``x -> s * sum_c conj(S_c) F^H F (S_c x) + lam x`` on
  this package's NUFFT, with ``s`` from the power method so the largest
  eigenvalue of the data term is 1.
"""

from __future__ import annotations

import math
from typing import Optional

import torch
from torch import Tensor

from . import linops

__all__ = [
    "radial_trajectory_3d",
    "gaussian_coil_maps_3d",
    "ellipsoid_phantom_3d",
    "random_error_field",
    "shell_field",
    "training_batch",
    "cg_solution_pairs",
    "training_manifest",
    "power_method",
    "SenseNormal",
]


def radial_trajectory_3d(nspokes: int, nread: int, n: int, device="cpu") -> Tensor:
    """[nspokes * nread, 3] float32 k-space locations in grid units of an n^3 image."""
    i = torch.arange(nspokes, dtype=torch.float64) + 0.5
    phi = torch.acos(1.0 - 2.0 * i / nspokes)
    theta = math.pi * (1.0 + 5.0**0.5) * i
    dirs = torch.stack([torch.cos(theta) * torch.sin(phi), torch.sin(theta) * torch.sin(phi), torch.cos(phi)], dim=-1)
    r = (torch.arange(nread, dtype=torch.float64) - nread / 2) * (n / nread)
    locs = dirs[:, None, :] * r[None, :, None]
    return locs.reshape(-1, 3).to(torch.float32).to(device)


def gaussian_coil_maps_3d(ncoil: int, n: int, sigma: float = 0.4, device="cpu") -> Tensor:
    """[ncoil, n, n, n] complex64 Gaussian sensitivities centred on a sphere of
    radius 0.3 (unit cube [-0.5, 0.5]^3), with a linear phase; normalised so
    that sum_c |S_c|^2 = 1 everywhere."""
    ax = torch.linspace(-0.5, 0.5, n, dtype=torch.float64)
    X, Y, Z = torch.meshgrid(ax, ax, ax, indexing="ij")
    maps = []
    for c in range(ncoil):
        i = c + 0.5
        phi = math.acos(1.0 - 2.0 * i / ncoil)
        theta = math.pi * (1.0 + 5.0**0.5) * i
        cx, cy, cz = (0.3 * math.cos(theta) * math.sin(phi), 0.3 * math.sin(theta) * math.sin(phi), 0.3 * math.cos(phi))
        g = torch.exp(-((X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2) / (2 * sigma**2))
        ph = torch.exp(1j * 2 * math.pi * (0.1 * X + 0.1 * Y + 0.1 * Z + c / ncoil))
        maps.append(g * ph)
    S = torch.stack(maps)
    S = S / torch.sqrt((S.abs() ** 2).sum(0, keepdim=True))
    return S.to(torch.complex64).to(device)


def ellipsoid_phantom_3d(n: int, n_ellipsoids: int = 10, gen: Optional[torch.Generator] = None, device="cpu") -> Tensor:
    """[n, n, n] complex64 sum of random ellipsoids (random axes, rotation,
    magnitude and phase), seeded by ``gen``."""
    gen = gen if gen is not None else torch.Generator().manual_seed(0)
    ax = torch.linspace(-0.5, 0.5, n, device=device)
    P = torch.stack(torch.meshgrid(ax, ax, ax, indexing="ij"), dim=-1)  # [n, n, n, 3]
    img = torch.zeros(n, n, n, dtype=torch.complex64, device=device)
    for _ in range(n_ellipsoids):
        centre = (torch.rand(3, generator=gen) - 0.5) * 0.6
        axes = 0.05 + torch.rand(3, generator=gen) * 0.25
        q, _ = torch.linalg.qr(torch.randn(3, 3, generator=gen))
        amp = 0.2 + 0.8 * torch.rand(1, generator=gen)
        phase = 2 * math.pi * torch.rand(1, generator=gen)
        u = (P - centre.to(device)) @ q.to(device)
        inside = ((u / axes.to(device)) ** 2).sum(-1) <= 1.0
        val = (amp * torch.exp(1j * phase)).to(torch.complex64).to(device)
        img = img + inside.to(torch.complex64) * val
    return img


def _noise(n: int, gen: torch.Generator, device) -> Tensor:
    """Complex white noise [n, n, n], drawn on the device by a generator that
    the CPU generator ``gen`` seeds (reproducible, and no host-side volume)."""
    seed = int(torch.randint(0, 2**62, (1,), generator=gen))
    dev = torch.device(device)
    g = torch.Generator(device=dev).manual_seed(seed)
    return torch.randn(n, n, n, dtype=torch.complex64, generator=g, device=dev)


def random_error_field(n: int, gen: torch.Generator, device="cpu", a_max: float = 2.0, band: float = 0.5) -> Tensor:
    """A CG-error-like field: a random phantom plus a Gaussian random field
    with a random power-law spectrum |k|^-a, a in [0, a_max], restricted to
    |k| <= band * n (the ball a radial trajectory samples)."""
    ph = ellipsoid_phantom_3d(n, 10, gen, device)
    a = a_max * float(torch.rand(1, generator=gen))
    noise = _noise(n, gen, device)
    k = torch.fft.fftfreq(n, device=device) * n
    KX, KY, KZ = torch.meshgrid(k, k, k, indexing="ij")
    kr = torch.sqrt(KX**2 + KY**2 + KZ**2)
    filt = kr.clamp(min=1.0) ** (-a) * (kr <= band * n)
    field = torch.fft.ifftn(torch.fft.fftn(noise) * filt)
    field = field / torch.linalg.vector_norm(field) * torch.linalg.vector_norm(ph).clamp(min=1e-6)
    w = float(torch.rand(1, generator=gen))
    return (w * ph + (1.0 - w) * field).to(torch.complex64)


def shell_field(n: int, gen: torch.Generator, k_lo: float, k_hi: float, device="cpu") -> Tensor:
    """Complex white noise restricted to the k-space shell k_lo <= |k| < k_hi
    (grid units), unit norm."""
    noise = _noise(n, gen, device)
    k = torch.fft.fftfreq(n, device=device) * n
    KX, KY, KZ = torch.meshgrid(k, k, k, indexing="ij")
    kr = torch.sqrt(KX**2 + KY**2 + KZ**2)
    field = torch.fft.ifftn(torch.fft.fftn(noise) * ((kr >= k_lo) & (kr < k_hi)))
    return (field / torch.linalg.vector_norm(field).clamp(min=1e-30)).to(torch.complex64)


def training_batch(A, n: int, gen: torch.Generator, batch: int = 4, device="cpu"):
    """(r, e) pairs with r = A e for preconditioner training: e from random
    k-space shells inside the sampled ball (so the batch spans the spectrum)
    and one phantom-plus-noise field."""
    pairs = []
    for i in range(batch):
        if i == 0:
            e = random_error_field(n, gen, device, a_max=1.0, band=0.5)
        else:
            c = float(torch.rand(1, generator=gen)) * n / 2
            w = n / 16 + float(torch.rand(1, generator=gen)) * n / 8
            e = shell_field(n, gen, max(c - w / 2, 0.0), max(c + w / 2, 1.0), device)
        pairs.append((A(e), e))
    return pairs


def cg_solution_pairs(A, n: int, count: int, seed: int = 0, rtol: float = 1e-6, max_iters: int = 500,
                      device="cpu", noise: float = 0.05):
    """(r, e) training pairs whose e are solutions that plain CG generates:
    for each of ``count`` seeded 10-ellipsoid phantoms x, the right-hand side
    r = A x + noise (white, ``noise`` times |A x| / sqrt(size)) and e = the
    plain-CG solution of A e = r to relative residual ``rtol``."""
    from . import alg

    pairs = []
    for i in range(count):
        g = torch.Generator().manual_seed(seed + i)
        x = ellipsoid_phantom_3d(n, 10, g, device)
        r = A(x)
        w = torch.complex(torch.randn(r.shape, generator=g), torch.randn(r.shape, generator=g)).to(device)
        r = (r + noise * torch.linalg.vector_norm(r) / math.sqrt(r.numel()) * w).contiguous()
        e, _ = alg.cg_solve(A, r, rtol=rtol, max_iters=max_iters)
        pairs.append((r, e))
    return pairs


def training_manifest(pairs, seed: int = 0, rtol: float = 1e-6, noise: float = 0.05) -> dict:
    """Manifest of :func:`cg_solution_pairs` training data for preconditioner
    checkpoints (``CNNPreconditioner.fit(..., manifest=...)``): the phantom
    seeds, the solver tolerance, the noise level and the SHA-256 of every CG
    solution's bytes, so that a resumed training refuses data that differ
    from what the checkpoint was trained on (other seeds, another operator,
    another solver result)."""
    import hashlib

    sums = [hashlib.sha256(e.detach().to("cpu").contiguous().numpy().tobytes()).hexdigest() for _, e in pairs]
    return {"source": "seeded 10-ellipsoid phantoms (+ white noise) solved by plain CG",
            "phantom_seeds": [seed + i for i in range(len(pairs))], "rtol": rtol, "noise": noise,
            "solution_sha256": sums}


def power_method(A, v: Tensor, iters: int = 30) -> float:
    """Largest eigenvalue of the self-adjoint PSD operator A (alg/powermethod.py:12-60)."""
    v = v / torch.linalg.vector_norm(v)
    lam = 0.0
    for _ in range(iters):
        w = A(v)
        lam = float(torch.linalg.vector_norm(w))
        v = w / lam
    return lam


class SenseNormal:
    """x -> s * sum_c conj(S_c) F^H F (S_c x) + lam * x for an n^3 image.

    F is this package's NUFFT. The coil maps, apodization, pad and both
    centring shifts (the k-space one as a modulation) go in one pass
    (``linops.pad_shift``) and the way back (modulation, shift, crop,
    apodization, conj maps, coil sum, scale and the lam x term) in another
    (``linops.crop_shift``); between them one FFT, one gather, one gridding
    and one inverse FFT for all coils at once."""

    def __init__(self, locs: Tensor, maps: Tensor, lam: float = 1e-3, oversamp: float = 1.25, width: float = 4.0,
                 normalise: bool = True, seed: int = 0):
        self.maps = maps.contiguous()
        self.n = tuple(maps.shape[1:])
        self.F = linops.NUFFT(locs, self.n, oversamp=oversamp, width=width)
        self.lam = lam
        self.scale = 1.0
        if normalise:
            g = torch.Generator().manual_seed(seed)
            v0 = torch.complex(torch.randn(*self.n, generator=g), torch.randn(*self.n, generator=g)).to(maps.device)
            self.scale = 1.0 / power_method(self.data_normal, v0)

    def _normal(self, x: Tensor, lam: float) -> Tensor:
        F = self.F
        z = linops.pad_shift(x, self.n, F.padded_size, maps=self.maps, apod=F.apodize_weight, modulate=True)
        z = torch.fft.fftn(z, dim=(-3, -2, -1), norm="ortho")
        y = F.interp(z)
        g = F.interp.H(y)
        g = torch.fft.ifftn(g, dim=(-3, -2, -1), norm="ortho")
        alpha = self.scale / F.scale_factor**2
        return linops.crop_shift(g, self.n, F.padded_size, maps=self.maps, apod=F.apodize_weight, alpha=alpha,
                                 add=x if lam != 0.0 else None, beta=lam, modulate=True)

    def data_normal(self, x: Tensor) -> Tensor:
        return self._normal(x, 0.0)

    def forward_op(self, x: Tensor) -> Tensor:
        """A x = sqrt(s) F(S x): [ncoil, npts] k-space data."""
        return math.sqrt(self.scale) * self.F(self.maps * x)

    def adjoint_op(self, y: Tensor) -> Tensor:
        return math.sqrt(self.scale) * (self.maps.conj() * self.F.H(y)).sum(0)

    def __call__(self, x: Tensor) -> Tensor:
        return self._normal(x, self.lam)
