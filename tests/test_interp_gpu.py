"""Parity of the CUDA interpolation kernels with the reference and the oracle.

Tolerance: 1e-5 relative L2 in complex64/float32 against the reference's own
torch path (golden vectors) and the float32 oracle; the FP64 oracle error is
checked alongside. Gridding must be bit-identical run to run.
"""

import math

import numpy as np
import pytest
import torch

from conftest import GOLDEN, load_cases, rel_l2, to_torch
from oracle import interp as OI

import torchlinops_gb300 as T

pytestmark = pytest.mark.gpu
TOL = 1e-5
DEV = "cuda"
INTERP = load_cases("interp_cases.npz")


def _kw(m):
    w = m["width"] if not isinstance(m["width"], list) else tuple(m["width"])
    return w, dict(kernel=m["kernel"], norm=1, pad_mode=m["pad_mode"], kernel_params=dict(beta=m["beta"]))


@pytest.mark.parametrize("case", sorted(INTERP))
def test_interp_matches_reference_golden(case):
    rec = INTERP[case]
    m = rec["meta"]
    cplx = m["complex"]
    locs = torch.from_numpy(rec["locs"]).to(DEV)
    img = to_torch(rec["img"], cplx).to(DEV)
    pts = to_torch(rec["pts"], cplx).to(DEV)
    w, kw = _kw(m)
    fwd = T.interpolate(img, locs, w, **kw)
    adj = T.interpolate_adjoint(pts, locs, tuple(m["grid_size"]), w, **kw)
    ref_fwd = to_torch(rec["fwd"], cplx)
    ref_adj = to_torch(rec["adj"], cplx)
    assert fwd.shape == ref_fwd.shape and adj.shape == ref_adj.shape
    assert fwd.dtype == ref_fwd.dtype and adj.dtype == ref_adj.dtype
    assert rel_l2(fwd.cpu(), ref_fwd) < TOL
    assert rel_l2(adj.cpu(), ref_adj) < TOL
    # error against the FP64 oracle stays at float32 level
    okw = dict(kernel=m["kernel"], norm=1, pad_mode=m["pad_mode"], beta=m["beta"])
    f64 = OI.ungrid(img.cpu(), locs.cpu(), w, dtype=torch.float64, **okw)
    assert rel_l2(fwd.cpu(), f64) < TOL


def test_config1_plain_2d():
    d = np.load(f"{GOLDEN}/config1_interp2d.npz")
    locs = torch.from_numpy(d["locs"]).to(DEV)
    img = to_torch(d["img"], True).to(DEV)
    pts = to_torch(d["pts"], True).to(DEV)
    kp = dict(beta=float(d["beta"]))
    fwd = T.interpolate(img, locs, 4.0, kernel_params=kp)
    adj = T.interpolate_adjoint(pts, locs, (64, 64), 4.0, kernel_params=kp)
    assert rel_l2(fwd.cpu(), to_torch(d["fwd"], True)) < TOL
    assert rel_l2(adj.cpu(), to_torch(d["adj"], True)) < TOL


@pytest.mark.parametrize("cplx", [False, True])
def test_exact_integer_location(cplx):
    d = np.load(f"{GOLDEN}/edge_intloc.npz")
    tag = "c" if cplx else "r"
    dt = torch.complex64 if cplx else torch.float32
    vals = torch.arange(1, 9).to(dt).to(DEV)
    locs = torch.tensor([[4.0]], device=DEV)
    fwd = T.ungrid(vals, locs, width=4.0, kernel="kaiser_bessel")
    adj = T.grid(torch.tensor([[1.0]]).to(dt).to(DEV), locs, (8,), width=4.0, kernel="kaiser_bessel")
    torch.testing.assert_close(fwd.cpu(), to_torch(d[f"fwd_{tag}"], cplx), rtol=1e-6, atol=0)
    torch.testing.assert_close(adj.cpu(), to_torch(d[f"adj_{tag}"], cplx), rtol=1e-6, atol=0)


def _ball_locs(n, radius, centre, gen, ndim=3):
    r = torch.rand(n, generator=gen) * radius
    u = torch.randn(n, ndim, generator=gen)
    u = u / u.norm(dim=-1, keepdim=True)
    return (centre + r[:, None] * u).to(torch.float32)


@pytest.mark.parametrize("ndim,n,npts,nb", [(3, 48, 60000, 4), (2, 160, 80000, 3), (1, 700, 30000, 9)])
@pytest.mark.parametrize("pad", ["circular", "zero"])
def test_dense_centre_against_oracle(ndim, n, npts, nb, pad):
    """1/r^2 density: dense tiles are split into parts and summed in order."""
    gen = torch.Generator().manual_seed(ndim * 7 + len(pad))
    locs = _ball_locs(npts, n / 2 + 1.5, n / 2, gen, ndim)
    img = torch.complex(torch.randn(nb, *(n,) * ndim, generator=gen), torch.randn(nb, *(n,) * ndim, generator=gen))
    pts = torch.complex(torch.randn(nb, npts, generator=gen), torch.randn(nb, npts, generator=gen))
    beta = OI.nufft_beta(4.0, 1.25)
    kw = dict(kernel="kaiser_bessel", pad_mode=pad)
    fwd = T.ungrid(img.to(DEV), locs.to(DEV), 4.0, kernel_params=dict(beta=beta), **kw).cpu()
    adj = T.grid(pts.to(DEV), locs.to(DEV), (n,) * ndim, 4.0, kernel_params=dict(beta=beta), **kw).cpu()
    o32f = OI.ungrid(img, locs, 4.0, beta=beta, **kw)
    o64f = OI.ungrid(img, locs, 4.0, beta=beta, dtype=torch.float64, **kw)
    o32a = OI.grid(pts, locs, (n,) * ndim, 4.0, beta=beta, **kw)
    o64a = OI.grid(pts, locs, (n,) * ndim, 4.0, beta=beta, dtype=torch.float64, **kw)
    assert rel_l2(fwd, o32f) < TOL and rel_l2(fwd, o64f) < TOL
    assert rel_l2(adj, o32a) < TOL and rel_l2(adj, o64a) < TOL


@pytest.mark.parametrize("shape", [(40, 36, 48), (40, 36, 45)])
@pytest.mark.parametrize("nb", [1, 2, 4, 8, 11])
@pytest.mark.parametrize("pad", ["circular", "zero"])
@pytest.mark.parametrize("kernel", ["kaiser_bessel", "spline"])
def test_eight_entry_3d_paths_against_oracle(shape, nb, pad, kernel):
    """3D, 8 complex entries per group: the TMA-staged gather (even Z) and its
    plain-load fallback (odd Z, wrapping edge regions), a ragged last group,
    batches below 8 entries run as one partly empty group, dense split
    tiles, points across every edge and exact-integer points."""
    from torchlinops_gb300 import _ext

    gen = torch.Generator().manual_seed(nb + len(pad) + shape[2])
    n = torch.tensor(shape, dtype=torch.float32)
    ball = _ball_locs(30000, 6.0, n / 2, gen)
    spread = torch.rand(20000, 3, generator=gen) * (n + 4) - 2  # edges and a little outside
    ints = torch.randint(0, min(shape), (500, 3), generator=gen).to(torch.float32)
    locs = torch.cat([ball, spread, ints])
    npts = locs.shape[0]
    img = torch.complex(torch.randn(nb, *shape, generator=gen), torch.randn(nb, *shape, generator=gen))
    pts = torch.complex(torch.randn(nb, npts, generator=gen), torch.randn(nb, npts, generator=gen))
    beta = OI.nufft_beta(4.0, 1.25)
    kw = dict(kernel=kernel, pad_mode=pad)
    _ext.device_status(clear=True)
    fwd = T.ungrid(img.to(DEV), locs.to(DEV), 4.0, kernel_params=dict(beta=beta), **kw).cpu()
    adj = T.grid(pts.to(DEV), locs.to(DEV), shape, 4.0, kernel_params=dict(beta=beta), **kw).cpu()
    assert _ext.device_status() == 0
    o32f = OI.ungrid(img, locs, 4.0, beta=beta, **kw)
    o64f = OI.ungrid(img, locs, 4.0, beta=beta, dtype=torch.float64, **kw)
    o32a = OI.grid(pts, locs, shape, 4.0, beta=beta, **kw)
    o64a = OI.grid(pts, locs, shape, 4.0, beta=beta, dtype=torch.float64, **kw)
    assert rel_l2(fwd, o32f) < TOL and rel_l2(fwd, o64f) < TOL
    assert rel_l2(adj, o32a) < TOL and rel_l2(adj, o64a) < TOL


@pytest.mark.parametrize("shape", [(160, 144), (90, 61)])
@pytest.mark.parametrize("nb", [1, 4, 8, 11])
@pytest.mark.parametrize("pad", ["circular", "zero"])
@pytest.mark.parametrize("kernel", ["kaiser_bessel", "spline"])
def test_eight_entry_2d_paths_against_oracle(shape, nb, pad, kernel):
    """2D, 8 complex entries per group: the TMA-staged gather (even Z) and its
    plain-load fallback (odd Z, wrapping edge regions), a ragged last group,
    batches below 8 entries run as one partly empty group, dense tiles,
    points across every edge and exact-integer points."""
    from torchlinops_gb300 import _ext

    gen = torch.Generator().manual_seed(nb + len(pad) + shape[1])
    n = torch.tensor(shape, dtype=torch.float32)
    ball = _ball_locs(20000, 10.0, n / 2, gen, ndim=2)
    spread = torch.rand(20000, 2, generator=gen) * (n + 4) - 2  # edges and a little outside
    ints = torch.randint(0, min(shape), (500, 2), generator=gen).to(torch.float32)
    locs = torch.cat([ball, spread, ints])
    npts = locs.shape[0]
    img = torch.complex(torch.randn(nb, *shape, generator=gen), torch.randn(nb, *shape, generator=gen))
    pts = torch.complex(torch.randn(nb, npts, generator=gen), torch.randn(nb, npts, generator=gen))
    beta = OI.nufft_beta(4.0, 1.25)
    kw = dict(kernel=kernel, pad_mode=pad)
    _ext.device_status(clear=True)
    fwd = T.ungrid(img.to(DEV), locs.to(DEV), 4.0, kernel_params=dict(beta=beta), **kw).cpu()
    adj = T.grid(pts.to(DEV), locs.to(DEV), shape, 4.0, kernel_params=dict(beta=beta), **kw).cpu()
    assert _ext.device_status() == 0
    assert rel_l2(fwd, OI.ungrid(img, locs, 4.0, beta=beta, **kw)) < TOL
    assert rel_l2(fwd, OI.ungrid(img, locs, 4.0, beta=beta, dtype=torch.float64, **kw)) < TOL
    assert rel_l2(adj, OI.grid(pts, locs, shape, 4.0, beta=beta, **kw)) < TOL
    assert rel_l2(adj, OI.grid(pts, locs, shape, 4.0, beta=beta, dtype=torch.float64, **kw)) < TOL


@pytest.mark.parametrize("nb", [8, 3, 1])
@pytest.mark.parametrize("kernel", ["kaiser_bessel", "spline"])
def test_grid_nonfinite_values_stay_in_their_windows(kernel, nb):
    """A NaN or Inf point value turns exactly the cells of its window
    non-finite (its valid taps, zero-weight ones included) and no other cell:
    the 3D block paths (8 entries, and 1, 2 or 4), whose rows of tap weights
    hold zeros outside a window, send such points through the per-tap path. The reference's own
    torch path multiplies every tap of the ceil(W+1)^3 patch by the value,
    masked taps included (grid.py:624, weights * mask * val), so there a NaN
    reaches the whole patch: a superset of the window."""
    gen = torch.Generator().manual_seed(9)
    shape = (32, 32, 32)
    locs = _ball_locs(20000, 12.0, torch.tensor([16.0, 16.0, 16.0]), gen)
    pts = torch.complex(torch.randn(nb, 20000, generator=gen), torch.randn(nb, 20000, generator=gen))
    bad = [(3 % nb, 17, complex(float("nan"), 0.0)), (5 % nb, 900, complex(float("inf"), 1.0)),
           (0, 4000, complex(0.0, float("-inf")))]
    for c, p, v in bad:
        pts[c, p] = v
    beta = OI.nufft_beta(4.0, 1.25)
    out = T.grid(pts.to(DEV), locs.to(DEV), shape, 4.0, kernel=kernel, kernel_params=dict(beta=beta)).cpu()
    ref = OI.grid(pts, locs, shape, 4.0, kernel=kernel, beta=beta)
    window = torch.zeros(nb, *shape, dtype=torch.bool)
    for c, p, _ in bad:
        taps = []
        for e in range(3):
            g, _d, ok = OI.axis_taps(locs[p : p + 1, e], 4.0, kernel, torch.float32)
            taps.append(g[0][ok[0]] % shape[e])
        for x, y, z in torch.cartesian_prod(*taps).tolist():
            window[c, x, y, z] = True
    assert torch.equal(~torch.isfinite(out), window)
    assert bool((~torch.isfinite(ref))[window].all())
    fin = torch.isfinite(ref)
    assert rel_l2(out[fin], ref[fin]) < TOL


@pytest.mark.parametrize("nb", [8, 4, 1])
def test_gridding_is_deterministic(nb):
    gen = torch.Generator().manual_seed(5)
    locs = _ball_locs(200000, 33, 32, gen).to(DEV)
    pts = torch.randn(nb, 200000, dtype=torch.complex64, generator=gen).to(DEV)
    a = T.grid(pts, locs, (64, 64, 64), 4.0)
    T.clear_plan_cache()
    b = T.grid(pts, locs, (64, 64, 64), 4.0)
    c = T.grid(pts, locs, (64, 64, 64), 4.0)
    assert torch.equal(a, b) and torch.equal(b, c)


@pytest.mark.parametrize("kernel", ["kaiser_bessel", "spline"])
@pytest.mark.parametrize("ndim", [1, 2, 3])
@pytest.mark.parametrize("pad", ["circular", "zero"])
def test_norm2_against_oracle(kernel, ndim, pad):
    gen = torch.Generator().manual_seed(11 + ndim)
    n = (12, 10, 9)[:ndim]
    locs = torch.stack([torch.rand(300, generator=gen) * (s + 4) - 2 for s in n], -1)
    img = torch.randn(2, *n, dtype=torch.complex64, generator=gen)
    pts = torch.randn(2, 300, dtype=torch.complex64, generator=gen)
    kp = dict(beta=3.0)
    fwd = T.ungrid(img.to(DEV), locs.to(DEV), 4.0, kernel, 2, pad, kp).cpu()
    adj = T.grid(pts.to(DEV), locs.to(DEV), n, 4.0, kernel, 2, pad, kp).cpu()
    assert rel_l2(fwd, OI.ungrid(img, locs, 4.0, kernel, 2, pad, 3.0, dtype=torch.float64)) < TOL
    assert rel_l2(adj, OI.grid(pts, locs, n, 4.0, kernel, 2, pad, 3.0, dtype=torch.float64)) < TOL


def _safe_points(n, size, width, gen, ndim):
    """Points at least 1e-3 away from any tap-window edge (FD steps stay smooth)."""
    out = []
    while len(out) < n:
        x = torch.rand(ndim, generator=gen) * (size - 1)
        frac = (x - width / 2) - torch.floor(x - width / 2)
        if torch.all((frac > 2e-3) & (frac < 1 - 2e-3)):
            out.append(x)
    return torch.stack(out).to(torch.float32)


@pytest.mark.parametrize("ndim", [1, 2, 3])
@pytest.mark.parametrize("kernel,norm", [("kaiser_bessel", 1), ("spline", 1), ("kaiser_bessel", 2)])
def test_trajectory_gradient(ndim, kernel, norm):
    gen = torch.Generator().manual_seed(3 * ndim + norm)
    size = (20, 18, 16)[:ndim]
    locs = _safe_points(200, min(size), 4.0, gen, ndim)
    img = torch.randn(3, *size, dtype=torch.complex64, generator=gen)
    a = torch.randn(3, 200, dtype=torch.complex64, generator=gen)
    kp = dict(beta=OI.nufft_beta(4.0, 1.25))
    L = locs.to(DEV).requires_grad_(True)
    out = T.interpolate(img.to(DEV), L, 4.0, kernel, norm, "circular", kp)
    (out.conj() * a.to(DEV)).real.sum().backward()
    # Re(conj(out) a) = Re(conj(a) out): the oracle's loss
    ref = OI.grad_locs_interp(img, a, locs, 4.0, kernel, norm, "circular", kp["beta"])
    assert rel_l2(L.grad.cpu(), ref) < 2e-5
    # adjoint operator: gradient of Re(conj(b) * grid(vals))
    vals = torch.randn(3, 200, dtype=torch.complex64, generator=gen)
    b = torch.randn(3, *size, dtype=torch.complex64, generator=gen)
    L2 = locs.to(DEV).requires_grad_(True)
    g = T.interpolate_adjoint(vals.to(DEV), L2, size, 4.0, kernel, norm, "circular", kp)
    (g.conj() * b.to(DEV)).real.sum().backward()
    ref2 = OI.grad_locs_adjoint(vals, b, locs, size, 4.0, kernel, norm, "circular", kp["beta"])
    assert rel_l2(L2.grad.cpu(), ref2) < 2e-5


@pytest.mark.parametrize("nb", [8, 11])
@pytest.mark.parametrize("pad", ["circular", "zero"])
@pytest.mark.parametrize("kernel", ["kaiser_bessel", "spline"])
def test_trajectory_gradient_2d_eight_entry_path(nb, pad, kernel):
    """d/dlocs of both operators on the 2D 8-entry path (gradient records,
    TMA-staged regions, one partial per coil group added in order), against
    the FP64 autograd restatement. Points stay clear of tap-window edges,
    where the kernels' derivatives are singular (Kaiser-Bessel) or undefined
    (spline); in z they reach the upper edge, where circular windows wrap."""
    gen = torch.Generator().manual_seed(nb + len(pad) + len(kernel))
    size = (48, 40)
    locs = _safe_points(4000, 40, 4.0, gen, 2)
    npts = locs.shape[0]
    img = torch.complex(torch.randn(nb, *size, generator=gen), torch.randn(nb, *size, generator=gen))
    a = torch.complex(torch.randn(nb, npts, generator=gen), torch.randn(nb, npts, generator=gen))
    beta = OI.nufft_beta(4.0, 1.25)
    kw = dict(kernel=kernel, pad_mode=pad)
    L = locs.to(DEV).requires_grad_(True)
    out = T.interpolate(img.to(DEV), L, 4.0, kernel_params=dict(beta=beta), **kw)
    (a.to(DEV).conj() * out).real.sum().backward()
    ref = OI.grad_locs_interp(img, a, locs, 4.0, kernel, 1, pad, beta)
    assert rel_l2(L.grad.cpu(), ref) < 1e-4
    # the gridding operator: grid := cotangent, a := point values
    vals = a
    b = torch.complex(torch.randn(nb, *size, generator=gen), torch.randn(nb, *size, generator=gen))
    L2 = locs.to(DEV).requires_grad_(True)
    g = T.interpolate_adjoint(vals.to(DEV), L2, size, 4.0, kernel_params=dict(beta=beta), **kw)
    (b.to(DEV).conj() * g).real.sum().backward()
    ref2 = OI.grad_locs_adjoint(vals, b, locs, size, 4.0, kernel, 1, pad, beta)
    assert rel_l2(L2.grad.cpu(), ref2) < 1e-4


@pytest.mark.parametrize("ndim,norm,nb", [(3, 1, 24), (2, 2, 20)])
def test_trajectory_gradient_split_over_coil_groups(ndim, norm, nb):
    """The generic gradient kernel with several coil groups of 8 entries,
    split over CTAs with partial sums added in a fixed order, against the
    FP64 autograd restatement."""
    gen = torch.Generator().manual_seed(40 + ndim)
    n = 24 if ndim == 3 else 48
    size = (n,) * ndim
    locs = _safe_points(3000, n, 4.0, gen, ndim)
    img = torch.complex(torch.randn(nb, *size, generator=gen), torch.randn(nb, *size, generator=gen))
    a = torch.complex(torch.randn(nb, 3000, generator=gen), torch.randn(nb, 3000, generator=gen))
    kp = dict(beta=OI.nufft_beta(4.0, 1.25))
    L = locs.to(DEV).requires_grad_(True)
    out = T.interpolate(img.to(DEV), L, 4.0, norm=norm, kernel_params=kp)
    (a.to(DEV).conj() * out).real.sum().backward()
    ref = OI.grad_locs_interp(img, a, locs, 4.0, "kaiser_bessel", norm, "circular", kp["beta"])
    assert rel_l2(L.grad.cpu(), ref) < 1e-4
    L2 = locs.to(DEV).requires_grad_(True)
    out2 = T.interpolate(img.to(DEV), L2, 4.0, norm=norm, kernel_params=kp)
    (a.to(DEV).conj() * out2).real.sum().backward()
    assert torch.equal(L.grad, L2.grad)  # fixed order of the partial sums


def test_batch_above_one_call_is_split():
    """A batch of MAX_BATCH + 3 entries (above one call of the C ABI) runs as
    two calls of MAX_BATCH and 3 entries: the forward and adjoint against the
    FP64 oracle on the entries either side of the split, and the trajectory
    gradient, a sum over the whole batch, against the FP64 restatement. The
    last 3 cotangent rows are scaled by 300 so that both calls carry a large
    share of the gradient."""
    from torchlinops_gb300 import interp as I

    M = I.MAX_BATCH
    nb, n, npts = M + 3, 16, 3
    gen = torch.Generator().manual_seed(12)
    locs = _safe_points(npts, n, 4.0, gen, 1)
    img = torch.randn(nb, n, dtype=torch.complex64, generator=gen)
    pts = torch.randn(nb, npts, dtype=torch.complex64, generator=gen)
    pts[M:] *= 300
    beta = OI.nufft_beta(4.0, 1.25)
    kp = dict(beta=beta)
    idx = torch.tensor([0, M - 1, M, M + 2])
    L = locs.to(DEV).requires_grad_(True)
    fwd = T.interpolate(img.to(DEV), L, 4.0, kernel_params=kp)
    assert fwd.shape == (nb, npts)
    assert rel_l2(fwd.detach().cpu()[idx], OI.ungrid(img[idx], locs, 4.0, beta=beta, dtype=torch.float64)) < TOL
    adj = T.interpolate_adjoint(pts.to(DEV), locs.to(DEV), (n,), 4.0, kernel_params=kp).cpu()
    assert adj.shape == (nb, n)
    assert rel_l2(adj[idx], OI.grid(pts[idx], locs, (n,), 4.0, beta=beta, dtype=torch.float64)) < TOL
    (pts.to(DEV).conj() * fwd).real.sum().backward()
    ref = OI.grad_locs_interp(img, pts, locs, 4.0, "kaiser_bessel", 1, "circular", beta)
    assert rel_l2(L.grad.cpu(), ref) < 1e-4


def test_trajectory_gradient_finite_differences():
    """d/dx by central differences of the FP64 oracle (h = 1e-4 grid units)."""
    gen = torch.Generator().manual_seed(21)
    size = (24, 24)
    locs = _safe_points(40, 24, 4.0, gen, 2)
    img = torch.randn(2, *size, dtype=torch.complex64, generator=gen)
    a = torch.randn(2, 40, dtype=torch.complex64, generator=gen)
    beta = OI.nufft_beta(4.0, 1.25)
    L = locs.to(DEV).requires_grad_(True)
    out = T.interpolate(img.to(DEV), L, 4.0, kernel_params=dict(beta=beta))
    (a.to(DEV).conj() * out).real.sum().backward()
    h = 1e-4
    fd = torch.zeros(40, 2, dtype=torch.float64)
    for e in range(2):
        for s in (1, -1):
            lp = locs.double().clone()
            lp[:, e] += s * h
            o = OI.ungrid(img, lp, 4.0, beta=beta, dtype=torch.float64)
            fd[:, e] += s * (a.to(torch.complex128).conj() * o).real.sum(0) / (2 * h)
    assert rel_l2(L.grad.cpu(), fd) < 1e-4


def test_vals_gradients_are_the_adjoint():
    """reference _interp/tests/test_interp_diff.py: d/dvals is the other operator."""
    gen = torch.Generator().manual_seed(2)
    locs = (torch.rand(500, 3, generator=gen) * 16).to(DEV)
    x = torch.randn(2, 16, 16, 16, dtype=torch.complex64, generator=gen).to(DEV).requires_grad_(True)
    y = T.interpolate(x, locs, 4.0)
    y.abs().sum().backward()
    ref = T.interpolate_adjoint(torch.sgn(y.detach()), locs, (16, 16, 16), 4.0)
    torch.testing.assert_close(x.grad, ref, rtol=1e-5, atol=1e-5)
    v = torch.randn(2, 500, dtype=torch.complex64, generator=gen).to(DEV).requires_grad_(True)
    g = T.interpolate_adjoint(v, locs, (16, 16, 16), 4.0)
    (g.real.sum() + g.imag.sum()).backward()
    ones = torch.complex(torch.ones(2, 16, 16, 16), torch.ones(2, 16, 16, 16)).to(DEV)
    torch.testing.assert_close(v.grad, T.interpolate(ones, locs, 4.0), rtol=1e-5, atol=1e-5)


def test_adjoint_identity_3d():
    gen = torch.Generator().manual_seed(8)
    locs = (torch.rand(3000, 3, generator=gen) * 30 - 3).to(DEV)
    x = torch.randn(4, 24, 24, 24, dtype=torch.complex128, generator=gen).to(torch.complex64).to(DEV)
    y = torch.randn(4, 3000, dtype=torch.complex64, generator=gen).to(DEV)
    for pad in ("circular", "zero"):
        Ax = T.ungrid(x, locs, 4.0, pad_mode=pad)
        AHy = T.grid(y, locs, (24, 24, 24), 4.0, pad_mode=pad)
        lhs = torch.vdot(Ax.flatten().to(torch.complex128), y.flatten().to(torch.complex128))
        rhs = torch.vdot(x.flatten().to(torch.complex128), AHy.flatten().to(torch.complex128))
        assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_invalid_points_read_as_zero():
    locs = torch.tensor([[float("nan"), 1.0], [100.0, 200.0], [3.0, 3.5]], device=DEV)
    img = torch.randn(1, 8, 8, device=DEV)
    out = T.ungrid(img, locs, 4.0, pad_mode="zero")
    assert out[0, 0] == 0 and out[0, 1] == 0 and out[0, 2] != 0
    g = T.grid(torch.ones(1, 3, device=DEV), locs, (8, 8), 4.0, pad_mode="zero")
    assert torch.isfinite(g).all()


def test_errors_match_reference():
    locs = torch.rand(10, 2, device=DEV) * 8
    with pytest.raises(ValueError):
        T.grid(torch.randn(10, device=DEV), locs, (8, 8, 8), 4.0)  # locs dim mismatch
    with pytest.raises(ValueError):
        T.ungrid(torch.randn(8, 8, device=DEV), locs, (4.0, 4.0, 4.0))  # width tuple length
    with pytest.raises(ValueError):
        T.ungrid(torch.randn(8, 8, device=DEV), locs, 4.0, kernel="triangle")
    with pytest.raises(ValueError):
        T.ungrid(torch.randn(8, 8, 8, device=DEV), torch.rand(5, 3, device=DEV), 9.5)  # too wide in 3D


def test_plan_cache_follows_inplace_edits():
    gen = torch.Generator().manual_seed(4)
    locs = (torch.rand(1000, 2, generator=gen) * 32).to(DEV)
    img = torch.randn(32, 32, dtype=torch.complex64, generator=gen).to(DEV)
    a = T.ungrid(img, locs, 4.0)
    locs.add_(0.5)  # bumps the version counter
    b = T.ungrid(img, locs, 4.0)
    ref = OI.ungrid(img.cpu(), locs.cpu(), 4.0)
    assert rel_l2(b.cpu(), ref) < TOL and not torch.allclose(a, b)


def test_plan_records_are_tied_to_the_kernel_parameters():
    """3D plans store each point's tap weights, so a plan is valid for the
    kernel, norm and beta it was built with; the C ABI rejects another beta."""
    import ctypes

    from torchlinops_gb300 import _ext, interp

    gen = torch.Generator().manual_seed(12)
    locs = (torch.rand(5000, 3, generator=gen) * 32).to(DEV)
    img = torch.randn(8, 32, 32, 32, dtype=torch.complex64, generator=gen).to(DEV)
    b1, b2 = 6.99666, 5.0
    plan = interp.get_plan(locs, (32, 32, 32), 4.0, "kaiser_bessel", "circular", b1)
    assert plan.info.off_records > 0
    d = interp._desc(3, (32, 32, 32), (4.0,) * 3, "kaiser_bessel", 1, "circular", b2, True, 8, 5000)
    out = torch.empty(8, 5000, dtype=torch.complex64, device=DEV)
    st = _ext.lib().tlgb_interp_forward(ctypes.byref(d), ctypes.byref(plan.info), _ext.ptr(plan.buffer),
                                         _ext.ptr(locs), _ext.ptr(torch.view_as_real(img)),
                                         _ext.ptr(torch.view_as_real(out)), _ext.stream_ptr(locs.device))
    assert st == _ext.TLGB_ERR_INVALID and b"beta" in _ext.lib().tlgb_last_error()
    # the Python layer keys its plan cache by beta, so both betas just work
    y1 = T.ungrid(img, locs, 4.0, kernel_params=dict(beta=b1)).cpu()
    y2 = T.ungrid(img, locs, 4.0, kernel_params=dict(beta=b2)).cpu()
    assert rel_l2(y2, OI.ungrid(img.cpu(), locs.cpu(), 4.0, beta=b2)) < TOL
    assert rel_l2(y1, OI.ungrid(img.cpu(), locs.cpu(), 4.0, beta=b1)) < TOL
