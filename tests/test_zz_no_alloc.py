"""tlgb_interp_adjoint_fixed: gridding that allocates no device memory.

It exists for callers that cannot allocate device memory at the moment they
grid, e.g. a host framework that only hands out memory from a pool reserved
at start-up, or an FFI caller without an allocator of its own for which
cudaMalloc would synchronise the device mid-pipeline. It must give the same
grid as tlgb_interp_adjoint (which takes the caller's scratch) on every call,
although all calls share one fixed device buffer for the partial tiles of
dense output tiles. This file is collected last so that a run stopping at its
first failure has already run every other test; it also passes on its own.
"""

import ctypes

import pytest
import torch

from conftest import rel_l2

import torchlinops_gb300 as T
from torchlinops_gb300 import _ext, interp

pytestmark = pytest.mark.gpu
DEV = "cuda"
TOL = 1e-5
FIXED_BYTES = 32 << 20  # TLGB_ADJOINT_FIXED_SCRATCH_BYTES


def _dense_case():
    gen = torch.Generator().manual_seed(77)
    n, npts, nb = 64, 200_000, 8
    r = torch.rand(npts, generator=gen) * (n / 2)
    u = torch.randn(npts, 3, generator=gen)
    locs = (n / 2 + r[:, None] * u / u.norm(dim=-1, keepdim=True)).float().to(DEV)
    vals = torch.randn(nb, npts, dtype=torch.complex64, generator=gen).to(DEV)
    return n, locs, vals


def _fixed_call(desc, plan, locs, vals, out):
    L = _ext.lib()
    with torch.cuda.device(out.device):
        return L.tlgb_interp_adjoint_fixed(
            ctypes.byref(desc), ctypes.byref(plan.info), _ext.ptr(plan.buffer), _ext.ptr(locs),
            _ext.ptr(torch.view_as_real(vals)), _ext.ptr(torch.view_as_real(out)), _ext.stream_ptr(out.device),
        )


def test_fixed_scratch_gridding_matches_caller_scratch_gridding():
    n, locs, vals = _dense_case()
    beta = T.kaiser_bessel_beta(4.0, 1.25)
    ref = T.grid(vals, locs, (n, n, n), 4.0, kernel_params=dict(beta=beta))
    plan = interp.get_plan(locs, (n, n, n), 4.0, "kaiser_bessel", "circular", beta)
    assert plan.info.n_blk_partials > 0, "the case must exercise the partial-block scratch"
    desc = interp._desc(3, (n, n, n), (4.0,) * 3, "kaiser_bessel", 1, "circular", beta, True, vals.shape[0],
                        vals.shape[1])
    for _ in range(2):  # the second call sees the first call's buffer contents
        out = torch.full((vals.shape[0], n, n, n), float("nan"), dtype=torch.complex64, device=DEV)
        assert _fixed_call(desc, plan, locs, vals, out) == _ext.TLGB_OK, _ext.lib().tlgb_last_error()
        torch.cuda.synchronize()
        assert rel_l2(out.cpu(), ref.cpu()) <= TOL
        assert torch.equal(out, ref)  # same kernels, fixed summation order


def test_fixed_scratch_rejects_plans_beyond_its_buffer():
    n, locs, vals = _dense_case()
    plan = interp.get_plan(locs, (n, n, n), 4.0, "kaiser_bessel", "circular")
    desc = interp._desc(3, (n, n, n), (4.0,) * 3, "kaiser_bessel", 1, "circular", 1.0, True, vals.shape[0],
                        vals.shape[1])
    big = _ext.PlanInfo()
    ctypes.memmove(ctypes.byref(big), ctypes.byref(plan.info), ctypes.sizeof(big))
    big.n_partials = 1 << 20  # far more partial tiles (and blocks) than the fixed buffer holds
    big.n_blk_partials = 1 << 20
    out = torch.zeros((vals.shape[0], n, n, n), dtype=torch.complex64, device=DEV)

    class _P:
        info = big
        buffer = plan.buffer

    st = _fixed_call(desc, _P, locs, vals, out)
    assert st == _ext.TLGB_ERR_WORKSPACE
    assert b"fixed" in _ext.lib().tlgb_last_error()


@pytest.mark.parametrize("ndim", [3, 2])
def test_fixed_scratch_without_room_for_the_transposed_values(ndim):
    """When the point-major copy of the values does not fit beside the
    partial tiles in the fixed buffer (600,000 points x 64 bytes > 32 MiB),
    the 8-entry gridding kernels stage the values straight from [entry][point]
    order: the same values in the same order, so the same grid bit for bit."""
    gen = torch.Generator().manual_seed(5 + ndim)
    # uniform points: few or no split tiles, so the partial tiles fit
    n, npts, nb = (128 if ndim == 3 else 160), 600_000, 8
    locs = (torch.rand(npts, ndim, generator=gen) * n).float().to(DEV)
    vals = torch.randn(nb, npts, dtype=torch.complex64, generator=gen).to(DEV)
    beta = T.kaiser_bessel_beta(4.0, 1.25)
    size = (n,) * ndim
    ref = T.grid(vals, locs, size, 4.0, kernel_params=dict(beta=beta))
    plan = interp.get_plan(locs, size, 4.0, "kaiser_bessel", "circular", beta)
    desc = interp._desc(ndim, size, (4.0,) * ndim, "kaiser_bessel", 1, "circular", beta, True, nb, npts)
    # the case is the one this test exists for: the partial tiles fit in the
    # fixed buffer, the partial tiles and the point-major values together do not
    sb = ctypes.c_size_t(0)
    assert _ext.lib().tlgb_interp_adjoint_scratch_size(ctypes.byref(desc), ctypes.byref(plan.info),
                                                       ctypes.byref(sb)) == _ext.TLGB_OK
    values_bytes = npts * 64  # one group of 8 complex entries per point
    partial_bytes = sb.value - values_bytes
    assert 0 <= partial_bytes <= FIXED_BYTES < sb.value
    out = torch.full((nb, *size), float("nan"), dtype=torch.complex64, device=DEV)
    st = _fixed_call(desc, plan, locs, vals, out)
    assert st == _ext.TLGB_OK, _ext.lib().tlgb_last_error()
    torch.cuda.synchronize()
    assert torch.equal(out, ref)
