"""Failure detection of the bounded in-kernel waits, in the allowed form: a
wait that runs out with nothing in flight, reported through the device
status word, and a context that stays usable.

The test hook tlgb_test_skip_region_copy makes the TMA-staged kernels (the
3D and 2D 8-entry gathers, the 2D trajectory gradient) launch without their
region copy and poll its mbarrier once, so each CTA's wait gives up at once:
the kernel sets status bit 1 and its CTAs return. Nothing faults, traps or
hangs: there is no copy in flight and no other CTA to wait for."""

import pytest
import torch

from conftest import rel_l2
from oracle import interp as OI

import torchlinops_gb300 as T
from torchlinops_gb300 import _ext, interp

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture
def hook():
    L = _ext.lib()
    yield L
    L.tlgb_test_skip_region_copy(0)
    _ext.device_status(clear=True)


def _case(ndim, gen):
    n, npts = (32, 3000) if ndim == 3 else (48, 4000)
    locs = (torch.rand(npts, ndim, generator=gen) * (n - 12) + 6).float()
    img = torch.randn(8, *(n,) * ndim, dtype=torch.complex64, generator=gen)
    return n, locs, img


@pytest.mark.parametrize("ndim", [3, 2])
def test_bounded_wait_timeout_sets_status_and_context_survives(hook, ndim):
    gen = torch.Generator().manual_seed(40 + ndim)
    n, locs, img = _case(ndim, gen)
    beta = T.kaiser_bessel_beta(4.0, 1.25)
    kp = dict(beta=beta)
    locs_d, img_d = locs.to(DEV), img.to(DEV)
    interp.get_plan(locs_d, (n,) * ndim, 4.0, "kaiser_bessel", "circular", beta)  # built before the hook
    _ext.device_status(clear=True)
    assert hook.tlgb_test_skip_region_copy(1) == 0
    T.ungrid(img_d, locs_d, 4.0, kernel_params=kp)  # the gather's waits run out
    st = _ext.device_status(clear=True)
    assert st & 1, f"status {st}: the timed-out wait was not reported"
    assert hook.tlgb_test_skip_region_copy(0) == 1
    # the context is intact: the same call now completes and matches the oracle
    y = T.ungrid(img_d, locs_d, 4.0, kernel_params=kp)
    assert _ext.device_status() == 0
    assert rel_l2(y.cpu(), OI.ungrid(img, locs, 4.0, beta=beta)) < 1e-5


def test_trajectory_gradient_timeout_is_reported(hook):
    gen = torch.Generator().manual_seed(44)
    n, locs, img = _case(2, gen)
    beta = T.kaiser_bessel_beta(4.0, 1.25)
    kp = dict(beta=beta)
    locs_d = locs.to(DEV).requires_grad_(True)
    a = torch.randn(8, locs.shape[0], dtype=torch.complex64, generator=gen).to(DEV)
    img_d = img.to(DEV)
    y = T.interpolate(img_d, locs_d, 4.0, kernel_params=kp)  # forward without the hook
    _ext.device_status(clear=True)
    hook.tlgb_test_skip_region_copy(1)
    (g,) = torch.autograd.grad((a.conj() * y).real.sum(), locs_d)
    assert _ext.device_status(clear=True) & 1
    hook.tlgb_test_skip_region_copy(0)
    y = T.interpolate(img_d, locs_d, 4.0, kernel_params=kp)
    (g2,) = torch.autograd.grad((a.conj() * y).real.sum(), locs_d)
    assert _ext.device_status() == 0 and torch.isfinite(g2).all()


def test_hook_is_off_by_default():
    assert _ext.lib().tlgb_test_skip_region_copy(0) == 0
