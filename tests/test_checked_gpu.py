"""The small parity cases under the range-checked debug build.

libtlgb_checked.so is the library compiled with -DTLGB_CHECKED: selected
global and shared-memory accesses of the interpolation and block kernels
check their index against its range, skip the access when it is out of
range, and record the source line; tlgb_device_status reports that as bit 4.
The cases run in a child process that loads the checked library (the
package loads one library per process): 3D and 2D 8-entry gathers and
gridding, the same kernels with 4 entries, the generic 1D kernels, the
trajectory gradient, unfold / fold with and without a mask. Each must match
the oracle and leave the status word at 0."""

import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CHILD = r"""
import json, sys, torch
sys.path[:0] = PATHS
import torchlinops_gb300 as T
from torchlinops_gb300 import _ext
from oracle import interp as OI, blocks as OB
from conftest import rel_l2
assert _ext.lib_path().endswith("libtlgb_checked.so")
dev = "cuda"
g = torch.Generator().manual_seed(0)
beta = T.kaiser_bessel_beta(4.0, 1.25)
kp = dict(beta=beta)
errs = {}
_ext.device_status(clear=True)
for ndim, n, nb in ((3, 32, 8), (2, 48, 8), (3, 20, 4), (1, 200, 3)):
    npts = 3000
    locs = (torch.rand(npts, ndim, generator=g) * n).float()
    locs[:7] = torch.round(locs[:7])  # exact-integer points: 5-tap windows
    img = torch.randn(nb, *(n,) * ndim, dtype=torch.complex64, generator=g)
    pts = torch.randn(nb, npts, dtype=torch.complex64, generator=g)
    y = T.ungrid(img.to(dev), locs.to(dev), 4.0, kernel_params=kp)
    a = T.grid(pts.to(dev), locs.to(dev), (n,) * ndim, 4.0, kernel_params=kp)
    errs[f"ungrid{ndim}d_{nb}"] = rel_l2(y.cpu(), OI.ungrid(img, locs, 4.0, beta=beta))
    errs[f"grid{ndim}d_{nb}"] = rel_l2(a.cpu(), OI.grid(pts, locs, (n,) * ndim, 4.0, beta=beta))
    if ndim == 2:
        ld = locs.to(dev).requires_grad_(True)
        out = T.interpolate(img.to(dev), ld, 4.0, kernel_params=kp)
        (gl,) = torch.autograd.grad((pts.to(dev).conj() * out).real.sum(), ld)
        ref = OI.grad_locs_interp(img, pts, locs, 4.0, beta=beta)
        # the exact-integer points sit on tap boundaries, where the kernel's
        # derivative is not defined: compare the others
        errs["grad2d"] = rel_l2(gl.cpu().double()[7:], ref[7:])
x = torch.randn(2, 24, 24, 24, dtype=torch.complex64, generator=g)
u = T.unfold(x.to(dev), (8, 8, 8), (4, 4, 4))
errs["unfold"] = 0.0 if torch.equal(u.cpu(), OB.unfold(x, (8, 8, 8), (4, 4, 4))) else 1.0
f = T.fold(u, (24, 24, 24), (8, 8, 8), (4, 4, 4))
errs["fold"] = 0.0 if torch.equal(f.cpu(), OB.fold(u.cpu(), (24, 24, 24), (8, 8, 8), (4, 4, 4))) else 1.0
m = torch.rand(3, 3, 3, generator=g) > 0.4
um = T.unfold(x[0].to(dev), (3, 3, 3), (1, 1, 1), m.to(dev))
errs["unfold_masked"] = 0.0 if torch.equal(um.cpu(), OB.unfold(x[0], (3, 3, 3), (1, 1, 1), m)) else 1.0
fm = T.fold(um, (24, 24, 24), (3, 3, 3), (1, 1, 1), m.to(dev))
errs["fold_masked"] = 0.0 if torch.equal(fm.cpu(), OB.fold(um.cpu(), (24, 24, 24), (3, 3, 3), (1, 1, 1), m)) else 1.0
print(json.dumps({"status": _ext.device_status(), "errs": errs}))
"""


def test_small_parity_cases_under_range_checks():
    from torchlinops_gb300 import _build

    path = _build.build(checked=True)
    env = dict(os.environ, TLGB_LIBRARY=path)
    paths = [ROOT, os.path.join(ROOT, "torch-named-linops_gb300"), os.path.join(ROOT, "tests")]
    src = CHILD.replace("PATHS", repr(paths))
    r = subprocess.run([sys.executable, "-c", src], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    print(res)
    assert res["status"] == 0, f"a checked index was out of range (status {res['status']})"
    assert max(v for k, v in res["errs"].items() if not k.startswith("grad")) < 1e-5, res["errs"]
    assert res["errs"]["grad2d"] < 1e-4
