"""The fused flexible preconditioned CG (tlgb_pcg_update, tlgb_pcg_direction)
against the same iteration in float64 torch."""

import pytest
import torch

from torchlinops_gb300 import alg

pytestmark = pytest.mark.gpu
DEV = "cuda"


def test_flexible_pcg_matches_a_float64_reference():
    """The fused flexible-PCG kernels against the same iteration in float64
    torch (Polak-Ribiere beta with r_new - r_old = -alpha Ap), on a complex
    SPD system with a fixed SPD diagonal preconditioner: the iterates agree
    to float32 rounding over the first iterations, and the solve converges
    judged by its float64 true residual."""
    gen = torch.Generator().manual_seed(11)
    n = 300
    Q, _ = torch.linalg.qr(torch.randn(n, n, dtype=torch.complex128, generator=gen))
    Mat = (Q * torch.logspace(0, 2, n, dtype=torch.float64)) @ Q.conj().T
    dvec = 1.0 / torch.diagonal(Mat).real
    xt = torch.randn(n, dtype=torch.complex128, generator=gen)
    b64 = Mat @ xt
    A32 = Mat.to(torch.complex64).to(DEV)
    d32 = dvec.to(torch.float32).to(DEV)
    A = lambda v: A32 @ v  # noqa: E731
    M = lambda v: d32 * v  # noqa: E731
    x, info = alg.cg_solve(A, b64.to(torch.complex64).to(DEV), rtol=1e-5, max_iters=500, M=M, check_every=1)
    assert info.converged and info.true_rel_residual <= 1e-5 and not info.fallback
    # the same iteration in float64 for 5 steps
    Ad = Mat.to(DEV)
    dd = dvec.to(DEV)
    bd = b64.to(DEV)
    x64 = torch.zeros_like(bd)
    r = bd.clone()
    z = dd * r
    p = z.clone()
    rz = torch.vdot(r, z).real
    for _ in range(5):
        Ap = Ad @ p
        a = rz / torch.vdot(p, Ap).real
        x64 = x64 + a * p
        r = r - a * Ap
        z = dd * r
        rz_new = torch.vdot(r, z).real
        beta = torch.clamp(-a * torch.vdot(Ap, z).real / rz, min=0.0)
        p = z + beta * p
        rz = rz_new
    x5, info5 = alg.cg_solve(A, b64.to(torch.complex64).to(DEV), rtol=1e-30, max_iters=5, M=M, check_every=5)
    assert info5.iters == 5
    rel = float(torch.linalg.vector_norm(x5.to(torch.complex128) - x64) / torch.linalg.vector_norm(x64))
    assert rel < 1e-4, rel
