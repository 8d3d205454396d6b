"""Conjugate gradients in float64 on the CPU (TEST INFRASTRUCTURE ONLY).

Textbook CG on a Hermitian positive definite operator, the algorithm of the
reference's ``conjugate_gradients`` (``alg/pcg.py:13-90``: ``r = b - A x``,
``p = r``, ``alpha = <r, r> / <p, A p>``, ``beta = <r', r'> / <r, r>``) with
every vector and scalar in float64 / complex128, stopping on the relative
residual |r| / |b|.
"""

from __future__ import annotations

import torch

__all__ = ["cg"]


def cg(A, b: torch.Tensor, x0=None, rtol: float = 1e-10, max_iters: int = 1000):
    b = b.to(torch.complex128 if b.is_complex() else torch.float64)
    x = torch.zeros_like(b) if x0 is None else x0.to(b.dtype).clone()
    r = b - A(x)
    p = r.clone()
    rs = torch.vdot(r.flatten(), r.flatten()).real
    bn = torch.linalg.vector_norm(b)
    it = 0
    while it < max_iters and torch.sqrt(rs) > rtol * bn:
        Ap = A(p)
        alpha = rs / torch.vdot(p.flatten(), Ap.flatten()).real
        x = x + alpha * p
        r = r - alpha * Ap
        rs_new = torch.vdot(r.flatten(), r.flatten()).real
        p = r + (rs_new / rs) * p
        rs = rs_new
        it += 1
    return x, it
