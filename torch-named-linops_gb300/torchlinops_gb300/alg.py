"""Conjugate gradients with float64 scalars on the GPU.

``conjugate_gradients`` keeps the reference signature and stopping rule
(alg/pcg.py:13-88, CGRun :92-176): plain CG on a Hermitian positive
(semi)definite operator, optional loss / gradient-norm tracking with the
``ltol`` / ``gtol`` criteria. What changes is the arithmetic of the scalars:
every inner product accumulates in float64 on the device (``tlgb_dot_f64``)
and alpha, beta and |r|^2 live in a float64 state vector on the device, so an
iteration issues no host synchronisation (the reference forms them in the
input precision, complex64 -> float32, and its tracking reads two scalars to
the host per iteration).

``cg_solve`` adds what a reconstruction needs: a relative-residual stop
``|b - A x| / |b| <= rtol`` checked every ``check_every`` iterations, an
optional (flexible, nonlinear-safe) preconditioner ``M`` with the
Polak-Ribiere beta, and a fallback to plain CG when the preconditioned
iteration stagnates or produces NaN. The float64 true residual
``|b - A x| / |b|`` decides convergence: a solve whose recursive residual
reached ``rtol`` but whose true residual did not continues as plain CG from
its iterate. Scalars are float64 on the device in both variants and are
rounded once to float32 where they scale a float32 vector.
"""

from __future__ import annotations

import ctypes
import math
import time
from collections import OrderedDict
from dataclasses import dataclass, field
from typing import Callable, Optional

import torch
from torch import Tensor

from . import _ext

__all__ = ["dot64", "norm64", "conjugate_gradients", "cg_solve", "CGInfo"]


def _flat(x: Tensor) -> Tensor:
    if not x.is_contiguous():
        raise ValueError("CG vectors must be contiguous")
    if x.dtype not in (torch.complex64, torch.float32):
        raise TypeError(f"CG supports complex64 and float32 vectors, got {x.dtype}")
    return x


_SCRATCH: "OrderedDict[tuple, Tensor]" = OrderedDict()
_SCRATCH_SIZE = 8


def _scratch(dev: torch.device) -> Tensor:
    """The float64 reductions' partial sums (32 KB), one buffer per (device,
    stream): reductions issued on different streams may run at the same time.
    The most recently used few are kept. Each buffer is allocated while its
    stream is current, so the caching allocator hands an evicted buffer's
    memory out again only in that stream's order, after the reductions queued
    there."""
    stream = torch.cuda.current_stream(dev)
    key = (dev, stream.cuda_stream)
    s = _SCRATCH.get(key)
    if s is None:
        s = torch.empty(int(_ext.lib().tlgb_cg_scratch_bytes()), dtype=torch.uint8, device=dev)
        _SCRATCH[key] = s
        while len(_SCRATCH) > _SCRATCH_SIZE:
            _SCRATCH.popitem(last=False)
    else:
        _SCRATCH.move_to_end(key)
    return s


def dot64(x: Tensor, y: Tensor, out: Optional[Tensor] = None) -> Tensor:
    """sum(conj(x) * y) accumulated in float64, as a float64 [re, im] device tensor."""
    dev = _ext.check_cuda(x, y)
    x, y = _flat(x.resolve_conj()), _flat(y.resolve_conj())
    if x.shape != y.shape or x.dtype != y.dtype:
        raise ValueError("dot64 needs two vectors of the same shape and dtype")
    if out is None:
        out = torch.empty(2, dtype=torch.float64, device=dev)
    sc = _scratch(dev)
    with torch.cuda.device(dev):
        _ext.check(
            _ext.lib().tlgb_dot_f64(_ext.ptr(x), _ext.ptr(y), x.numel(), 1 if x.is_complex() else 0, _ext.ptr(out),
                                    _ext.ptr(sc), sc.numel(), _ext.stream_ptr(dev)),
            "dot64",
        )
    return out


def norm64(x: Tensor) -> Tensor:
    """|x|_2 in float64 (device scalar)."""
    return dot64(x, x)[0].clamp_min(0).sqrt()


def _cdot(x: Tensor, y: Tensor) -> Tensor:
    d = dot64(x, y)
    return torch.complex(d[0], d[1])


def conjugate_gradients(
    A: Callable,
    y: Tensor,
    x0: Optional[Tensor] = None,
    max_num_iters: int = 20,
    gtol: float = 1e-3,
    ltol: float = 1e-5,
    disable_tracking: bool = False,
    tqdm_kwargs: Optional[dict] = None,
) -> Tensor:
    """Solve A x = y by CG (reference alg/pcg.py:13), float64 scalars on the GPU."""
    dev = _ext.check_cuda(y)
    x = torch.zeros_like(y) if x0 is None else x0.clone()
    x = x.contiguous()
    r = (y - A(x)).contiguous()
    p = r.clone()
    state = torch.zeros(_ext.CG_STATE_LEN, dtype=torch.float64, device=dev)
    state[_ext.CG_RS] = dot64(r, r)[0]
    sc = _scratch(dev)
    L = _ext.lib()
    n = y.numel()
    cplx = 1 if y.is_complex() else 0
    prev_loss = None
    for _ in range(max_num_iters):
        Ap = A(p).contiguous()
        with torch.cuda.device(dev):
            st = _ext.stream_ptr(dev)
            _ext.check(L.tlgb_cg_set_pap(_ext.ptr(p), _ext.ptr(Ap), n, cplx, _ext.ptr(state), _ext.ptr(sc), sc.numel(), st), "cg")
            _ext.check(L.tlgb_cg_step(_ext.ptr(x), _ext.ptr(r), _ext.ptr(p), _ext.ptr(Ap), n, cplx, _ext.ptr(state),
                                      _ext.ptr(sc), sc.numel(), st), "cg")
        if not disable_tracking:
            # CGRun.update / is_converged (pcg.py:135-176) with float64 scalars
            Ax = A(x)
            xy = _cdot(x, y)
            loss = float((_cdot(x, Ax) - xy - xy.conj()).real)
            gnorm = float(norm64((Ax - y).contiguous()))
            if prev_loss is not None and abs(loss - prev_loss) < ltol and gnorm < gtol:
                break
            prev_loss = loss
    return x


@dataclass
class CGInfo:
    """What one ``cg_solve`` did; ``record()`` gives it as a JSON-ready dict."""

    iters: int = 0
    converged: bool = False
    rel_residual: float = float("nan")  # recursive |r| / |b|
    true_rel_residual: float = float("nan")  # |b - A x| / |b| recomputed in float64
    seconds: float = 0.0
    fallback: bool = False
    restarts: int = 0  # continuations because the true residual was above rtol
    history: list = field(default_factory=list)

    def record(self, history: bool = False) -> dict:
        """The solve as plain numbers and flags (non-finite residuals as None,
        so the record stays valid JSON); the residual history on request."""
        def num(v):
            return float(v) if math.isfinite(v) else None

        out = {"iters": int(self.iters), "converged": bool(self.converged), "seconds": float(self.seconds),
               "rel_residual": num(self.rel_residual), "true_rel_residual": num(self.true_rel_residual),
               "fallback": bool(self.fallback), "restarts": int(self.restarts)}
        if history:
            out["history"] = [num(float(h)) for h in self.history]
        return out


def cg_solve(
    A: Callable,
    b: Tensor,
    x0: Optional[Tensor] = None,
    rtol: float = 1e-4,
    max_iters: int = 200,
    M: Optional[Callable] = None,
    check_every: int = 1,
    restart_on_stagnation: bool = True,
) -> tuple[Tensor, CGInfo]:
    """CG / flexible preconditioned CG to |b - A x| / |b| <= rtol.

    With ``M`` the flexible variant is used (beta = <z_k+1, r_k+1 - r_k> /
    <z_k, r_k>, Polak-Ribiere), valid for a preconditioner that changes from
    step to step (e.g. a neural network). If the preconditioned iteration
    produces NaN/Inf, or its residual falls by less than 10% over 10
    checks, it restarts from its last finite iterate as plain CG.
    """
    dev = _ext.check_cuda(b)
    t0 = time.perf_counter()
    info = CGInfo()
    bnorm = float(norm64(b.contiguous()))
    if bnorm == 0:
        info.converged = True
        info.rel_residual = info.true_rel_residual = 0.0
        return torch.zeros_like(b), info
    x = torch.zeros_like(b) if x0 is None else x0.clone().contiguous()
    r = (b - A(x)).contiguous() if x0 is not None else b.clone().contiguous()
    use_m = M is not None
    if not use_m:
        # fused device-side iteration (no host sync between checks)
        p = r.clone()
        state = torch.zeros(_ext.CG_STATE_LEN, dtype=torch.float64, device=dev)
        state[_ext.CG_RS] = dot64(r, r)[0]
        sc = _scratch(dev)
        L = _ext.lib()
        n = b.numel()
        cplx = 1 if b.is_complex() else 0
        for k in range(1, max_iters + 1):
            Ap = A(p).contiguous()
            with torch.cuda.device(dev):
                st = _ext.stream_ptr(dev)
                _ext.check(L.tlgb_cg_set_pap(_ext.ptr(p), _ext.ptr(Ap), n, cplx, _ext.ptr(state), _ext.ptr(sc), sc.numel(), st), "cg")
                _ext.check(L.tlgb_cg_step(_ext.ptr(x), _ext.ptr(r), _ext.ptr(p), _ext.ptr(Ap), n, cplx, _ext.ptr(state),
                                          _ext.ptr(sc), sc.numel(), st), "cg")
            info.iters = k
            if k % check_every == 0 or k == max_iters:
                rel = math.sqrt(max(float(state[_ext.CG_RS]), 0.0)) / bnorm
                info.history.append(rel)
                info.rel_residual = rel
                if not math.isfinite(rel):
                    break
                if rel <= rtol:
                    info.converged = True
                    break
    else:
        # flexible PCG, fused on the device like plain CG: float64 <r, z>,
        # <p, Ap>, <Ap, z>, alpha and the Polak-Ribiere beta stay in the state
        # vector; no host synchronisation between checks
        z = M(r).contiguous()
        p = z.clone()
        state = torch.zeros(_ext.CG_STATE_LEN, dtype=torch.float64, device=dev)
        state[_ext.CG_RS] = dot64(r, z)[0]
        sc = _scratch(dev)
        L = _ext.lib()
        n = b.numel()
        cplx = 1 if b.is_complex() else 0
        for k in range(1, max_iters + 1):
            Ap = A(p).contiguous()
            with torch.cuda.device(dev):
                st = _ext.stream_ptr(dev)
                _ext.check(L.tlgb_cg_set_pap(_ext.ptr(p), _ext.ptr(Ap), n, cplx, _ext.ptr(state), _ext.ptr(sc),
                                             sc.numel(), st), "pcg")
                _ext.check(L.tlgb_pcg_update(_ext.ptr(x), _ext.ptr(r), _ext.ptr(p), _ext.ptr(Ap), n, cplx,
                                             _ext.ptr(state), st), "pcg")
            z = M(r).contiguous()
            with torch.cuda.device(dev):
                _ext.check(L.tlgb_pcg_direction(_ext.ptr(r), _ext.ptr(z), _ext.ptr(Ap), _ext.ptr(p), n, cplx,
                                                _ext.ptr(state), _ext.ptr(sc), sc.numel(), _ext.stream_ptr(dev)),
                           "pcg")
            info.iters = k
            if k % check_every == 0 or k == max_iters:
                rel = float(norm64(r)) / bnorm
                info.history.append(rel)
                info.rel_residual = rel
                if rel <= rtol:
                    info.converged = True
                    break
                if not math.isfinite(rel):
                    info.fallback = True
                    break
                # stagnation: less than a 10% residual reduction over the
                # last 10 checks (plain CG on a well-posed problem does far
                # better; an indefinite or erratic preconditioner does not)
                h = info.history
                if restart_on_stagnation and len(h) > 10 and h[-1] > 0.9 * h[-11]:
                    info.fallback = True
                    break
        if info.fallback:
            x = torch.where(torch.isfinite(x), x, torch.zeros_like(x)).contiguous()
            x, sub = cg_solve(A, b, x, rtol, max_iters - info.iters, None, check_every)
            _merge(info, sub)
            info.seconds = time.perf_counter() - t0
            return x, info
    # The float64 true residual judges every solve: a recursive residual that
    # drifted below rtol (float32 vectors, or a learned preconditioner's
    # inexact steps) does not count as convergence. Such a solve continues as
    # plain CG from its iterate, within the iteration budget.
    info.true_rel_residual = float(norm64((b - A(x)).contiguous())) / bnorm
    if info.converged and not info.true_rel_residual <= rtol:
        info.converged = False
        remaining = max_iters - info.iters
        if remaining > 0 and math.isfinite(info.true_rel_residual):
            info.restarts += 1
            x, sub = cg_solve(A, b, x, rtol, remaining, None, check_every)
            _merge(info, sub)
    torch.cuda.synchronize(dev)
    info.seconds = time.perf_counter() - t0
    return x, info


def _merge(info: CGInfo, sub: CGInfo) -> None:
    """Fold a continuation solve's record into the solve that started it."""
    info.iters += sub.iters
    info.converged = sub.converged
    info.rel_residual = sub.rel_residual
    info.true_rel_residual = sub.true_rel_residual
    info.restarts += sub.restarts
    info.history += sub.history
