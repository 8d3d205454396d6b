"""Learned preconditioner for CG on the multicoil NUFFT normal equations.

A 4-layer 3^3 CNN with 16 channels maps a residual ``r`` to a search
direction ``z ~ (A^H A + lam I)^{-1} r``:

    z = |r| N^T N (r / |r|) + c0 r

``N`` is two conv layers (1 -> 8 -> 8 features per real component) and
``N^T`` the same two layers transposed (flipped taps, swapped channels), so the
four layers compose to a symmetric positive semi-definite operator and, with
``c0 > 0``, ``M`` is symmetric positive definite: the condition standard PCG
needs. The real and imaginary parts share the weights (channels 0-7 and 8-15
of every hidden layer hold the same features of the two parts), so ``M`` is
complex-linear. It is also positively homogeneous, so normalising by ``|r|``
costs nothing. The warm start is ``N = grad`` (forward differences), which
makes ``N^T N = -lap`` and ``M`` the classical ``c0 I - lap``, a good start
for radial sampling, whose density falls as 1/|k|^2; training on this
operator's own spectrum then improves on it.

Every convolution, forward and backward, runs on this package's tensor-core
kernels (``tlgb_conv3d_*``: BF16 operands, FP32 accumulation). The optimiser
(Adam on FP32 master weights) and the loss are plain torch arithmetic on the
GPU. The preconditioner has no counterpart in the reference (torchlinops
has no learned preconditioner).
"""

from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass, field
from typing import Callable, Optional

import torch
from torch import Tensor

from . import _ext

__all__ = [
    "conv3d",
    "conv3d_wgrad",
    "flip_weights",
    "pack",
    "unpack",
    "expand_weights",
    "collapse_grads",
    "laplacian_params",
    "CNNPreconditioner",
    "TrainLog",
    "save_train_checkpoint",
    "load_train_checkpoint",
]

C = 16  # channels of every activation (narrower layers are zero-padded)
TAPS = 27


def _desc(shape, mode: int, out_f32: bool) -> _ext.ConvDesc:
    D, H, W = (int(s) for s in shape)
    return _ext.ConvDesc(D=D, H=H, W=W, cin=C, cout=C, mode=mode, out_f32=1 if out_f32 else 0, reserved=0)


def _check_act(x: Tensor, name: str) -> None:
    if x.dtype != torch.bfloat16 or x.dim() != 4 or x.shape[-1] != C or not x.is_contiguous():
        raise ValueError(f"{name}: expected a contiguous [D, H, W, {C}] bfloat16 tensor, got {x.dtype} {tuple(x.shape)}")


def conv3d(x: Tensor, w: Tensor, mode: int = _ext.TLGB_CONV_PLAIN, aux: Optional[Tensor] = None,
           out_f32: bool = False) -> Tensor:
    """y[v, co] = sum_{t, ci} w[t, co, ci] x[v + off(t), ci] (zero padding 1)."""
    _ext.check_cuda(x, w, aux)
    _check_act(x, "conv3d input")
    if w.dtype != torch.bfloat16 or tuple(w.shape) != (TAPS, C, C) or not w.is_contiguous():
        raise ValueError(f"conv3d weights: expected contiguous [27, 16, 16] bfloat16, got {w.dtype} {tuple(w.shape)}")
    if mode == _ext.TLGB_CONV_MASK:
        if aux is None:
            raise ValueError("conv3d: the mask epilogue needs aux")
        _check_act(aux, "conv3d aux")
    y = torch.empty(x.shape, dtype=torch.float32 if out_f32 else torch.bfloat16, device=x.device)
    d = _desc(x.shape[:3], mode, out_f32)
    _ext.check(
        _ext.lib().tlgb_conv3d_fwd(ctypes.byref(d), _ext.ptr(x), _ext.ptr(w), _ext.ptr(aux), _ext.ptr(y),
                                   _ext.stream_ptr(x.device)),
        "conv3d",
    )
    return y


def conv3d_wgrad(x: Tensor, gy: Tensor) -> Tensor:
    """dw[t, co, ci] = sum_v gy[v, co] x[v + off(t), ci] in float32 (fixed summation order)."""
    _ext.check_cuda(x, gy)
    _check_act(x, "conv3d_wgrad input")
    _check_act(gy, "conv3d_wgrad grad")
    if x.shape != gy.shape:
        raise ValueError(f"conv3d_wgrad: input {tuple(x.shape)} and grad {tuple(gy.shape)} differ")
    d = _desc(x.shape[:3], _ext.TLGB_CONV_PLAIN, False)
    L = _ext.lib()
    sb = ctypes.c_size_t(0)
    _ext.check(L.tlgb_conv3d_wgrad_scratch_size(ctypes.byref(d), ctypes.byref(sb)), "conv3d_wgrad")
    scratch = torch.empty(max(sb.value, 16), dtype=torch.uint8, device=x.device)
    dw = torch.empty(TAPS, C, C, dtype=torch.float32, device=x.device)
    _ext.check(
        L.tlgb_conv3d_wgrad(ctypes.byref(d), _ext.ptr(x), _ext.ptr(gy), _ext.ptr(dw), _ext.ptr(scratch), sb.value,
                            _ext.stream_ptr(x.device)),
        "conv3d_wgrad",
    )
    return dw


def flip_weights(w: Tensor) -> Tensor:
    """Weights of the data gradient: w'[26 - t, ci, co] = w[t, co, ci]."""
    return w.flip(0).transpose(1, 2).contiguous()


def pack(z: Tensor, scale: Optional[Tensor] = None, hilo: bool = False) -> Tensor:
    """complex64 [D, H, W] (times the device scalar ``scale``) -> [D, H, W, 16]
    bfloat16; with ``hilo`` channels 2, 3 carry the bf16 rounding remainders."""
    _ext.check_cuda(z, scale)
    if z.dtype != torch.complex64 or z.dim() != 3:
        raise ValueError(f"pack: expected a [D, H, W] complex64 tensor, got {z.dtype} {tuple(z.shape)}")
    z = z.resolve_conj().resolve_neg().contiguous()
    out = torch.empty(*z.shape, C, dtype=torch.bfloat16, device=z.device)
    sc = None if scale is None else scale.to(torch.float32).contiguous()
    _ext.check(_ext.lib().tlgb_conv3d_pack(_ext.ptr(z), z.numel(), _ext.ptr(sc), 1 if hilo else 0, _ext.ptr(out),
                                           _ext.stream_ptr(z.device)), "pack")
    return out


def unpack(y: Tensor, z: Optional[Tensor] = None, scale: Optional[Tensor] = None, skip: float = 0.0) -> Tensor:
    """scale * (y[..., 0] + i y[..., 1]) + skip * z as complex64 [D, H, W]."""
    _ext.check_cuda(y, z, scale)
    if y.dtype != torch.float32 or y.dim() != 4 or y.shape[-1] != C:
        raise ValueError(f"unpack: expected a [D, H, W, 16] float32 tensor, got {y.dtype} {tuple(y.shape)}")
    if z is not None:
        z = z.resolve_conj().resolve_neg().contiguous()
    out = torch.empty(y.shape[:3], dtype=torch.complex64, device=y.device)
    sc = None if scale is None else scale.to(torch.float32).contiguous()
    _ext.check(_ext.lib().tlgb_conv3d_unpack(_ext.ptr(y), _ext.ptr(z), y.shape[0] * y.shape[1] * y.shape[2],
                                             _ext.ptr(sc), ctypes.c_float(skip), _ext.ptr(out),
                                             _ext.stream_ptr(y.device)), "unpack")
    return out


@dataclass
class TrainLog:
    losses: list = field(default_factory=list)
    seconds: float = 0.0
    resumed_from: int = 0  # the step a resumed training continued from (0: a fresh start)


CHECKPOINT_VERSION = 1


def save_train_checkpoint(path: str, model: "CNNPreconditioner", opt, sched, step: int, losses: list,
                          manifest: Optional[dict]) -> None:
    """Write a training checkpoint: the weights, the optimiser and schedule
    state, the next step, the loss log and the manifest of the training data
    (whatever identifies it: phantom seeds, solver tolerance, batch size,
    learning rate). The file is replaced atomically, so an interrupted save
    leaves the previous checkpoint intact."""
    ck = {"version": CHECKPOINT_VERSION, "step": int(step), "model": model.state_dict(),
          "optim": opt.state_dict(), "sched": sched.state_dict() if sched is not None else None,
          "losses": list(losses), "manifest": manifest}
    tmp = f"{path}.tmp"
    torch.save(ck, tmp)
    os.replace(tmp, path)


def load_train_checkpoint(path: str, model: "CNNPreconditioner", opt, sched, manifest: Optional[dict]) -> tuple:
    """Restore a checkpoint written by ``save_train_checkpoint`` into the
    model, optimiser and schedule; returns (next step, loss log). A checkpoint
    of another training run (its manifest differs from ``manifest``) raises
    ValueError instead of mixing two runs' data."""
    ck = torch.load(path, map_location="cpu", weights_only=False)
    if ck.get("version") != CHECKPOINT_VERSION:
        raise ValueError(f"{path}: checkpoint version {ck.get('version')!r}, expected {CHECKPOINT_VERSION}")
    if manifest is not None and ck.get("manifest") != manifest:
        raise ValueError(f"{path}: checkpoint of another training run (manifest {ck.get('manifest')!r}, "
                         f"this run {manifest!r})")
    model.load_state_dict(ck["model"])
    opt.load_state_dict(ck["optim"])
    if sched is not None and ck.get("sched") is not None:
        sched.load_state_dict(ck["sched"])
    return int(ck["step"]), list(ck["losses"])


FEAT = 8  # features per real component (channels 0-7: real part, 8-15: imaginary part)


def expand_weights(v1: Tensor, v2: Tensor):
    """The four [27, 16, 16] layer weights from the free parameters
    v1 [27, 8] (scalar field -> 8 features) and v2 [27, 8, 8].

    Input channels of layer 1: 0 / 1 = real / imaginary (bf16), 2 / 3 = their
    rounding remainders (same weights). Layers 3 and 4 are the transposes of
    2 and 1; layer 4's output channels 0 / 1 are the real / imaginary result.
    """
    w1 = v1.new_zeros(TAPS, C, C)
    for comp in (0, 1):
        rows = slice(comp * FEAT, (comp + 1) * FEAT)
        w1[:, rows, comp] = v1
        w1[:, rows, comp + 2] = v1
    w2 = v1.new_zeros(TAPS, C, C)
    w2[:, :FEAT, :FEAT] = v2
    w2[:, FEAT:, FEAT:] = v2
    return [w1, w2, flip_weights(w2), flip_weights(w1)]


def collapse_grads(g1: Tensor, g2: Tensor, g3: Tensor, g4: Tensor):
    """Gradients of v1, v2 from those of the four expanded layer weights."""
    d1 = g1 + flip_weights(g4)
    d2 = g2 + flip_weights(g3)
    dv1 = d1[:, :FEAT, 0] + d1[:, :FEAT, 2] + d1[:, FEAT:, 1] + d1[:, FEAT:, 3]
    dv2 = d2[:, :FEAT, :FEAT] + d2[:, FEAT:, FEAT:]
    return dv1, dv2


def laplacian_params(noise: float = 0.0, gen: Optional[torch.Generator] = None):
    """v1, v2 with N = (forward differences along d, h, w): N^T N = -lap."""
    ctr, plus = 13, (22, 16, 14)  # centre tap; taps reading (+1, 0, 0), (0, +1, 0), (0, 0, +1)
    v1 = torch.zeros(TAPS, FEAT)
    v2 = torch.zeros(TAPS, FEAT, FEAT)
    for j, t in enumerate(plus):
        v1[ctr, j] = -1.0
        v1[t, j] = 1.0
        v2[ctr, j, j] = 1.0
    if noise > 0:
        gen = gen if gen is not None else torch.Generator().manual_seed(0)
        # small weights on the unused features only: the start stays exact
        v1[:, 3:] += noise * torch.randn(TAPS, FEAT - 3, generator=gen) / math.sqrt(TAPS)
        v2[:, 3:, :] += noise * torch.randn(TAPS, FEAT - 3, FEAT, generator=gen) / math.sqrt(TAPS * FEAT)
    return v1, v2


class CNNPreconditioner:
    """z = |r| N^T N (r/|r|) + c0 r on the BF16 tensor-core convolutions (see the module doc)."""

    def __init__(self, device="cuda", seed: int = 0, c0: float = 0.02, noise: float = 0.05, init: str = "laplacian"):
        if init not in ("laplacian", "random"):
            raise ValueError(f"init must be 'laplacian' or 'random', got {init!r}")
        gen = torch.Generator().manual_seed(seed)
        if init == "laplacian":
            v1, v2 = laplacian_params(noise, gen)
        else:
            v1 = torch.randn(TAPS, FEAT, generator=gen) / math.sqrt(TAPS)
            v2 = torch.randn(TAPS, FEAT, FEAT, generator=gen) / math.sqrt(TAPS * FEAT)
        self.v1 = v1.to(device).requires_grad_(True)
        self.v2 = v2.to(device).requires_grad_(True)
        self.skip = torch.tensor([c0], device=device, requires_grad=True)
        self._cache = None  # (bf16 layer weights, host skip) for the current parameters

    # -- parameters ------------------------------------------------------------
    def parameters(self):
        return [self.v1, self.v2, self.skip]

    def layer_weights(self):
        """The four bfloat16 layer weights and the skip weight (host float)."""
        if self._cache is None:
            ws = expand_weights(self.v1.detach().to(torch.bfloat16).float(), self.v2.detach().to(torch.bfloat16).float())
            self._cache = ([w.to(torch.bfloat16).contiguous() for w in ws], float(self.skip.detach()))
        return self._cache

    def state_dict(self) -> dict:
        return {"v1": self.v1.detach().cpu().clone(), "v2": self.v2.detach().cpu().clone(),
                "skip": self.skip.detach().cpu().clone()}

    def load_state_dict(self, sd: dict) -> None:
        with torch.no_grad():
            self.v1.copy_(sd["v1"].to(self.v1.device))
            self.v2.copy_(sd["v2"].to(self.v2.device))
            self.skip.copy_(sd["skip"].to(self.skip.device).reshape(1))
        self._cache = None

    # -- inference -------------------------------------------------------------
    def _forward(self, r: Tensor, keep: bool):
        if r.dtype != torch.complex64 or r.dim() != 3:
            raise ValueError(f"the preconditioner takes a [D, H, W] complex64 residual, got {r.dtype} {tuple(r.shape)}")
        wb, c0 = self.layer_weights()
        nrm = torch.linalg.vector_norm(r).to(torch.float32).reshape(1)
        inv = torch.where(nrm > 0, 1.0 / nrm, torch.zeros_like(nrm))
        x0 = pack(r, inv, hilo=True)
        a1 = conv3d(x0, wb[0])
        a2 = conv3d(a1, wb[1])
        a3 = conv3d(a2, wb[2])
        y = conv3d(a3, wb[3], out_f32=True)
        z = unpack(y, r, nrm, c0)
        return z, ((wb, nrm, x0, a1, a2, a3) if keep else None)

    @torch.no_grad()
    def __call__(self, r: Tensor) -> Tensor:
        shape = r.shape
        z, _ = self._forward(r.reshape(shape[-3:]) if r.dim() > 3 else r, keep=False)
        return z.reshape(shape)

    # -- training --------------------------------------------------------------
    def _backward(self, cache, gz: Tensor):
        """Gradients of v1, v2 given dL/dz (complex64), through this package's kernels."""
        wb, nrm, x0, a1, a2, a3 = cache
        g4 = pack(gz, nrm)  # dL/dy = |r| dL/dz on channels 0, 1
        dw4 = conv3d_wgrad(a3, g4)
        g3 = conv3d(g4, flip_weights(wb[3]))
        dw3 = conv3d_wgrad(a2, g3)
        g2 = conv3d(g3, flip_weights(wb[2]))
        dw2 = conv3d_wgrad(a1, g2)
        g1 = conv3d(g2, flip_weights(wb[1]))
        dw1 = conv3d_wgrad(x0, g1)
        return collapse_grads(dw1, dw2, dw3, dw4)

    def loss_and_grads(self, pairs, kind: str = "scale_invariant"):
        """Loss over a batch of (r, e) pairs with r = (A^H A + lam) e, and the
        gradients of (v1, v2, skip).

        * "scale_invariant": L = sum_i |s z_i - e_i|^2 / |e_i|^2 / B with the
          one scale s that fits the whole batch best. CG is blind to the
          scale of M but not to how it differs between spectral components,
          which the batch exposes when its samples cover different bands.
        * "mse": the same with s = 1.
        """
        if isinstance(pairs, tuple) and len(pairs) == 2 and isinstance(pairs[0], Tensor):
            pairs = [pairs]
        with torch.no_grad():
            outs = [self._forward(r, keep=True) for r, _ in pairs]
            ens = [torch.linalg.vector_norm(e) ** 2 for _, e in pairs]
            if kind == "mse":
                s = torch.ones((), device=pairs[0][0].device)
            elif kind == "scale_invariant":
                num = sum(torch.real(torch.vdot(z.flatten(), e.flatten())) / en for (z, _), (_, e), en in zip(outs, pairs, ens))
                den = sum(torch.linalg.vector_norm(z) ** 2 / en for (z, _), en in zip(outs, ens))
                s = num / den
            else:
                raise ValueError(f"unknown loss {kind!r}")
            B = len(pairs)
            loss = 0.0
            dv1 = torch.zeros_like(self.v1)
            dv2 = torch.zeros_like(self.v2)
            gskip = torch.zeros_like(self.skip)
            for (z, cache), (r, e), en in zip(outs, pairs, ens):
                diff = s * z - e
                loss = loss + torch.linalg.vector_norm(diff) ** 2 / (en * B)
                gz = (2.0 * s / (en * B)) * diff  # s is optimal: no term through s
                g1, g2 = self._backward(cache, gz)
                dv1 += g1
                dv2 += g2
                gskip += torch.real(torch.vdot(r.flatten(), gz.flatten()))
        return loss, [dv1, dv2, gskip]

    def fit(self, sample: Callable[[int], object], steps: int, lr: float = 1e-3, log_every: int = 0,
            loss: str = "scale_invariant", checkpoint: Optional[str] = None, checkpoint_every: int = 0,
            manifest: Optional[dict] = None) -> TrainLog:
        """Adam over ``steps`` batches ``sample(step)`` (lists of (r, e) pairs).

        With ``checkpoint`` (a file path), the training state is saved there
        every ``checkpoint_every`` steps and after the last one, and a
        training that finds the file resumes after its last saved step. So
        ``sample`` must give the same batch for the same step (seeded by the
        step), and ``manifest`` names the training data: a checkpoint with
        another manifest is refused rather than resumed."""
        import time

        params = self.parameters()
        opt = torch.optim.Adam(params, lr=lr)
        sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, T_max=max(steps, 1), eta_min=lr * 0.05)
        log = TrainLog()
        start = 0
        if checkpoint and os.path.exists(checkpoint):
            start, log.losses = load_train_checkpoint(checkpoint, self, opt, sched, manifest)
            log.resumed_from = start
        t0 = time.perf_counter()
        for step in range(start, steps):
            lval, grads = self.loss_and_grads(sample(step), loss)
            for p, g in zip(params, grads):
                p.grad = g
            opt.step()
            sched.step()
            with torch.no_grad():
                self.skip.clamp_(min=1e-6)  # keep M positive definite
            self._cache = None
            if log_every and (step % log_every == 0 or step == steps - 1):
                log.losses.append((step, float(lval)))
            if checkpoint and ((checkpoint_every and (step + 1) % checkpoint_every == 0) or step == steps - 1):
                save_train_checkpoint(checkpoint, self, opt, sched, step + 1, log.losses, manifest)
        torch.cuda.synchronize()
        log.seconds = time.perf_counter() - t0
        return log
