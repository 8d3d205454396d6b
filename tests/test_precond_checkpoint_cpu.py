"""Checkpoints of the preconditioner training (CPU: the state round trip and
the refusals; the resumed training itself runs in tests/test_precond_gpu.py)."""

import os

import pytest
import torch

from torchlinops_gb300 import mri
from torchlinops_gb300 import precond as P


def _setup(seed):
    m = P.CNNPreconditioner(device="cpu", seed=seed)
    opt = torch.optim.Adam(m.parameters(), lr=1e-3)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, T_max=10, eta_min=1e-5)
    return m, opt, sched


def _step(m, opt, sched, k):
    for i, p in enumerate(m.parameters()):  # a deterministic stand-in for the conv gradients
        p.grad = torch.full_like(p, 0.01 * (k + 1) * (i + 1))
    opt.step()
    sched.step()


def test_checkpoint_round_trip(tmp_path):
    path = str(tmp_path / "train.ckpt")
    manifest = {"source": "seeded phantoms", "seeds": [0, 1, 2], "rtol": 1e-6}
    a, oa, sa = _setup(0)
    for k in range(3):
        _step(a, oa, sa, k)
    P.save_train_checkpoint(path, a, oa, sa, 3, [(0, 1.0), (2, 0.5)], manifest)
    assert os.path.exists(path) and not os.path.exists(path + ".tmp")
    b, ob, sb = _setup(1)  # other initial weights: the checkpoint overwrites them
    step, losses = P.load_train_checkpoint(path, b, ob, sb, manifest)
    assert step == 3 and losses == [(0, 1.0), (2, 0.5)]
    for pa, pb in zip(a.parameters(), b.parameters()):
        assert torch.equal(pa.detach(), pb.detach())
    # the optimiser and schedule continue identically
    for k in range(3, 6):
        _step(a, oa, sa, k)
        _step(b, ob, sb, k)
    for pa, pb in zip(a.parameters(), b.parameters()):
        assert torch.equal(pa.detach(), pb.detach())
    assert sa.last_epoch == sb.last_epoch == 6


def test_checkpoint_of_another_run_is_refused(tmp_path):
    path = str(tmp_path / "train.ckpt")
    a, oa, sa = _setup(0)
    P.save_train_checkpoint(path, a, oa, sa, 1, [], {"seeds": [0, 1]})
    b, ob, sb = _setup(0)
    with pytest.raises(ValueError, match="another training run"):
        P.load_train_checkpoint(path, b, ob, sb, {"seeds": [0, 2]})
    ck = torch.load(path, weights_only=False)
    ck["version"] = 99
    torch.save(ck, path)
    with pytest.raises(ValueError, match="version"):
        P.load_train_checkpoint(path, b, ob, sb, {"seeds": [0, 1]})


def test_manifest_of_cg_training_data_pins_the_solutions(tmp_path):
    """The manifest of (r, e) pairs from plain-CG solutions carries the
    phantom seeds and a hash of every solution: the same data give the same
    manifest, and a checkpoint refuses data whose solutions differ."""
    gen = torch.Generator().manual_seed(4)
    pairs = [(torch.randn(6, 6, 6, dtype=torch.complex64, generator=gen),
              torch.randn(6, 6, 6, dtype=torch.complex64, generator=gen)) for _ in range(3)]
    m = mri.training_manifest(pairs, seed=10, rtol=1e-6)
    assert m == mri.training_manifest([(r.clone(), e.clone()) for r, e in pairs], seed=10, rtol=1e-6)
    assert m["phantom_seeds"] == [10, 11, 12] and len(set(m["solution_sha256"])) == 3
    changed = list(pairs)
    e = pairs[1][1].clone()
    e[0, 0, 0] += 1e-6
    changed[1] = (pairs[1][0], e)
    other = mri.training_manifest(changed, seed=10, rtol=1e-6)
    assert other["solution_sha256"][1] != m["solution_sha256"][1] and other["solution_sha256"][0] == m["solution_sha256"][0]
    path = str(tmp_path / "train.ckpt")
    a, oa, sa = _setup(0)
    P.save_train_checkpoint(path, a, oa, sa, 2, [], m)
    b, ob, sb = _setup(0)
    assert P.load_train_checkpoint(path, b, ob, sb, m)[0] == 2
    with pytest.raises(ValueError, match="another training run"):
        P.load_train_checkpoint(path, b, ob, sb, other)
