"""Learned preconditioner in flexible CG on a SENSE normal operator: what the
trained network gains over plain CG and over its own warm start, and that
plain CG stays the fallback. Small problem (32^3, 4 coils, 3D radial)."""

import pytest
import torch

from torchlinops_gb300 import alg, mri, precond

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def problem():
    n = 32
    locs = mri.radial_trajectory_3d(400, 64, n, DEV)
    maps = mri.gaussian_coil_maps_3d(4, n, device=DEV)
    A = mri.SenseNormal(locs, maps, lam=1e-3)
    xt = mri.ellipsoid_phantom_3d(n, 10, torch.Generator().manual_seed(1234), DEV)
    return n, A, A(xt)


def test_trained_preconditioner_beats_plain_cg(problem):
    n, A, b = problem
    _, plain = alg.cg_solve(A, b, rtol=1e-4, max_iters=400)
    M = precond.CNNPreconditioner(DEV, seed=1, init="laplacian", c0=0.02)
    _, warm = alg.cg_solve(A, b, rtol=1e-4, max_iters=400, M=M)
    gen = torch.Generator().manual_seed(0)
    log = M.fit(lambda step: mri.training_batch(A, n, gen, 4, DEV), 150, lr=1e-3, log_every=50)
    assert log.losses[-1][1] < log.losses[0][1]
    _, learned = alg.cg_solve(A, b, rtol=1e-4, max_iters=400, M=M)
    for info in (plain, warm, learned):
        assert info.converged and info.true_rel_residual < 2e-4
    assert not learned.fallback
    assert learned.iters <= warm.iters
    assert learned.iters * 2 <= plain.iters, (plain.iters, warm.iters, learned.iters)


def test_trained_weights_round_trip(problem):
    n, A, b = problem
    M = precond.CNNPreconditioner(DEV, seed=5, init="random", c0=0.1)
    M2 = precond.CNNPreconditioner(DEV, seed=6, init="laplacian")
    M2.load_state_dict(M.state_dict())
    r = b / torch.linalg.vector_norm(b)
    assert torch.equal(M(r), M2(r))


@pytest.mark.parametrize("bad", ["nan", "indefinite"])
def test_plain_cg_is_the_fallback(problem, bad):
    """A preconditioner that returns non-finite values, or one that is
    indefinite (a fixed random +-1 per voxel), breaks or stalls flexible CG;
    the solve restarts as plain CG from its last finite iterate and still
    converges, judged by its float64 true residual."""
    _, A, b = problem
    if bad == "nan":
        M = lambda r: r * float("nan")  # noqa: E731
    else:
        sign = torch.where(torch.rand(b.shape, generator=torch.Generator().manual_seed(3)) < 0.5, -1.0, 1.0).to(DEV)
        M = lambda r: r * sign  # noqa: E731
    _, info = alg.cg_solve(A, b, rtol=1e-4, max_iters=600, M=M)
    assert info.fallback and info.converged and info.true_rel_residual < 2e-4


def test_training_resumes_from_its_checkpoint(problem, tmp_path):
    """A training interrupted after a checkpoint and started again with the
    same data ends where the uninterrupted training ends."""
    n, A, b = problem

    def sample(step):  # the same batch for the same step
        return mri.training_batch(A, n, torch.Generator().manual_seed(100 + step), 2, DEV)

    manifest = {"sample": "mri.training_batch, seed 100 + step, 2 pairs", "n": n, "lr": 1e-3}
    full = precond.CNNPreconditioner(DEV, seed=2)
    full.fit(sample, 6, lr=1e-3)

    def interrupted(step):
        if step == 4:
            raise RuntimeError("interrupted")
        return sample(step)

    path = str(tmp_path / "precond.ckpt")
    first = precond.CNNPreconditioner(DEV, seed=2)
    with pytest.raises(RuntimeError, match="interrupted"):
        first.fit(interrupted, 6, lr=1e-3, checkpoint=path, checkpoint_every=3, manifest=manifest)
    again = precond.CNNPreconditioner(DEV, seed=7)  # other initial weights: the checkpoint replaces them
    log = again.fit(sample, 6, lr=1e-3, checkpoint=path, checkpoint_every=3, manifest=manifest)
    assert log.resumed_from == 3
    for p, q in zip(full.parameters(), again.parameters()):
        assert torch.allclose(p.detach(), q.detach(), rtol=1e-6, atol=1e-7)
    with pytest.raises(ValueError, match="another training run"):
        precond.CNNPreconditioner(DEV).fit(sample, 6, checkpoint=path, manifest={"other": 1})
