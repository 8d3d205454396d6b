"""Time the reference's own CPU path beside the oracle port (CHECKER TOOLING).

The GPU machine cannot import the reference (a Python package that does not
travel there), so the timed CPU baseline of ``bench.py`` is the oracle, the
restatement of the reference's torch path under ``oracle/``. This script,
run where the reference is importable, times both on the same inputs and
threads, so the port's figures can be read as the reference's:

    TORCHLINOPS_SRC=<torch-named-linops checkout>/src python oracle/time_reference.py

Workloads (each the bench's, or a stated sample of it):
* 2D interpolate, 64^2 complex64, 4096 points, W 4, beta for oversampling
  1.25 (forward and adjoint, median of 10 after 3 warm-ups);
* 3D gridding and ungridding, 256^3 x 8 coils complex64, the first 65,536 of
  the 2^21 points of the 1/r^2 ball (median of 3);
* unfold / fold, one 160^3 complex64 batch entry of the 16, block 8^3,
  stride 4 (median of 3; fold once);
* the functional 2D NUFFT forward and adjoint, one 256^2 slice x 8 coils of
  the 32, 402 x 512 golden-angle radial points (median of 3).
Prints one markdown table.
"""

from __future__ import annotations

import math
import os
import statistics
import sys
import time

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def med(fn, reps, warm=1):
    for _ in range(warm):
        fn()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts) * 1e3


def main():
    src = os.environ.get("TORCHLINOPS_SRC")
    if not src:
        sys.exit("set TORCHLINOPS_SRC to the reference's src/ directory")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden", "_stubs"))
    sys.path.insert(0, src)
    sys.path.insert(0, ROOT)
    import torchlinops.functional as F

    from oracle import blocks as OB
    from oracle import interp as OI
    from oracle import nufft as ONU

    threads = len(os.sched_getaffinity(0))
    torch.set_num_threads(threads)
    beta = OI.nufft_beta(4.0, 1.25)
    kp = dict(beta=beta)
    g = torch.Generator().manual_seed(0)
    rows = []

    img = torch.complex(torch.randn(64, 64, generator=g), torch.randn(64, 64, generator=g))
    locs = torch.rand(4096, 2, generator=g) * 64
    pts = torch.complex(torch.randn(4096, generator=g), torch.randn(4096, generator=g))
    rows.append(("interp 2D 64^2, 4096 pts, forward",
                 med(lambda: F.interpolate(img, locs, 4.0, kernel_params=kp), 10, 3),
                 med(lambda: OI.ungrid(img, locs, 4.0, beta=beta), 10, 3)))
    rows.append(("interp 2D 64^2, 4096 pts, adjoint",
                 med(lambda: F.interpolate_adjoint(pts, locs, (64, 64), 4.0, kernel_params=kp), 10, 3),
                 med(lambda: OI.grid(pts, locs, (64, 64), 4.0, beta=beta), 10, 3)))

    n, P = 256, 1 << 16
    gb = torch.Generator().manual_seed(0)
    r = torch.rand(1 << 21, generator=gb) * (n / 2)
    u = torch.randn(1 << 21, 3, generator=gb)
    l3 = (n / 2 + r[:, None] * u / u.norm(dim=-1, keepdim=True)).to(torch.float32)[:P].contiguous()
    im3 = torch.randn(8, n, n, n, dtype=torch.complex64, generator=g)
    v3 = torch.randn(8, P, dtype=torch.complex64, generator=g)
    rows.append(("ungrid 256^3 x 8, 65,536 of 2^21 pts",
                 med(lambda: F.interpolate(im3, l3, 4.0, kernel_params=kp), 3),
                 med(lambda: OI.ungrid(im3, l3, 4.0, beta=beta), 3)))
    rows.append(("grid 256^3 x 8, 65,536 of 2^21 pts",
                 med(lambda: F.interpolate_adjoint(v3, l3, (n, n, n), 4.0, kernel_params=kp), 3),
                 med(lambda: OI.grid(v3, l3, (n, n, n), 4.0, beta=beta), 3)))
    del im3

    x = torch.complex(torch.randn(1, 160, 160, 160, generator=g), torch.randn(1, 160, 160, 160, generator=g))
    b, st = (8, 8, 8), (4, 4, 4)
    rows.append(("unfold 1 x 160^3, block 8^3, stride 4",
                 med(lambda: F.array_to_blocks(x, b, st), 3), med(lambda: OB.unfold(x, b, st), 3)))
    y = OB.unfold(x, b, st)
    rows.append(("fold 1 x 160^3, block 8^3, stride 4",
                 med(lambda: F.blocks_to_array(y, (160, 160, 160), b, st), 1, 0),
                 med(lambda: OB.fold(y, (160, 160, 160), b, st), 1, 0)))
    del x, y

    SP, RD, N = 402, 512, 256
    ang = torch.arange(SP, dtype=torch.float64) * math.pi * (math.sqrt(5.0) - 1.0) / 2.0
    rr = (torch.arange(RD, dtype=torch.float64) - RD // 2) * (N / RD)
    l2 = torch.stack([rr[None, :] * torch.cos(ang[:, None]), rr[None, :] * torch.sin(ang[:, None])], dim=-1)
    l2 = (l2 + 0.1 * torch.randn(l2.shape, generator=g, dtype=torch.float64)).to(torch.float32)
    xi = torch.complex(torch.randn(8, N, N, generator=g), torch.randn(8, N, N, generator=g))
    ys = torch.complex(torch.randn(8, SP, RD, generator=g), torch.randn(8, SP, RD, generator=g))
    rows.append(("NUFFT 2D forward, 8 x 256^2, 402 x 512 pts",
                 med(lambda: F.nufft(xi, l2, 1.25, 4.0), 3), med(lambda: ONU.nufft(xi, l2, dtype=torch.float32), 3)))
    rows.append(("NUFFT 2D adjoint, 8 x 256^2, 402 x 512 pts",
                 med(lambda: F.nufft_adjoint(ys, l2, (N, N), 1.25, 4.0), 3),
                 med(lambda: ONU.nufft_adjoint(ys, l2, (N, N), dtype=torch.float32), 3)))

    print(f"Host: {threads} threads, torch {torch.__version__}\n")
    print("| Workload | reference CPU path (ms) | oracle port (ms) | port / reference |")
    print("|---|---|---|---|")
    for name, ref, port in rows:
        print(f"| {name} | {ref:.2f} | {port:.2f} | {port / ref:.2f} |")


if __name__ == "__main__":
    main()
