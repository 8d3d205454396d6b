"""Benchmark: 3D multicoil gridding + ungridding on one GB300 (and replicas).

Workload (the configuration the headline metric is quoted on): oversampled
grid 256^3 complex64 x 8 coils; 2^21 points float32 in a ball of radius 128
centred on the grid with radial density ~ 1/r^2 (r ~ U(0,128), direction a
normalised N(0, I3)); Kaiser-Bessel width 4, beta for oversampling 1.25.
One step = one ungrid (forward interpolation) + one grid (adjoint) of all
coils: the interpolation half of one NUFFT normal operator.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Prints one JSON line. ``value`` = point-coil samples interpolated per second
(both directions counted) with inputs resident in HBM; ``e2e`` = the same
through the public API from pinned host buffers, copies included.
``roofline`` is for the dominant kernel (gridding) against the measured HBM
copy bandwidth; ``cpu_baseline`` times the CPU restatement of the reference's
torch path (oracle) on a bounded sample on the host cores.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "torch-named-linops_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import torch  # noqa: E402

N_GRID = 256
N_COIL = 8
N_PTS = 1 << 21
WIDTH = 4.0
OVERSAMP = 1.25
# algorithmic bytes of one launch (either direction): grid + locs + point values
ALGO_BYTES = N_COIL * N_GRID**3 * 8 + N_PTS * 3 * 4 + N_COIL * N_PTS * 8
# unfold / fold workload: 16 x 160^3 complex64, block 8^3, stride 4
BLK_SHAPE = (16, 160, 160, 160)
BLK = (8, 8, 8)
BLK_STRIDE = (4, 4, 4)


def kb_beta(width=WIDTH, os_=OVERSAMP):
    return math.pi * (((width / os_) * (os_ - 0.5)) ** 2 - 0.8) ** 0.5


def make_locs(n=None, seed=0):
    n = N_PTS if n is None else n
    g = torch.Generator().manual_seed(seed)
    r = torch.rand(n, generator=g) * (N_GRID / 2)
    u = torch.randn(n, 3, generator=g)
    u = u / u.norm(dim=-1, keepdim=True)
    return (N_GRID / 2 + r[:, None] * u).to(torch.float32)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per gridding launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f).get("grid_dram_bytes_per_launch")
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL,
            )
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
            os.unlink(self.path)
        except Exception:
            pass
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------- CPU baseline


class CpuSample:
    """Oracle (CPU restatement of the reference torch path) on a sample of the
    workload: all 8 coils, the full 256^3 grid, the first `sample_pts` points."""

    def __init__(self, sample_pts: int):
        from oracle import interp as OI

        self.OI = OI
        self.threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
        torch.set_num_threads(self.threads)
        self.n = sample_pts
        self.locs = make_locs()[:sample_pts].contiguous()
        g = torch.Generator().manual_seed(1)
        self.img = torch.randn(N_COIL, N_GRID, N_GRID, N_GRID, dtype=torch.complex64, generator=g)
        self.vals = torch.randn(N_COIL, sample_pts, dtype=torch.complex64, generator=g)
        self.beta = kb_beta()

    def run(self) -> float:
        t0 = time.perf_counter()
        self.OI.ungrid(self.img, self.locs, WIDTH, beta=self.beta)
        self.OI.grid(self.vals, self.locs, (N_GRID,) * 3, WIDTH, beta=self.beta)
        return time.perf_counter() - t0

    def describe(self, t: float, reps: int) -> dict:
        return {
            "value": 2 * self.n * N_COIL / t,
            "unit": "point-coil samples/s",
            "cores": self.threads,
            "kind": "port",
            "sample": f"{self.n} of {N_PTS} points, all {N_COIL} coils, full {N_GRID}^3 grid; ungrid+grid, median of {reps}",
        }


def _median_time(fn, reps: int, warmup: int = 1) -> float:
    for _ in range(warmup):
        fn()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts)


def cpu_config_baselines():
    """The other workloads' CPU baselines: the oracle (the reference's torch
    path restated) on the host cores, each a bounded sample stated beside
    its figure, scaled to the whole workload where the sample is a fixed
    fraction of it (about 20 s in all)."""
    from oracle import blocks as OB
    from oracle import cg as OCG
    from oracle import interp as OI
    from oracle import nufft as ONU
    from torchlinops_gb300 import mri

    threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    torch.set_num_threads(threads)
    out = {"cores": threads, "kind": "port"}
    # plain 2D interpolate, 64^2, 4096 points, W 4, beta for oversampling 1.25 (the whole workload)
    g = torch.Generator().manual_seed(0)
    img = torch.complex(torch.randn(64, 64, generator=g), torch.randn(64, 64, generator=g))
    locs = torch.rand(4096, 2, generator=g) * 64
    pts = torch.complex(torch.randn(4096, generator=g), torch.randn(4096, generator=g))
    beta = kb_beta()
    f = _median_time(lambda: OI.ungrid(img, locs, 4.0, beta=beta), 10, 3)
    a = _median_time(lambda: OI.grid(pts, locs, (64, 64), 4.0, beta=beta), 10, 3)
    out["interp2d_64sq_4096pts"] = {"fwd_ms": f * 1e3, "adj_ms": a * 1e3, "sample": "whole workload, median of 10"}
    # unfold / fold 16 x 160^3 c64, block 8^3, stride 4: one of the 16 batch entries, times 16
    x = torch.complex(torch.randn(1, 160, 160, 160, generator=g), torch.randn(1, 160, 160, 160, generator=g))
    u = _median_time(lambda: OB.unfold(x, BLK, BLK_STRIDE), 3)
    y = OB.unfold(x, BLK, BLK_STRIDE)
    fo = _median_time(lambda: OB.fold(y, BLK_SHAPE[1:], BLK, BLK_STRIDE), 1, 0)
    del x, y
    out["blocks3d_16x160cube"] = {"unfold_ms": 16 * u * 1e3, "fold_ms": 16 * fo * 1e3,
                                  "sample": "1 of 16 batch entries (unfold median of 3, fold one run), scaled by 16"}
    # 2D NUFFT forward / adjoint (float32 arithmetic): 1 of 32 slices x 8 coils, times 32
    SP, RD, N = 402, 512, 256
    ang = torch.arange(SP, dtype=torch.float64) * math.pi * (math.sqrt(5.0) - 1.0) / 2.0
    r = (torch.arange(RD, dtype=torch.float64) - RD // 2) * (N / RD)
    l2 = torch.stack([r[None, :] * torch.cos(ang[:, None]), r[None, :] * torch.sin(ang[:, None])], dim=-1)
    l2 = (l2 + 0.1 * torch.randn(l2.shape, generator=g, dtype=torch.float64)).to(torch.float32)
    xi = torch.complex(torch.randn(8, N, N, generator=g), torch.randn(8, N, N, generator=g))
    ys = torch.complex(torch.randn(8, SP, RD, generator=g), torch.randn(8, SP, RD, generator=g))
    nf = _median_time(lambda: ONU.nufft(xi, l2, dtype=torch.float32), 3)
    na = _median_time(lambda: ONU.nufft_adjoint(ys, l2, (N, N), dtype=torch.float32), 3)
    out["nufft2d_32x8x256sq"] = {"fwd_ms": 32 * nf * 1e3, "adj_ms": 32 * na * 1e3,
                                 "sample": "1 of 32 slices (8 coils), median of 3, scaled by 32"}
    # plain CG to 1e-4 on a reduced normal equation of the same kind: 32^3
    # image, 1 coil, 1024 x 64 Fibonacci-sphere radial points, the data term
    # scaled to a unit largest eigenvalue (power method) plus lam 1e-3, float64
    # (the CG workload itself is 128^3 x 8 coils x 2^20 points)
    n5 = 32
    l5 = mri.radial_trajectory_3d(1024, 64, n5, "cpu")

    def data(v):
        return ONU.nufft_adjoint(ONU.nufft(v, l5), l5, (n5,) * 3)

    v = torch.complex(torch.randn(n5, n5, n5, generator=g), torch.randn(n5, n5, n5, generator=g)).to(torch.complex128)
    for _ in range(15):
        v = data(v)
        v = v / torch.linalg.vector_norm(v)
    scale = 1.0 / float(torch.vdot(v.flatten(), data(v).flatten()).real)
    xt = torch.complex(torch.randn(n5, n5, n5, generator=g), torch.randn(n5, n5, n5, generator=g)).to(torch.complex128)

    def normal(w):
        return scale * data(w) + 1e-3 * w

    b = normal(xt)
    t0 = time.perf_counter()
    _, iters = OCG.cg(normal, b, rtol=1e-4, max_iters=300)
    out["cg_sense_reduced"] = {"seconds": time.perf_counter() - t0, "iters": iters,
                               "sample": "32^3 image, 1 coil, 65,536 radial points, unit-normalised data term + "
                                         "1e-3 I, float64, plain CG to relative residual 1e-4"}
    return out


def cpu_baseline(sample_pts: int, reps: int = 3):
    cs = CpuSample(sample_pts)
    cs.run()  # warm-up
    t = statistics.median(cs.run() for _ in range(reps))
    return cs.describe(t, reps)


def run_reference(args, world, rank):
    if rank != 0:
        return
    cs = CpuSample(args.ref_points)
    per = [cs.run() for _ in range(args.warmup + args.steps)]
    timed = per[args.warmup:]
    t = statistics.median(timed)
    value = 2 * args.ref_points * N_COIL / t
    desc = cs.describe(t, len(timed))
    line = {
        "impl": "reference",
        "metric": "3D multicoil gridding+ungridding throughput (256^3 x 8 coils, 2^21 points, KB W=4)",
        "value": value,
        "unit": "point-coil samples/s",
        "n_gpus": world,  # the job's GPU count; this arm computes on the host cores only
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "c64",
        "data": "synthetic (1/r^2 ball trajectory, N(0,1) complex values), seeded",
        "config": {"workload": f"interp3d_{N_GRID}cube_{N_COIL}coil_{N_PTS}pts", "grid": [N_GRID] * 3, "coils": N_COIL,
                   "points": N_PTS, "width": WIDTH, "oversamp": OVERSAMP, "sample_points": args.ref_points,
                   "step": "ungrid + grid of the sample points on the CPU (reference torch path, restated)",
                   "device": "host CPU"},
        "cpu_baseline": {k: desc[k] for k in ("cores", "kind", "sample")} | {"value": value, "unit": "point-coil samples/s"},
        "e2e": {"value": value, "unit": "point-coil samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU arm


def run_gpu(args, world, rank, local):
    import torchlinops_gb300 as T
    from torchlinops_gb300.interp import get_plan

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    beta = kb_beta()
    kp = dict(beta=beta)
    locs_h = make_locs()
    locs = locs_h.to(dev)
    gen = torch.Generator(device=dev).manual_seed(1234 + rank)
    img = torch.randn(N_COIL, N_GRID, N_GRID, N_GRID, dtype=torch.complex64, device=dev, generator=gen)
    vals = torch.randn(N_COIL, N_PTS, dtype=torch.complex64, device=dev, generator=gen)

    # plan (one-time per trajectory), timed separately
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plan = get_plan(locs, (N_GRID,) * 3, WIDTH, "kaiser_bessel", "circular", beta)
    torch.cuda.synchronize()
    plan_ms = (time.perf_counter() - t0) * 1e3
    # per step: the gather, the point-major value transpose, the gridding and
    # (when dense tiles are split) the ordered sum of their parts
    blocks = plan.info.n_blk_items > 0  # 3D gridding on block lists
    n_split = plan.info.n_blk_split if blocks else plan.info.n_split_tiles
    launches_per_step = 3 + (1 if n_split > 0 else 0)

    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        T.ungrid(img, locs, WIDTH, kernel_params=kp)
        T.grid(vals, locs, (N_GRID,) * 3, WIDTH, kernel_params=kp)
    torch.cuda.synchronize()

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    barrier(world)
    torch.cuda.synchronize()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for i in range(args.steps):
        ev[i][0].record(stream)
        out = T.ungrid(img, locs, WIDTH, kernel_params=kp)
        ev[i][1].record(stream)
        g = T.grid(vals, locs, (N_GRID,) * 3, WIDTH, kernel_params=kp)
        ev[i][2].record(stream)
        del out, g
    t_end.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clocks = sampler.stop()
    total_ms = t_start.elapsed_time(t_end)
    total_ms = max_over_ranks(total_ms, world)
    fwd_ms = statistics.mean(e[0].elapsed_time(e[1]) for e in ev)
    adj_ms = statistics.mean(e[1].elapsed_time(e[2]) for e in ev)
    ms_step = total_ms / args.steps
    value = world * 2 * N_PTS * N_COIL / (ms_step / 1e3)

    # end to end through the public API, pinned host buffers, copies inside
    img_h = torch.empty(img.shape, dtype=img.dtype, pin_memory=True)
    img_h.copy_(img)
    vals_h = torch.empty(vals.shape, dtype=vals.dtype, pin_memory=True)
    vals_h.copy_(vals)
    out_h = torch.empty(N_COIL, N_PTS, dtype=torch.complex64, pin_memory=True)
    grid_h = torch.empty(img.shape, dtype=img.dtype, pin_memory=True)
    e2e_steps = max(2, min(args.steps, 5))
    # the two halves of a step are independent, so they run on two streams:
    # the point values go in first, and the gridding and its 1.07 GB copy
    # back overlap the 1.07 GB grid copy in and the gather
    s_grid, s_ungrid = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    torch.cuda.synchronize()
    e2e_times = []
    for i in range(e2e_steps + 1):
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(s_grid):
            va_d = vals_h.to(dev, non_blocking=True)
            g = T.grid(va_d, locs, (N_GRID,) * 3, WIDTH, kernel_params=kp)
            grid_h.copy_(g, non_blocking=True)
        with torch.cuda.stream(s_ungrid):
            im_d = img_h.to(dev, non_blocking=True)
            o = T.ungrid(im_d, locs, WIDTH, kernel_params=kp)
            out_h.copy_(o, non_blocking=True)
        torch.cuda.synchronize()
        if i > 0:  # first pass is a warm-up of the pinned paths
            e2e_times.append(time.perf_counter() - t0)
        del im_d, va_d, o, g
    e2e_s = max_over_ranks(statistics.median(e2e_times), world)
    h2d = img_h.numel() * 8 + vals_h.numel() * 8
    d2h = out_h.numel() * 8 + grid_h.numel() * 8

    peak, peak_kind = measured_peaks()
    dom_ms = max(adj_ms, fwd_ms)
    dom = "grid" if adj_ms >= fwd_ms else "ungrid"
    achieved = ALGO_BYTES / (dom_ms / 1e3) / 1e9
    kernels = {
        "ungrid": {"ms": fwd_ms, "GBps": ALGO_BYTES / (fwd_ms / 1e3) / 1e9,
                   "frac": ALGO_BYTES / (fwd_ms / 1e3) / 1e9 / peak},
        "grid": {"ms": adj_ms, "GBps": ALGO_BYTES / (adj_ms / 1e3) / 1e9,
                 "frac": ALGO_BYTES / (adj_ms / 1e3) / 1e9 / peak,
                 "split": ({"blocks": int(plan.info.n_blk_split), "partial_blocks": int(plan.info.n_blk_partials),
                            "block_entries": int(plan.info.n_blk_entries), "items": int(plan.info.n_blk_items)}
                           if blocks else {"tiles": int(plan.info.n_split_tiles),
                                           "partial_tiles": int(plan.info.n_partials)})},
        "plan_build_ms": plan_ms,
        "plan_entries": int(plan.info.n_entries),
    }
    del img, vals, img_h, grid_h
    torch.cuda.empty_cache()
    kernels["one_coil"] = bench_one_coil(locs, dev, peak)
    if not args.skip_blocks:
        kernels.update(bench_blocks(dev, peak, args))
    if not args.skip_nufft2d:
        kernels["nufft2d"] = bench_nufft2d(dev, peak)
    if not args.skip_nufft3d:
        kernels["nufft3d"] = bench_nufft3d(locs_h, dev)
    if not args.skip_blocks:
        kernels["index"] = bench_index(dev, peak)
    line = None
    if rank == 0:
        cpu = cpu_others = None
        if world == 1 and not args.skip_cpu:
            cpu = cpu_baseline(args.ref_sample)
            cpu_others = cpu_config_baselines()
        cg = None
        if world == 1 and not args.skip_cg:
            cg = bench_cg(dev, args)
        line = {
            "metric": "3D multicoil gridding+ungridding throughput (256^3 x 8 coils, 2^21 points, KB W=4)",
            "value": value,
            "unit": "point-coil samples/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_step,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "c64",
            "data": "synthetic (1/r^2 ball trajectory, N(0,1) complex values), seeded",
            "config": {
                "workload": f"interp3d_{N_GRID}cube_{N_COIL}coil_{N_PTS}pts",
                "grid": [N_GRID] * 3,
                "coils": N_COIL,
                "points": N_PTS,
                "width": WIDTH,
                "oversamp": OVERSAMP,
                "kernel": "kaiser_bessel",
                "step": "ungrid + grid (interpolation half of one normal op)",
                "l2": "inputs larger than L2 (grid 1.07 GB per direction); no flush",
                "e2e": "pinned host buffers; per step the inputs in and the results out, the grid and ungrid halves on two streams",
                "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            },
            "e2e": {
                "value": world * 2 * N_PTS * N_COIL / e2e_s,
                "unit": "point-coil samples/s",
                "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
            },
            "roofline": {
                "kernel": dom,
                "bound": "hbm",
                "achieved": achieved,
                "peak": peak,
                "peak_kind": peak_kind,
                "unit": "GB/s",
                "frac": achieved / peak,
                "traffic": profiled_traffic(),
                "algorithmic_bytes_per_launch": ALGO_BYTES,
            },
            "cpu_baseline": cpu,
            "cpu_baselines_other_workloads": cpu_others,
            "clocks": clocks,
            "gpu_launches": launches_per_step * args.steps,
            "kernels": kernels,
            "cg": cg,
        }
        print(json.dumps(line), flush=True)
    return line


def bench_blocks(dev, peak, args):
    """ArrayToBlocks / BlocksToArray, 16 x 160^3 complex64, block 8^3, stride 4."""
    import torchlinops_gb300 as T

    gen = torch.Generator(device=dev).manual_seed(7)
    x = torch.randn(BLK_SHAPE, dtype=torch.complex64, device=dev, generator=gen)
    nb = tuple((s - b) // st + 1 for s, b, st in zip(BLK_SHAPE[1:], BLK, BLK_STRIDE))
    nbytes = x.numel() * 8 + BLK_SHAPE[0] * math.prod(nb) * math.prod(BLK) * 8
    y = T.unfold(x, BLK, BLK_STRIDE)
    for _ in range(3):
        T.unfold(x, BLK, BLK_STRIDE, output=y)
        T.fold(y, BLK_SHAPE[1:], BLK, BLK_STRIDE, output=x)
    torch.cuda.synchronize()
    reps = max(3, min(args.steps, 10))
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    s = torch.cuda.current_stream(dev)
    e[0].record(s)
    for _ in range(reps):
        T.unfold(x, BLK, BLK_STRIDE, output=y)
    e[1].record(s)
    for _ in range(reps):
        T.fold(y, BLK_SHAPE[1:], BLK, BLK_STRIDE, output=x)
    e[2].record(s)
    torch.cuda.synchronize()
    u_ms = e[0].elapsed_time(e[1]) / reps
    f_ms = e[1].elapsed_time(e[2]) / reps
    del x, y
    torch.cuda.empty_cache()
    return {
        "unfold": {"ms": u_ms, "GBps": nbytes / (u_ms / 1e3) / 1e9, "frac": nbytes / (u_ms / 1e3) / 1e9 / peak,
                   "workload": f"{BLK_SHAPE[0]}x160^3 c64, block 8^3, stride 4"},
        "fold": {"ms": f_ms, "GBps": nbytes / (f_ms / 1e3) / 1e9, "frac": nbytes / (f_ms / 1e3) / 1e9 / peak},
    }


def bench_nufft2d(dev, peak):
    """The differentiable 2D NUFFT: 32 slices x 8 coils of a 256^2 complex64
    image (padded 320^2), golden-angle radial 402 spokes x 512 readouts with
    N(0, 0.1) jitter, through the functional nufft. Times the forward, the
    forward + backward for the image gradient (trajectory fixed: one plan),
    and the forward + backward for image and trajectory gradients (the plan
    is rebuilt every call, as when the trajectory changes each step)."""
    from torchlinops_gb300 import linops

    S, C, N, SP, RD = 32, 8, 256, 402, 512
    g = torch.Generator().manual_seed(4)
    ang = torch.arange(SP, dtype=torch.float64) * math.pi * (math.sqrt(5.0) - 1.0) / 2.0
    r = (torch.arange(RD, dtype=torch.float64) - RD // 2) * (N / RD)
    locs = torch.stack([r[None, :] * torch.cos(ang[:, None]), r[None, :] * torch.sin(ang[:, None])], dim=-1)
    locs = (locs + 0.1 * torch.randn(locs.shape, generator=g, dtype=torch.float64)).to(torch.float32).to(dev)
    gd = torch.Generator(device=dev).manual_seed(5)
    x = torch.randn(S, C, N, N, dtype=torch.complex64, device=dev, generator=gd)
    a = torch.randn(S, C, SP, RD, dtype=torch.complex64, device=dev, generator=gd)
    s = torch.cuda.current_stream(dev)

    def timed(fn, reps=10):
        # median of per-call CUDA-event times (a call includes host work:
        # autograd, plan lookups), so one slow call does not skew the figure
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
        for e0, e1 in ev:
            e0.record(s)
            fn()
            e1.record(s)
        torch.cuda.synchronize()
        return statistics.median(e0.elapsed_time(e1) for e0, e1 in ev)

    def fwd():
        with torch.no_grad():
            linops.nufft(x, locs)

    xg = x.clone().requires_grad_(True)

    def fwd_bwd_image():
        xg.grad = None
        (a.conj() * linops.nufft(xg, locs)).real.sum().backward()

    lg = locs.clone().requires_grad_(True)

    def fwd_bwd_both():
        xg.grad = None
        lg.grad = None
        (a.conj() * linops.nufft(xg, lg)).real.sum().backward()

    f_ms, fb_ms, fbl_ms = timed(fwd), timed(fwd_bwd_image), timed(fwd_bwd_both)
    # one ungrid of this workload: grid 256 x 320^2 c64 + locs + 256 x 205,824 c64 values
    ungrid_bytes = S * C * 320 * 320 * 8 + SP * RD * 2 * 4 + S * C * SP * RD * 8
    # the trajectory-gradient kernel alone, on the padded grid and the point
    # cotangents of this workload: reads the 256 x 320^2 grid, the 256 x
    # 205,824 point values and the locations, writes the gradient
    from torchlinops_gb300 import interp as I

    kl = linops.prep_locs(locs, (N, N), (320, 320))
    gk = torch.randn(S * C, 320, 320, dtype=torch.complex64, device=dev, generator=gd)
    beta = I.kaiser_bessel_beta(4.0, 1.25)
    grad_ms = timed(lambda: I._grad_locs(gk, a.reshape(S * C, SP, RD), kl, 4.0, "kaiser_bessel", 1, "circular",
                                         dict(beta=beta)))
    grad_bytes = S * C * 320 * 320 * 8 + S * C * SP * RD * 8 + 2 * SP * RD * 2 * 4
    del x, a, xg, lg, gk
    torch.cuda.empty_cache()
    return {
        "workload": "32 slices x 8 coils x 256^2 c64, padded 320^2, golden-angle radial 402 x 512 (+N(0,0.1) jitter)",
        "fwd_ms": f_ms,
        "fwd_bwd_image_ms": fb_ms,
        "fwd_bwd_image_and_locs_ms": fbl_ms,
        "ungrid_algorithmic_bytes": ungrid_bytes,
        "samples_per_s_fwd": S * C * SP * RD / (f_ms / 1e3),
        "grad_locs_kernel": {"ms": grad_ms, "algorithmic_bytes": grad_bytes,
                             "GBps": grad_bytes / (grad_ms / 1e3) / 1e9,
                             "frac": grad_bytes / (grad_ms / 1e3) / 1e9 / peak},
    }


def bench_cg(dev, args):
    """Learned-preconditioned vs plain CG to relative residual 1e-4 on 3D
    SENSE: 128^3 image, 8 Gaussian coil maps, 3D radial 2048 spokes x 512
    readouts (2^20 points), lam = 1e-3, A normalised by the power method.
    Wall time of each solve (float64 true residual included); the
    preconditioner is trained here first, on the GPU, by the package's own
    convolution kernels (its time is reported separately)."""
    from torchlinops_gb300 import alg, mri, precond

    n, ncoil, nspokes, nread, lam = 128, 8, 2048, 512, 1e-3
    locs = mri.radial_trajectory_3d(nspokes, nread, n, dev)
    maps = mri.gaussian_coil_maps_3d(ncoil, n, device=dev)
    A = mri.SenseNormal(locs, maps, lam=lam)
    xt = mri.ellipsoid_phantom_3d(n, 10, torch.Generator().manual_seed(1234), dev)
    b = A(xt)

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps * 1e3

    def solve(M):
        alg.cg_solve(A, b, rtol=1e-4, max_iters=500, M=M)  # warm-up
        runs = [alg.cg_solve(A, b, rtol=1e-4, max_iters=500, M=M)[1] for _ in range(3)]
        best = min(runs, key=lambda i: i.seconds)
        return {"iters": best.iters, "seconds": best.seconds, "converged": best.converged,
                "true_rel_residual": best.true_rel_residual, "fallback": best.fallback}

    normal_ms = timed(lambda: A(b))
    toeplitz = bench_toeplitz(locs, maps, xt, n, dev)
    plain = solve(None)
    M = precond.CNNPreconditioner(dev, seed=1, init="laplacian", c0=0.02)
    warm = solve(M)
    batch = 4
    # training data: seeded 10-ellipsoid phantoms (+5% noise) solved by plain
    # CG to 1e-6, the recipe of this workload with fewer phantoms than its
    # 2000 (about 0.3 s of CG each); batches drawn from them with replacement
    t0 = time.perf_counter()
    pairs = mri.cg_solution_pairs(A, n, args.precond_phantoms, seed=5000, device=dev)
    gen_s = time.perf_counter() - t0
    gen = torch.Generator().manual_seed(0)

    def cg_batch(step):
        idx = torch.randint(0, len(pairs), (batch,), generator=gen)
        return [pairs[int(i)] for i in idx]

    log = M.fit(cg_batch, args.cg_steps, lr=1e-3, log_every=max(args.cg_steps // 10, 1))
    learned = solve(M)
    m_ms = timed(lambda: M(b))
    del pairs
    compare = None
    if args.precond_compare:
        # the same network and step count trained on (r = A e, e) pairs, e
        # random k-space shells and phantom-plus-noise fields
        M2 = precond.CNNPreconditioner(dev, seed=1, init="laplacian", c0=0.02)
        gen2 = torch.Generator().manual_seed(0)
        log2 = M2.fit(lambda step: mri.training_batch(A, n, gen2, batch, dev), args.cg_steps, lr=1e-3)
        learned2 = solve(M2)
        compare = {"train_seconds": log2.seconds, "learned": learned2,
                   "speedup_wall": plain["seconds"] / learned2["seconds"],
                   "speedup_iters": plain["iters"] / learned2["iters"]}
        del M2
    return {
        "workload": f"sense3d_{n}cube_{ncoil}coil_{nspokes}x{nread}radial_lam{lam:g}",
        "rtol": 1e-4,
        "normal_op_ms": normal_ms,
        "toeplitz": toeplitz,
        "preconditioner_ms": m_ms,
        "plain": plain,
        "warm_start": warm,
        "learned": learned,
        "speedup_wall": plain["seconds"] / learned["seconds"],
        "speedup_iters": plain["iters"] / learned["iters"],
        "trained_on_random_fields": compare,
        "train": {"source": f"{args.precond_phantoms} seeded phantoms (+5% noise) solved by plain CG to 1e-6",
                  "generation_seconds": gen_s, "steps": args.cg_steps, "samples": args.cg_steps * batch,
                  "seconds": log.seconds,
                  "loss_first": log.losses[0][1] if log.losses else None,
                  "loss_last": log.losses[-1][1] if log.losses else None},
        "data": "synthetic: ellipsoid phantom, Gaussian coil maps, Fibonacci-sphere radial trajectory, seeded",
    }


def bench_nufft3d(locs_h, dev):
    """The same trajectory at the NUFFT level: 8 coil images of 205^3
    (padded 1.25x to 256^3), the ball's points centred and scaled by 205/256.
    Forward (apodize, pad, centred FFT, ungrid, scale), adjoint and the
    explicit normal operator (forward then adjoint), each the median of 3
    CUDA-event timings; the plan is built before the timings."""
    from torchlinops_gb300 import linops

    n = 205
    locs = ((locs_h - N_GRID / 2) * (n / N_GRID)).to(dev)
    gen = torch.Generator(device=dev).manual_seed(7)
    x = torch.randn(N_COIL, n, n, n, dtype=torch.complex64, device=dev, generator=gen)
    A = linops.NUFFT(locs, (n,) * 3)
    s = torch.cuda.current_stream(dev)
    y = A(x)
    AH, AN = A.H, A.normal()
    AH(y)
    torch.cuda.synchronize()

    def med(fn, reps=3):
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            fn()
            e1.record(s)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    out = {"workload": f"3D NUFFT, {N_COIL} coils x {n}^3 c64, padded to {int(n * 1.25)}^3, {locs.shape[0]} points",
           "forward_ms": med(lambda: A(x)), "adjoint_ms": med(lambda: AH(y)), "normal_ms": med(lambda: AN(x))}
    del x, y, A, AH, AN
    torch.cuda.empty_cache()
    return out


def bench_one_coil(locs, dev, peak):
    """The headline trajectory with one batch entry (a one-coil NUFFT, the
    Toeplitz kernel's single image): ungrid a 256^3 complex image at the 2^21
    points and grid the points back, each the mean of 10 CUDA-event timings
    with a 512 MB write between timings to flush L2 (the image alone is about
    the size of L2). The 8-entry kernels run with the other 7 entries empty;
    the algorithmic bytes are one entry's grid and values plus the
    coordinates."""
    import torchlinops_gb300 as T

    kp = dict(beta=kb_beta())
    gen = torch.Generator(device=dev).manual_seed(11)
    img = torch.randn(1, N_GRID, N_GRID, N_GRID, dtype=torch.complex64, device=dev, generator=gen)
    vals = torch.randn(1, N_PTS, dtype=torch.complex64, device=dev, generator=gen)
    flush = torch.empty(1 << 27, dtype=torch.float32, device=dev)
    s = torch.cuda.current_stream(dev)
    for _ in range(3):
        T.ungrid(img, locs, WIDTH, kernel_params=kp)
        T.grid(vals, locs, (N_GRID,) * 3, WIDTH, kernel_params=kp)

    def mean_ms(fn, reps=10):
        ts = []
        for _ in range(reps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            fn()
            e1.record(s)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.mean(ts)

    fwd = mean_ms(lambda: T.ungrid(img, locs, WIDTH, kernel_params=kp))
    adj = mean_ms(lambda: T.grid(vals, locs, (N_GRID,) * 3, WIDTH, kernel_params=kp))
    algo = N_GRID**3 * 8 + N_PTS * 3 * 4 + N_PTS * 8
    del img, vals, flush
    torch.cuda.empty_cache()

    def entry(ms):
        gbps = algo / (ms / 1e3) / 1e9
        return {"ms": ms, "GBps": gbps, "frac": gbps / peak, "samples_per_s": N_PTS / (ms / 1e3)}

    return {"workload": f"interp3d_{N_GRID}cube_1coil_{N_PTS}pts", "algorithmic_bytes": algo,
            "l2": "512 MB write between timings", "ungrid": entry(fwd), "grid": entry(adj)}


def bench_toeplitz(locs, maps, xt, n, dev):
    """The NUFFT normal operator on the 8 coil images S_c x of the CG workload
    (128^3, 2^20 radial points): its Toeplitz embedding (PSF kernel on the 2x
    grid, built once; then pad + FFT + multiply + inverse FFT + crop) against
    the explicit chain (forward NUFFT then adjoint), each the median of 5
    CUDA-event timings, and the two results' relative difference."""
    from torchlinops_gb300 import linops

    x8 = (maps * xt[None]).contiguous()
    s = torch.cuda.current_stream(dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    T = linops.NUFFT(locs, (n,) * 3, toeplitz=True).normal()
    T(x8[:1])
    torch.cuda.synchronize()
    build_ms = (time.perf_counter() - t0) * 1e3
    E = linops.NUFFT(locs, (n,) * 3).normal()

    def med(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            fn()
            e1.record(s)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    t_ms = med(lambda: T(x8))
    e_ms = med(lambda: E(x8))
    t1_ms = med(lambda: T(x8[:1]))
    e1_ms = med(lambda: E(x8[:1]))
    ty, ey = T(x8), E(x8)
    rel = float(torch.linalg.vector_norm((ty - ey).flatten()) / torch.linalg.vector_norm(ey.flatten()))
    del x8, ty, ey, T, E
    torch.cuda.empty_cache()
    return {"workload": f"NUFFT normal of 8 coil images, {n}^3, {locs.shape[0]} radial points",
            "toeplitz_ms": t_ms, "explicit_ms": e_ms, "toeplitz_1coil_ms": t1_ms, "explicit_1coil_ms": e1_ms,
            "kernel_build_ms": build_ms, "rel_diff_vs_explicit": rel}


def bench_index(dev, peak):
    """Sampling at integer locations (the Sampling linop, NUFFT mode
    "sampling"): the reference's own benchmark shape for index_adjoint
    (functional/_index/tests/bench_indexing.py: float32 values of shape
    48 x 500 x 1600, one random index per dim into a 220^3 grid) and a
    multicoil case (8 coils complex64, 2^20 samples into 160^3). Plans are
    built once per index set (timed separately); each figure is the median
    of 10 CUDA-event timings."""
    import torchlinops_gb300 as T

    s = torch.cuda.current_stream(dev)

    def med(fn, reps=10):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            fn()
            e1.record(s)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)

    out = {}
    gd = torch.Generator(device=dev).manual_seed(9)
    cases = (("float32_48x500x1600_into_220cube", (220, 220, 220), (48, 500, 1600), 1, torch.float32),
             ("c64_8coil_2^20_into_160cube", (160, 160, 160), (1 << 20,), 8, torch.complex64))
    for name, grid, shape, coils, dt in cases:
        idx = tuple(torch.randint(0, n, shape, device=dev, generator=gd) for n in grid)
        vshape = ((coils,) if coils > 1 else ()) + shape
        vals = torch.randn(vshape, dtype=dt, device=dev, generator=gd)
        img = torch.randn(((coils,) if coils > 1 else ()) + grid, dtype=dt, device=dev, generator=gd)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        T.index_adjoint(vals, idx, grid)
        torch.cuda.synchronize()
        first_ms = (time.perf_counter() - t0) * 1e3
        adj_ms = med(lambda: T.index_adjoint(vals, idx, grid))
        fwd_ms = med(lambda: T.index(img, idx))
        m = math.prod(shape)
        es = vals.element_size()
        # values in and the grid out (adjoint) or the grid in and samples out
        # (forward), plus the 4-byte cell of each sample the plan holds
        nbytes = coils * m * es + coils * math.prod(grid) * es + 4 * m
        out[name] = {"adjoint_ms": adj_ms, "forward_ms": fwd_ms, "first_call_with_plan_ms": first_ms,
                     "algorithmic_bytes": nbytes, "adjoint_GBps": nbytes / (adj_ms / 1e3) / 1e9,
                     "adjoint_frac": nbytes / (adj_ms / 1e3) / 1e9 / peak,
                     "forward_GBps": nbytes / (fwd_ms / 1e3) / 1e9}
        del idx, vals, img
        torch.cuda.empty_cache()
    return out


def _resize(grid: int, points: int) -> None:
    global N_GRID, N_PTS, ALGO_BYTES
    N_GRID, N_PTS = grid, points
    ALGO_BYTES = N_COIL * N_GRID**3 * 8 + N_PTS * 3 * 4 + N_COIL * N_PTS * 8


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="tlgb", choices=["tlgb", "reference"])
    ap.add_argument("--ref-sample", type=int, default=1 << 19,
                    help="points in the GPU arm's CPU baseline sample (about 10 s of CPU work)")
    ap.add_argument("--ref-points", type=int, default=None,
                    help="points per step of the reference arm (default: all of them, the same workload as the GPU arm)")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-blocks", action="store_true")
    ap.add_argument("--skip-cg", action="store_true", help="skip the learned vs plain CG comparison")
    ap.add_argument("--skip-nufft2d", action="store_true", help="skip the differentiable 2D NUFFT timing")
    ap.add_argument("--skip-nufft3d", action="store_true", help="skip the 3D NUFFT-level timing (205^3 x 8 coils)")
    ap.add_argument("--cg-steps", type=int, default=500, help="preconditioner training steps (4 samples each)")
    ap.add_argument("--precond-phantoms", type=int, default=64,
                    help="phantoms solved by plain CG to 1e-6 for the preconditioner's training data")
    ap.add_argument("--precond-compare", action="store_true",
                    help="also train on random (A e, e) pairs and report that network")
    ap.add_argument("--grid", type=int, default=N_GRID, help="grid edge (smaller cases for profiling)")
    ap.add_argument("--points", type=int, default=N_PTS, help="number of points (smaller cases for profiling)")
    ap.add_argument("--blocks-batch", type=int, default=BLK_SHAPE[0],
                    help="array entries of the unfold/fold workload (smaller cases for profiling)")
    ap.add_argument("--nufft2d-only", action="store_true",
                    help="profiling: run only the 2D NUFFT timing and print its figures (not the bench line)")
    ap.add_argument("--index-only", action="store_true",
                    help="profiling: run only the sampling-op timing and print its figures (not the bench line)")
    args = ap.parse_args()
    _resize(args.grid, args.points)
    if args.ref_points is None:
        args.ref_points = N_PTS
    globals()["BLK_SHAPE"] = (args.blocks_batch,) + BLK_SHAPE[1:]
    args.warmup = max(args.warmup, 3)
    if args.nufft2d_only or args.index_only:
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(dev)
        if args.nufft2d_only:
            print(json.dumps({"nufft2d": bench_nufft2d(dev, measured_peaks()[0])}), flush=True)
        else:
            print(json.dumps({"index": bench_index(dev, measured_peaks()[0])}), flush=True)
        return
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
