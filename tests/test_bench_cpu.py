"""bench.py's output contract, on the CPU: the reference arm at a tiny size
prints one JSON line with the keys the benchmark contract names, and the GPU
arm refuses to run without a GPU (there is no CPU fallback to time)."""

import json
import os
import subprocess
import sys

import pytest
import torch

from conftest import ROOT

TINY = ["--grid", "32", "--points", "4096", "--steps", "1", "--warmup", "1"]


def _run(*args):
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, capture_output=True,
                          text=True, timeout=600)


def test_reference_arm_prints_the_contract_line():
    r = _run("--impl", "reference", *TINY)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 1 and line["steps"] == 1
    assert line["warmup"] >= 3  # the contract's minimum, whatever was asked
    assert line["unit"] == "point-coil samples/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["ms_per_step"] > 0 and line["vs_baseline"] is None
    assert line["config"]["workload"] == "interp3d_32cube_8coil_4096pts"
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a GPU")
def test_gpu_arm_fails_loudly_without_a_gpu():
    r = _run("--skip-cpu", "--skip-blocks", "--skip-cg", "--skip-nufft2d", "--skip-nufft3d", *TINY)
    assert r.returncode != 0
    assert not r.stdout.strip().startswith("{")
