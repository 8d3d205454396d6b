"""Shared pytest setup: import paths, the ``gpu`` marker, golden-fixture loaders."""

import json
import os
import sys

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_ROOT = os.path.join(ROOT, "torch-named-linops_gb300")
for p in (ROOT, PKG_ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running test")


def pytest_collection_modifyitems(config, items):
    if torch.cuda.is_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


def to_torch(a: np.ndarray, is_complex: bool) -> torch.Tensor:
    t = torch.from_numpy(np.ascontiguousarray(a))
    return torch.view_as_complex(t) if is_complex else t


def load_cases(name: str):
    """Golden cases of ``tests/golden/<name>.npz`` as {case: {field: value}}."""
    data = np.load(os.path.join(GOLDEN, name))
    cases = {}
    for key in data.files:
        case, field = key.split("|")
        cases.setdefault(case, {})[field] = data[key]
    for rec in cases.values():
        if "meta" in rec:
            rec["meta"] = json.loads(str(rec["meta"]))
    return cases


def rel_l2(a: torch.Tensor, b: torch.Tensor) -> float:
    a = a.to(torch.complex128) if a.is_complex() or b.is_complex() else a.double()
    b = b.to(a.dtype)
    den = torch.linalg.vector_norm(b).item()
    num = torch.linalg.vector_norm(a - b).item()
    return num / den if den > 0 else num
