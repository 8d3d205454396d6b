"""Compile the tlgb CUDA library (libtlgb.so) in-tree for sm_103a.

    python -m torchlinops_gb300._build        # from torch-named-linops_gb300/

Every ``csrc/*.cu`` translation unit is compiled in parallel with nvcc for
``arch=compute_103a,code=sm_103a`` and linked into
``torchlinops_gb300/_lib/libtlgb.so``. Only the sources that changed since the
last build are recompiled. No torch headers are involved: the library exposes
a plain C ABI (``include/tlgb.h``).
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
PROJECT_DIR = os.path.dirname(PKG_DIR)
REPO_DIR = os.path.dirname(PROJECT_DIR)
CSRC = os.path.join(PROJECT_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
BUILD_DIR = os.path.join(PROJECT_DIR, "_build")
LIB_DIR = os.path.join(PKG_DIR, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libtlgb.so")
# debug variant: selected global and shared-memory indices range-checked
# (-DTLGB_CHECKED); a failed check is reported by tlgb_device_status (bit 4)
CHECKED_BUILD_DIR = os.path.join(PROJECT_DIR, "_build_checked")
CHECKED_LIB_PATH = os.path.join(LIB_DIR, "libtlgb_checked.so")

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "--expt-relaxed-constexpr",
]


def _nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the tlgb CUDA library cannot be built")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None, checked: bool = False) -> str:
    """Build libtlgb.so (or, with ``checked``, the range-checked debug variant
    libtlgb_checked.so) if any source or header is newer; return its path."""
    build_dir = CHECKED_BUILD_DIR if checked else BUILD_DIR
    lib_path = CHECKED_LIB_PATH if checked else LIB_PATH
    flags = NVCC_FLAGS + (["-DTLGB_CHECKED"] if checked else [])
    os.makedirs(build_dir, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    objs, todo = [], []
    for src in _sources():
        obj = os.path.join(build_dir, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH_FLAGS, *flags, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
            todo.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for out in ex.map(run, todo):
                if verbose and out:
                    print(out)
    if todo or _stale(lib_path, objs):
        tmp = lib_path + ".tmp"
        cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", tmp, *objs]
        run(cmd)
        os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, checked="--checked" in sys.argv))
