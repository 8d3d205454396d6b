"""ctypes binding of the tlgb C ABI (``include/tlgb.h``).

The CUDA library is the only compute path of this package: there is no CPU
or Triton fallback. ``lib()`` raises if ``libtlgb.so`` has not been built and
``check_cuda`` raises for tensors that are not on a CUDA device.
"""

from __future__ import annotations

import ctypes
import os
import threading

import torch

from ._build import LIB_PATH

TLGB_OK = 0
TLGB_ERR_INVALID = 1
TLGB_ERR_UNSUPPORTED = 2
TLGB_ERR_CUDA = 3
TLGB_ERR_WORKSPACE = 4
TLGB_ERR_DEVICE = 5

KERNELS = {"kaiser_bessel": 0, "spline": 1}
PAD_MODES = {"circular": 0, "zero": 1}

BLOCK_DTYPES = {torch.float32: 0, torch.float64: 1, torch.complex64: 2, torch.complex128: 3}


class InterpDesc(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int32),
        ("kernel", ctypes.c_int32),
        ("norm", ctypes.c_int32),
        ("pad_mode", ctypes.c_int32),
        ("is_complex", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("grid_size", ctypes.c_int64 * 3),
        ("width", ctypes.c_float * 3),
        ("beta", ctypes.c_float),
        ("nbatch", ctypes.c_int64),
        ("npts", ctypes.c_int64),
    ]


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("n_entries", ctypes.c_int64),
        ("n_tiles", ctypes.c_int64),
        ("tile", ctypes.c_int32 * 3),
        ("n_tile", ctypes.c_int32 * 3),
        ("n_fwd_items", ctypes.c_int64),
        ("n_adj_items", ctypes.c_int64),
        ("n_partials", ctypes.c_int64),
        ("n_split_tiles", ctypes.c_int64),
        ("chunk", ctypes.c_int64),
        ("off_entries", ctypes.c_int64),
        ("off_fwd_items", ctypes.c_int64),
        ("off_adj_items", ctypes.c_int64),
        ("off_split", ctypes.c_int64),
        ("plan_bytes", ctypes.c_int64),
        ("n_home", ctypes.c_int64),
        ("off_records", ctypes.c_int64),
        ("kernel_key", ctypes.c_int64),
        ("n_blk_entries", ctypes.c_int64),
        ("n_blk_items", ctypes.c_int64),
        ("n_blk_partials", ctypes.c_int64),
        ("n_blk_split", ctypes.c_int64),
        ("off_blk_entries", ctypes.c_int64),
        ("off_blk_items", ctypes.c_int64),
        ("off_blk_split", ctypes.c_int64),
        ("off_blk_rows", ctypes.c_int64),
    ]


class BlocksDesc(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("nbatch", ctypes.c_int64),
        ("im_size", ctypes.c_int64 * 3),
        ("block", ctypes.c_int64 * 3),
        ("stride", ctypes.c_int64 * 3),
        ("nnz", ctypes.c_int64),
        ("mask_idx", ctypes.c_void_p),
        ("mask_inv", ctypes.c_void_p),
    ]


INDEX_MAX_DIM = 8
# element types of the sampling ops (include/tlgb.h); raw types are copied only
TLGB_I32, TLGB_I64, TLGB_RAW8, TLGB_RAW16 = 4, 5, 6, 7


class IndexDesc(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("nbatch", ctypes.c_int64),
        ("grid_size", ctypes.c_int64 * INDEX_MAX_DIM),
        ("npts", ctypes.c_int64),
    ]


class IndexPlanInfo(ctypes.Structure):
    _fields_ = [
        ("ncells", ctypes.c_int64),
        ("npts", ctypes.c_int64),
        ("off_flat", ctypes.c_int64),
        ("off_perm", ctypes.c_int64),
        ("off_cells", ctypes.c_int64),
        ("plan_bytes", ctypes.c_int64),
    ]


CIRCPAD_MAX_DIM = 8


class CircPadDesc(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("nbatch", ctypes.c_int64),
        ("size", ctypes.c_int64 * CIRCPAD_MAX_DIM),
        ("pad_lo", ctypes.c_int64 * CIRCPAD_MAX_DIM),
        ("pad_hi", ctypes.c_int64 * CIRCPAD_MAX_DIM),
    ]


class ConvDesc(ctypes.Structure):
    _fields_ = [
        ("D", ctypes.c_int32),
        ("H", ctypes.c_int32),
        ("W", ctypes.c_int32),
        ("cin", ctypes.c_int32),
        ("cout", ctypes.c_int32),
        ("mode", ctypes.c_int32),
        ("out_f32", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


_P = ctypes.c_void_p
_SIGNATURES = {
    "tlgb_last_error": ([], ctypes.c_char_p),
    "tlgb_version": ([], ctypes.c_int),
    "tlgb_device_status": ([ctypes.POINTER(ctypes.c_int32), ctypes.c_int32], ctypes.c_int),
    "tlgb_test_skip_region_copy": ([ctypes.c_int32], ctypes.c_int),
    "tlgb_interp_plan_size": ([_P, _P, _P], ctypes.c_int),
    "tlgb_interp_plan_build": ([_P, _P, _P, ctypes.c_size_t, _P, ctypes.c_size_t, _P, _P], ctypes.c_int),
    "tlgb_interp_adjoint_scratch_size": ([_P, _P, _P], ctypes.c_int),
    "tlgb_interp_forward": ([_P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "tlgb_interp_adjoint": ([_P, _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "tlgb_interp_grad_scratch_size": ([_P, _P, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "tlgb_interp_grad_locs": ([_P, _P, _P, _P, _P, _P, _P, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "tlgb_interp_adjoint_fixed": ([_P, _P, _P, _P, _P, _P, _P], ctypes.c_int),
    "tlgb_unfold": ([_P, _P, _P, _P], ctypes.c_int),
    "tlgb_fold": ([_P, _P, _P, _P], ctypes.c_int),
    "tlgb_index_plan_size": ([_P, _P, _P], ctypes.c_int),
    "tlgb_index_plan_build": ([_P, _P, _P, ctypes.c_size_t, _P, ctypes.c_size_t, _P, _P], ctypes.c_int),
    "tlgb_index_forward": ([_P, _P, _P, _P, _P, _P], ctypes.c_int),
    "tlgb_index_adjoint": ([_P, _P, _P, _P, _P, _P], ctypes.c_int),
    "tlgb_circular_pad": ([_P, _P, _P, _P], ctypes.c_int),
    "tlgb_circular_pad_adjoint": ([_P, _P, _P, _P], ctypes.c_int),
    "tlgb_cg_scratch_bytes": ([], ctypes.c_size_t),
    "tlgb_dot_f64": ([_P, _P, ctypes.c_int64, ctypes.c_int, _P, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "tlgb_cg_set_pap": ([_P, _P, ctypes.c_int64, ctypes.c_int, _P, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "tlgb_cg_step": ([_P, _P, _P, _P, ctypes.c_int64, ctypes.c_int, _P, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "tlgb_pcg_update": ([_P, _P, _P, _P, ctypes.c_int64, ctypes.c_int, _P, _P], ctypes.c_int),
    "tlgb_pcg_direction": ([_P, _P, _P, _P, ctypes.c_int64, ctypes.c_int, _P, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "tlgb_pad_shift_c64": ([_P, ctypes.c_int64, ctypes.c_int32, _P, _P, _P, _P, ctypes.c_int32, _P, _P,
                            ctypes.c_int32, _P, _P], ctypes.c_int),
    "tlgb_crop_shift_c64": ([_P, ctypes.c_int64, ctypes.c_int32, _P, _P, _P, _P, ctypes.c_int32, _P, _P,
                             ctypes.c_int32, ctypes.c_float, _P, ctypes.c_float, _P, _P], ctypes.c_int),
    "tlgb_conv3d_fwd": ([_P, _P, _P, _P, _P, _P], ctypes.c_int),
    "tlgb_conv3d_wgrad_scratch_size": ([_P, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int),
    "tlgb_conv3d_wgrad": ([_P, _P, _P, _P, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "tlgb_conv3d_pack": ([_P, ctypes.c_int64, _P, ctypes.c_int32, _P, _P], ctypes.c_int),
    "tlgb_conv3d_unpack": ([_P, _P, ctypes.c_int64, _P, ctypes.c_float, _P, _P], ctypes.c_int),
}

# conv3d epilogue modes (include/tlgb.h)
TLGB_CONV_PLAIN, TLGB_CONV_RELU, TLGB_CONV_MASK = 0, 1, 2

# float64 CG state vector slots (include/tlgb.h)
CG_RS, CG_RS_OLD, CG_PAP, CG_ALPHA, CG_BETA, CG_ITERS, CG_TMP, CG_STATE_LEN = 0, 1, 2, 3, 4, 5, 6, 8

_lib = None
_lock = threading.Lock()


def lib_path() -> str:
    return os.environ.get("TLGB_LIBRARY") or LIB_PATH


def lib() -> ctypes.CDLL:
    """The loaded tlgb library; raises if it has not been built."""
    global _lib
    if _lib is None:
        with _lock:
            if _lib is None:
                path = lib_path()
                if not os.path.exists(path):
                    raise RuntimeError(
                        f"tlgb CUDA library not found at {path}; build it with "
                        "`python -m torchlinops_gb300._build` (there is no CPU fallback)"
                    )
                L = ctypes.CDLL(path)
                for name, (args, res) in _SIGNATURES.items():
                    f = getattr(L, name)
                    f.argtypes = args
                    f.restype = res
                _lib = L
    return _lib


def exported_symbols():
    return list(_SIGNATURES)


def check(status: int, what: str) -> None:
    if status == TLGB_OK:
        return
    msg = lib().tlgb_last_error().decode(errors="replace")
    text = f"{what}: {msg}"
    if status in (TLGB_ERR_INVALID, TLGB_ERR_UNSUPPORTED):
        raise ValueError(text)
    raise RuntimeError(text)


def device_status(clear: bool = False) -> int:
    """The device status word (0 = no kernel gave up a bounded wait); synchronises."""
    v = ctypes.c_int32(0)
    check(lib().tlgb_device_status(ctypes.byref(v), 1 if clear else 0), "tlgb_device_status")
    return int(v.value)


def check_cuda(*tensors: torch.Tensor) -> torch.device:
    dev = None
    for t in tensors:
        if t is None:
            continue
        if not t.is_cuda:
            raise RuntimeError(
                "torchlinops_gb300 runs on CUDA tensors only (GB300 kernels, no CPU fallback); "
                f"got a tensor on {t.device}"
            )
        if dev is None:
            dev = t.device
        elif t.device != dev:
            raise ValueError(f"tensors on different devices: {dev} and {t.device}")
    return dev


def stream_ptr(device: torch.device) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def ptr(t: torch.Tensor | None) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr() if t is not None else 0)
