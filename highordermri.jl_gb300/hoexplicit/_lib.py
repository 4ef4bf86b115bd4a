"""ctypes binding of libhoexplicit.so (declarations in include/hoexplicit.h).

The library is the only compute path: if it cannot be loaded, every operator
constructor raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent.parent
LIB_PATH = Path(os.environ.get("HOE_LIBRARY", PKG_DIR / "libhoexplicit.so"))

HOE_ABI_VERSION = 2
HOE_OK = 0
HOE_ERR_ARG = -1
HOE_ERR_DIM = -2
HOE_ERR_OOM = -3
HOE_ERR_CUDA = -4
HOE_ERR_TIMEOUT = -5
HOE_ERR_CLOSED = -6
HOE_ERR_UNSUPPORTED = -7

HOE_ENGINE_FP32_SIMT = 0
HOE_ENGINE_TC_BF16X3 = 1
HOE_ENGINE_AUTO = 2

HOE_GRAD_KSPHA = 1
HOE_GRAD_FIELDMAP = 2
HOE_GRAD_T0_B0 = 4
HOE_GRAD_T0_COEF = 8

EXPORTED = (
    "hoe_version", "hoe_abi_version", "hoe_create", "hoe_close", "hoe_free", "hoe_is_closed",
    "hoe_last_error", "hoe_get_info", "hoe_set_engine", "hoe_forward", "hoe_adjoint",
    "hoe_normal", "hoe_derivative", "hoe_backward", "hoe_set_timing", "hoe_get_timings",
    "hoe_forward_noalloc", "hoe_check", "hoe_plan", "hoe_recon",
    "hoe_batch_create", "hoe_batch_free", "hoe_batch_last_error", "hoe_batch_get_info",
    "hoe_batch_forward", "hoe_batch_adjoint", "hoe_batch_normal", "hoe_batch_recon", "hoe_batch_check",
    "hoe_set_kspha", "hoe_kdot_stencil", "hoe_interp_traj_time", "hoe_find_delay", "hoe_autotune",
    "hoe_coil_gram", "hoe_coil_fit", "hoe_coil_apply", "hoe_sfu_rate", "hoe_find_delay_multishot",
)

HOE_CG_ITERATION_LIMIT = 0
HOE_CG_CONVERGED = 1
HOE_CG_STOPPED = 2


class ArgumentError(ValueError):
    """Julia ``ArgumentError`` counterpart."""


class DimensionMismatch(ValueError):
    """Julia ``DimensionMismatch`` counterpart."""


class OutOfMemoryError(MemoryError):
    """Julia ``OutOfMemoryError`` counterpart (device allocation failed)."""


class HoeError(RuntimeError):
    """CUDA runtime failure or unsupported mode reported by the library."""


class HoeDesc(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int32),
        ("nX", ctypes.c_int32), ("nY", ctypes.c_int32), ("nZ", ctypes.c_int32),
        ("nSam", ctypes.c_int32), ("nCha", ctypes.c_int32), ("nTerm", ctypes.c_int32),
        ("has_concomitant", ctypes.c_int32), ("nVox", ctypes.c_int32),
        ("engine", ctypes.c_int32), ("device", ctypes.c_int32),
        ("tc_plan", ctypes.c_int32), ("reserved", ctypes.c_int32),
        ("split_hint", ctypes.c_int32),
        ("mask_idx", ctypes.POINTER(ctypes.c_int32)),
        ("bf", ctypes.POINTER(ctypes.c_double)),
        ("kspha", ctypes.POINTER(ctypes.c_double)),
        ("times", ctypes.POINTER(ctypes.c_double)),
        ("fieldmap", ctypes.POINTER(ctypes.c_double)),
        ("csm", ctypes.POINTER(ctypes.c_double)),
        ("kspha_dt", ctypes.POINTER(ctypes.c_double)),
    ]


class HoeRawModel(ctypes.Structure):
    _fields_ = [
        ("nVox", ctypes.c_int32), ("nSam", ctypes.c_int32), ("nCha", ctypes.c_int32),
        ("nTermEff", ctypes.c_int32),
        ("mask_idx", ctypes.c_void_p), ("bf", ctypes.c_void_p), ("kspha", ctypes.c_void_p),
        ("times", ctypes.c_void_p), ("fieldmap", ctypes.c_void_p), ("csm", ctypes.c_void_p),
    ]


class HoeTimings(ctypes.Structure):
    _fields_ = [
        ("forward_kernel_ms", ctypes.c_float), ("adjoint_kernel_ms", ctypes.c_float),
        ("forward_total_ms", ctypes.c_float), ("adjoint_total_ms", ctypes.c_float),
        ("launches", ctypes.c_int64),
    ]


class HoeCgParams(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int32), ("use_graph", ctypes.c_int32),
        ("rel_tol", ctypes.c_double), ("lambda_", ctypes.c_double),
    ]


class HoeCgStats(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int32), ("status", ctypes.c_int32),
        ("residual0", ctypes.c_double), ("residual", ctypes.c_double),
    ]


class HoeDelayParams(ctypes.Structure):
    _fields_ = [
        ("start_time", ctypes.c_double), ("dt", ctypes.c_double), ("dtau_min", ctypes.c_double),
        ("jump_fact", ctypes.c_double), ("lambda_", ctypes.c_double),
        ("term_mask", ctypes.POINTER(ctypes.c_double)),
        ("iter_max", ctypes.c_int32), ("max_outer", ctypes.c_int32),
    ]


class HoeDelayResult(ctypes.Structure):
    _fields_ = [
        ("tau", ctypes.c_double), ("tau_last", ctypes.c_double), ("dtau", ctypes.c_double),
        ("jump", ctypes.c_double), ("iterations", ctypes.c_int32), ("status", ctypes.c_int32),
    ]


class HoeTuneResult(ctypes.Structure):
    _fields_ = [
        ("engine", ctypes.c_int32), ("split_forward", ctypes.c_int32), ("split_adjoint", ctypes.c_int32),
        ("candidates", ctypes.c_int32), ("cand_engine", ctypes.c_int32 * 8), ("cand_split", ctypes.c_int32 * 8),
        ("cand_ms", ctypes.c_float * 8), ("tc_plan", ctypes.c_int32), ("cand_plan", ctypes.c_int32 * 8),
    ]


class HoeBatchInfo(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int32), ("contraction_launches", ctypes.c_int32), ("launches", ctypes.c_int64),
    ]


class HoeInfo(ctypes.Structure):
    _fields_ = [
        ("nSam", ctypes.c_int32), ("nCha", ctypes.c_int32), ("nVox", ctypes.c_int32),
        ("nTermEff", ctypes.c_int32), ("nFull", ctypes.c_int32), ("engine", ctypes.c_int32),
        ("tile_samples", ctypes.c_int32), ("tile_voxels", ctypes.c_int32),
        ("n_sample_tiles", ctypes.c_int32), ("n_voxel_tiles", ctypes.c_int32),
        ("split_forward", ctypes.c_int32), ("split_adjoint", ctypes.c_int32),
        ("residual_rank", ctypes.c_int32), ("residual_width", ctypes.c_int32),
        ("residual_phase_bound", ctypes.c_double), ("device_bytes", ctypes.c_int64),
        ("tc_plan", ctypes.c_int32), ("tc_plans", ctypes.c_int32),
    ]


_lib = None


def load():
    """Load libhoexplicit.so once; raise if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"libhoexplicit.so not found at {LIB_PATH}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(str(LIB_PATH))
    vp = ctypes.c_void_p
    H = ctypes.c_void_p
    lib.hoe_version.restype = ctypes.c_char_p
    lib.hoe_abi_version.restype = ctypes.c_int
    lib.hoe_create.argtypes = [ctypes.POINTER(H), ctypes.POINTER(HoeDesc)]
    lib.hoe_close.argtypes = [H]
    lib.hoe_free.argtypes = [H]
    lib.hoe_free.restype = None
    lib.hoe_is_closed.argtypes = [H]
    lib.hoe_last_error.argtypes = [H]
    lib.hoe_last_error.restype = ctypes.c_char_p
    lib.hoe_get_info.argtypes = [H, ctypes.POINTER(HoeInfo)]
    lib.hoe_set_engine.argtypes = [H, ctypes.c_int32]
    lib.hoe_forward.argtypes = [H, vp, vp, vp]
    lib.hoe_adjoint.argtypes = [H, vp, vp, vp]
    lib.hoe_normal.argtypes = [H, vp, vp, vp, vp]
    lib.hoe_derivative.argtypes = [H, vp, vp, vp]
    lib.hoe_backward.argtypes = [H, vp, vp, vp, vp, vp, ctypes.c_int32, vp]
    lib.hoe_set_timing.argtypes = [H, ctypes.c_int32]
    lib.hoe_get_timings.argtypes = [H, ctypes.POINTER(HoeTimings)]
    lib.hoe_check.argtypes = [H, vp]
    lib.hoe_plan.argtypes = [ctypes.POINTER(HoeDesc), ctypes.POINTER(HoeInfo)]
    lib.hoe_forward_noalloc.argtypes = [ctypes.POINTER(HoeRawModel), vp, vp, vp]
    lib.hoe_recon.argtypes = [H, vp, vp, vp, ctypes.POINTER(HoeCgParams), ctypes.POINTER(HoeCgStats), vp]
    PP = ctypes.POINTER(ctypes.c_void_p)
    lib.hoe_batch_create.argtypes = [ctypes.POINTER(H), PP, ctypes.c_int32]
    lib.hoe_batch_free.argtypes = [H]
    lib.hoe_batch_free.restype = None
    lib.hoe_batch_last_error.argtypes = [H]
    lib.hoe_batch_last_error.restype = ctypes.c_char_p
    lib.hoe_batch_get_info.argtypes = [H, ctypes.POINTER(HoeBatchInfo)]
    lib.hoe_batch_forward.argtypes = [H, PP, PP, vp]
    lib.hoe_batch_adjoint.argtypes = [H, PP, PP, vp]
    lib.hoe_batch_normal.argtypes = [H, PP, PP, PP, vp]
    lib.hoe_batch_recon.argtypes = [H, PP, PP, PP, ctypes.POINTER(HoeCgParams), ctypes.POINTER(HoeCgStats), vp]
    lib.hoe_batch_check.argtypes = [H, vp]
    I64 = ctypes.c_int64
    lib.hoe_set_kspha.argtypes = [H, vp, vp, vp]
    lib.hoe_autotune.argtypes = [H, ctypes.c_int32, ctypes.POINTER(HoeTuneResult), vp]
    DP = ctypes.POINTER(ctypes.c_double)
    lib.hoe_coil_gram.argtypes = [vp, ctypes.c_int32, I64, ctypes.c_int32, ctypes.c_int32, DP, vp]
    lib.hoe_coil_fit.argtypes = [vp, ctypes.c_int32, I64, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, DP,
                                 ctypes.c_double, DP, DP, ctypes.POINTER(ctypes.c_int32), DP, vp]
    lib.hoe_coil_apply.argtypes = [vp, I64, ctypes.c_int32, vp, ctypes.c_int32, vp, vp]
    lib.hoe_kdot_stencil.argtypes = [vp, I64, ctypes.c_int32, ctypes.c_double, vp, vp]
    lib.hoe_sfu_rate.argtypes = [DP, vp]
    lib.hoe_interp_traj_time.argtypes = [vp, I64, ctypes.c_int32, ctypes.c_double, ctypes.c_double, vp, I64, vp,
                                         ctypes.c_int32, vp]
    lib.hoe_find_delay.argtypes = [H, ctypes.POINTER(HoeDelayParams), vp, vp, vp, I64, vp,
                                   ctypes.POINTER(HoeDelayResult), vp]
    lib.hoe_find_delay_multishot.argtypes = [H, H, ctypes.POINTER(HoeDelayParams), ctypes.c_int32, DP, vp, vp,
                                             vp, I64, vp, ctypes.POINTER(HoeDelayResult), vp]
    for name in EXPORTED:
        if name not in ("hoe_free", "hoe_batch_free"):
            getattr(lib, name).restype = getattr(lib, name).restype or ctypes.c_int
    if lib.hoe_abi_version() != HOE_ABI_VERSION:
        raise ImportError("libhoexplicit.so ABI version mismatch")
    _lib = lib
    return lib


def check(rc: int, handle=None, batch=None) -> None:
    """Map a status code to the exception type the reference would raise."""
    if rc == HOE_OK:
        return
    if batch is not None:
        msg = load().hoe_batch_last_error(batch).decode(errors="replace")
    else:
        msg = load().hoe_last_error(handle).decode(errors="replace")
    if rc in (HOE_ERR_ARG, HOE_ERR_CLOSED, HOE_ERR_UNSUPPORTED):
        raise ArgumentError(msg)
    if rc == HOE_ERR_DIM:
        raise DimensionMismatch(msg)
    if rc == HOE_ERR_OOM:
        raise OutOfMemoryError(msg)
    raise HoeError(f"[{rc}] {msg}")
