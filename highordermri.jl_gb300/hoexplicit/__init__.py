"""hoexplicit — host-side interface of the GB300 explicit higher-order MRI
encoding operator (libhoexplicit.so).

Mirrors the operator surface of HighOrderMRI.jl's ``HighOrderExplicitOp``
(constructor, ``op * x``, ``adjoint(op) * y``, ``normalOperator``,
``explicit_gpu_normal``, ``close``, ``recon_HOOp``) on torch CUDA vectors.
"""
from ._lib import (ArgumentError, DimensionMismatch, HoeError, OutOfMemoryError,  # noqa: F401
                   LIB_PATH, load)
from .model import Grid, basisfunc_spha, prep_concomitant, prep_kspha  # noqa: F401
from .operator import (AdjointOp, ExplicitGB300Op, HighOrderExplicitOp, NormalOp,  # noqa: F401
                       WeightedOp, WeightingOp, close, compose, explicit_gpu_normal,
                       normalOperator)
from .recon import CGNR, L2Regularization, recon_HOOp  # noqa: F401
from .batch import OperatorBatch  # noqa: F401
from .sync import FindDelay, FindDelay_multishot, InterpTrajTime, kspha_dt, set_kspha  # noqa: F401
from .coils import (CoilCompressionTransform, apply_coil_compression, compress_coils,  # noqa: F401
                    estimate_noise_covariance, fit_coil_compression, noise_prewhitening_scale_factor)

__all__ = [
    "ArgumentError", "DimensionMismatch", "HoeError", "OutOfMemoryError", "Grid",
    "basisfunc_spha", "prep_kspha", "prep_concomitant", "HighOrderExplicitOp", "ExplicitGB300Op",
    "AdjointOp", "NormalOp", "WeightingOp", "WeightedOp", "compose", "normalOperator",
    "explicit_gpu_normal", "close", "load", "CGNR", "L2Regularization", "recon_HOOp",
    "OperatorBatch", "FindDelay", "FindDelay_multishot", "InterpTrajTime", "kspha_dt", "set_kspha",
    "CoilCompressionTransform", "apply_coil_compression", "compress_coils", "estimate_noise_covariance",
    "fit_coil_compression", "noise_prewhitening_scale_factor",
]
