"""``recon_HOOp`` for the GB300 explicit operator: the weighted CGNR solve of
src/Recon/recon_HOOp.jl:52-88 run on the device through ``hoe_recon``.

The reference weights data and operator with the raw sample weights repeated
over coils (``Data .* repeat(weight, nCha)``, ``W ∘ HOOp``, :75-77), forms the
normal ``EᴴE = HOOpᴴ WᴴW HOOp`` (:78) and hands both to RegularizedLeastSquares'
``CGNR`` with ``recParams`` merged over MRIReco's defaults (:73, :79-80).  Here
the whole solve, including its FP64 scalar recurrence, runs on the GPU as one
captured CUDA graph; the image comes back as a host array of ``reconSize``
(``Array(reshape(x, recParams[:reconSize]))``, :81).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import ArgumentError, DimensionMismatch

# RegularizedLeastSquares CGNR keyword defaults: iterations = 10,
# relTol = eps of the operator's real type.
DEFAULT_ITERATIONS = 10
DEFAULT_REL_TOL = float(np.finfo(np.float32).eps)

STATUS = {_lib.HOE_CG_ITERATION_LIMIT: "iterations", _lib.HOE_CG_CONVERGED: "converged",
          _lib.HOE_CG_STOPPED: "stopped"}


class CGNR:
    """Solver tag for ``recParams["solver"]`` (RegularizedLeastSquares.CGNR)."""


class L2Regularization:
    """``L2Regularization(λ)``: Tikhonov term λ‖x‖² (λ ≥ 0)."""

    def __init__(self, lam: float):
        lam = float(lam)
        if not np.isfinite(lam) or lam < 0:
            raise ArgumentError("L2Regularization weight must be finite and >= 0")
        self.λ = lam

    @property
    def lam(self) -> float:
        return self.λ


def _param(recParams: dict, name: str):
    for key in (name, ":" + name):
        if key in recParams:
            return recParams[key], True
    return None, False


def _required(recParams: dict, name: str):
    value, found = _param(recParams, name)
    if not found:
        raise KeyError(f"recParams must contain :{name}")
    return value


def _solver_ok(solver) -> bool:
    if solver is CGNR or isinstance(solver, CGNR):
        return True
    return isinstance(solver, str) and solver.lower() == "cgnr"


def _reg_lambda(reg) -> float:
    if isinstance(reg, (list, tuple)):
        if len(reg) != 1:
            raise ArgumentError("the :gb300 solver supports a single L2Regularization term")
        reg = reg[0]
    if isinstance(reg, L2Regularization):
        return reg.λ
    raise ArgumentError("the :gb300 solver supports L2Regularization only")


def _device_vector(op, v, rows: int, cols: int, name: str):
    """Column-major ``vec`` of a (rows, cols) array as a contiguous complex64
    CUDA tensor on the operator's device."""
    import torch
    if isinstance(v, np.ndarray):
        a = np.asarray(v)
        if a.ndim == 1 and cols == 1:
            a = a.reshape(-1, 1)
        if a.shape != (rows, cols):
            raise DimensionMismatch(f"{name} has shape {a.shape}, expected {(rows, cols)}")
        flat = np.ascontiguousarray(a.reshape(-1, order="F"), dtype=np.complex64)
        return torch.from_numpy(flat).to(op.torch_device)
    if isinstance(v, torch.Tensor):
        t = v.reshape(-1, 1) if (v.dim() == 1 and cols == 1) else v
        if tuple(t.shape) != (rows, cols):
            raise DimensionMismatch(f"{name} has shape {tuple(t.shape)}, expected {(rows, cols)}")
        if t.device.type == "cuda" and t.device.index != op.device:
            raise ArgumentError(f"{name} is on cuda:{t.device.index}, operator on cuda:{op.device}")
        return t.to(device=op.torch_device, dtype=torch.complex64).t().contiguous().reshape(-1)
    raise ArgumentError(f"{name} must be a numpy array or torch tensor")


def solve(op, data, weight=None, *, iterations: int = DEFAULT_ITERATIONS, rel_tol: float = DEFAULT_REL_TOL,
          lam: float = 0.0, use_graph: bool = True, out=None, stats: bool = True):
    """Device-level solve: returns (image tensor on the device, stats dict or None).

    ``data`` is (nSam, nCha), ``weight`` (nSam,) raw complex weights or None.
    """
    import torch
    h = op._handle()
    d = _device_vector(op, data, op.nSam, op.nCha, "Data")
    w = None if weight is None else _device_vector(op, weight, op.nSam, 1, "weight")
    if out is None:
        out = torch.empty(op.ncol, dtype=torch.complex64, device=op.torch_device)
    elif out.numel() != op.ncol or out.dtype != torch.complex64 or not out.is_contiguous():
        raise DimensionMismatch("out must be a contiguous complex64 vector of length prod(matrixSize)")
    p = _lib.HoeCgParams(int(iterations), int(bool(use_graph)), float(rel_tol), float(lam))
    st = _lib.HoeCgStats()
    _lib.check(_lib.load().hoe_recon(h, d.data_ptr(), None if w is None else w.data_ptr(), out.data_ptr(),
                                     ctypes.byref(p), ctypes.byref(st) if stats else None, op._stream()), h)
    # keep the inputs alive until the stream has consumed them
    op._recon_inputs = (d, w)
    if not stats:
        return out, None
    return out, {"iterations": st.iterations, "status": STATUS.get(st.status, st.status),
                 "residual0": st.residual0, "residual": st.residual}


def recon_HOOp(HOOp, Data, weight, recParams: dict, *, release_backend: bool = True,
               use_graph: bool = True, return_stats: bool = False):
    """Reconstruct an image with a :gb300 explicit operator (recon_HOOp.jl:52-88).

    ``recParams`` must contain ``solver`` (CGNR), ``reg``
    (``L2Regularization(λ)``) and ``reconSize``; ``iterations`` and ``relTol``
    default to the CGNR defaults.  Keys may be given as ``"solver"`` or
    ``":solver"``.  Returns a host complex64 array of shape ``reconSize``
    (column-major reshape, as Julia's ``reshape``).
    """
    from .operator import ExplicitGB300Op
    del release_backend  # the resident explicit operator owns no distributed backend
    if not isinstance(HOOp, ExplicitGB300Op):
        raise ArgumentError("recon_HOOp on the :gb300 backend needs an ExplicitGB300Op")
    solver = _required(recParams, "solver")
    reg = _required(recParams, "reg")
    recon_size = tuple(int(n) for n in _required(recParams, "reconSize"))
    if not _solver_ok(solver):
        raise ArgumentError("the :gb300 reconstruction runs CGNR only")
    lam = _reg_lambda(reg)
    iterations, found = _param(recParams, "iterations")
    iterations = DEFAULT_ITERATIONS if not found else int(iterations)
    rel_tol, found = _param(recParams, "relTol")
    rel_tol = DEFAULT_REL_TOL if not found else float(rel_tol)
    if int(np.prod(recon_size)) != HOOp.ncol:
        raise DimensionMismatch(f"reconSize {recon_size} does not match the operator's {HOOp.ncol} columns")
    x, stats = solve(HOOp, Data, weight, iterations=iterations, rel_tol=rel_tol, lam=lam,
                     use_graph=use_graph, stats=True)
    image = x.cpu().numpy().reshape(recon_size, order="F")
    return (image, stats) if return_stats else image
