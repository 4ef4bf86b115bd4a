"""Delay synchronisation and trajectory preprocessing on the GPU
(src/Synchronization/FindDelay.jl, InterpTraj.jl) over libhoexplicit.so.

* ``kspha_dt(kspha, dt)`` — the k̇ stencil of FindDelay.jl:179-180.
* ``InterpTrajTime(traj, dt, delTime, datatime)`` — InterpTraj.jl:18-40,
  Akima interpolation per column, zero outside the shifted interval.
* ``FindDelay(...)`` — FindDelay.jl:139-214 with the whole outer iteration
  (interpolation at the current delay, sample-side operator re-plan, weighted
  CGNR image, y1 = data − E x, y2 = B x, Δτ = J·Re(y2 \\ y1)) captured as one
  CUDA graph.  Density weights are a fixed input (the reference recomputes
  them with NFFT at every τ); the outer loop is bounded by ``max_outer``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import ArgumentError, DimensionMismatch
from .model import Grid
from .recon import L2Regularization

STATUS = {0: "converged", 1: "max_outer", 2: "stopped"}


def _torch():
    import torch
    return torch


def _colmajor(a, name):
    """(rows, cols) array -> contiguous float64 CUDA buffer in column-major order."""
    torch = _torch()
    if isinstance(a, np.ndarray):
        if a.ndim != 2:
            raise DimensionMismatch(f"{name} must be a matrix")
        return torch.from_numpy(np.asfortranarray(a, dtype=np.float64).reshape(-1, order="F")).cuda(), a.shape, "numpy"
    if isinstance(a, torch.Tensor):
        if a.dim() != 2:
            raise DimensionMismatch(f"{name} must be a matrix")
        return a.to(device="cuda", dtype=torch.float64).t().contiguous().reshape(-1), tuple(a.shape), "torch"
    raise ArgumentError(f"{name} must be a numpy array or torch tensor")


def _vec64(a, name):
    torch = _torch()
    if isinstance(a, np.ndarray):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).reshape(-1)).cuda()
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda", dtype=torch.float64).reshape(-1).contiguous()
    raise ArgumentError(f"{name} must be a numpy array or torch tensor")


def _out(buf, rows, cols, kind):
    m = buf.reshape(cols, rows).t()  # column-major (rows, cols)
    return m.cpu().numpy() if kind == "numpy" else m


def kspha_dt(kspha, dt: float):
    """d kspha/dt of FindDelay.jl:179-180 for a (nFieldSample, nTerm) series."""
    torch = _torch()
    buf, (n, nT), kind = _colmajor(kspha, "kspha")
    out = torch.empty_like(buf)
    _lib.check(_lib.load().hoe_kdot_stencil(buf.data_ptr(), n, nT, float(dt), out.data_ptr(),
                                            torch.cuda.current_stream().cuda_stream))
    return _out(out, n, nT, kind)


def InterpTrajTime(traj, dt: float, delTime, datatime=None):
    """(nFieldSample, nTerm) -> (len(datatime), nTerm); datatime defaults to
    dt*(0:nFieldSample-1) (InterpTraj.jl:18-66).  A (nShot, nFieldSample,
    nTerm) series with one delTime per shot and datatime (nShot, nADCSample)
    gives (nShot, nADCSample, nTerm), each shot interpolated on its own
    (InterpTraj.jl:79-99)."""
    if getattr(traj, "ndim", 2) == 3:
        if datatime is None:
            raise ArgumentError("the per-shot overload needs datatime (nShot, nADCSample)")
        delTime = np.asarray(delTime, dtype=np.float64).reshape(-1)
        nShot = traj.shape[0]
        if nShot != delTime.size:
            raise DimensionMismatch("Number of shots in trajectory must match length of delTime vector")
        if getattr(datatime, "ndim", 0) != 2 or datatime.shape[0] != delTime.size:
            raise DimensionMismatch("Number of shots in datatime must match length of delTime vector")
        shots = [InterpTrajTime(traj[i], dt, float(delTime[i]), datatime[i]) for i in range(nShot)]
        torch = _torch()
        return torch.stack(shots) if isinstance(shots[0], torch.Tensor) else np.stack(shots)
    torch = _torch()
    buf, (n, nT), kind = _colmajor(traj, "traj")
    if datatime is None:
        datatime = float(dt) * np.arange(n)
    t = _vec64(datatime, "datatime")
    out = torch.empty(t.numel() * nT, dtype=torch.float64, device=t.device)
    _lib.check(_lib.load().hoe_interp_traj_time(buf.data_ptr(), n, nT, float(dt), float(delTime), t.data_ptr(),
                                                t.numel(), out.data_ptr(), 0,
                                                torch.cuda.current_stream().cuda_stream))
    return _out(out, t.numel(), nT, kind)


def term_mask(recon_terms: str, nTerm: int) -> np.ndarray:
    """Per-term factors of prep_kspha's order flags (prep_kspha.jl:1-56);
    first order cannot be switched off here (it needs k_nominal)."""
    expected = 3 if nTerm == 9 else (4 if nTerm == 16 else 0)
    if expected == 0:
        raise ArgumentError(f"kspha requires 9 or 16 terms, got {nTerm}")
    if len(recon_terms) != expected or any(c not in "01" for c in recon_terms):
        raise ArgumentError(f"recon_terms must contain {expected} binary digits for nTerm={nTerm}")
    if recon_terms[1] != "1":
        raise ArgumentError("FindDelay keeps first-order terms (recon_terms[2] must be '1')")
    order = [0, 1, 1, 1, 2, 2, 2, 2, 2] + [3] * 7
    return np.array([1.0 if recon_terms[order[l]] == "1" else 0.0 for l in range(nTerm)])


def FindDelay(gridding: Grid, data, kspha, datatime, StartTime: float, dt: float, *, JumpFact: float = 3,
              dtau_min: float = 5e-9, fieldmap=None, csm=None, recon_terms: str = "111", iter_max: int = 10,
              reg=None, weights=None, max_outer: int = 50, engine: str | None = None, return_info: bool = False):
    """Synchronisation delay τ (seconds) between ``data`` (nSample, nCha) and
    the coefficient series ``kspha`` (nFieldSample, nTerm); apply it as
    ``StartTime + τ`` in InterpTrajTime.  ``dtau_min`` is the reference's
    ``Δτ_min`` (same time unit as dt)."""
    from .operator import DEFAULT_ENGINE, HighOrderExplicitOp
    from .recon import _device_vector
    torch = _torch()
    if gridding.nZ != 1:
        raise ArgumentError("FindDelay needs a two-dimensional grid (nZ == 1)")
    data = np.asarray(data) if not isinstance(data, torch.Tensor) else data
    nSample, nCha = tuple(data.shape)
    datatime = np.asarray(datatime, dtype=np.float64).reshape(-1)
    if datatime.size != nSample:
        raise DimensionMismatch("data and datatime must have the same number of samples")
    kspha = np.asarray(kspha, dtype=np.float64)
    nField, nTerm = kspha.shape
    mask = term_mask(recon_terms, nTerm)
    if fieldmap is None:
        fieldmap = np.zeros((gridding.nX, gridding.nY))
    if csm is None:
        csm = np.ones((gridding.nX, gridding.nY, 1), dtype=np.complex128)
    if np.asarray(csm).shape[-1] != nCha:
        raise DimensionMismatch("data and csm must have the same number of coil channels")
    lam = 0.0 if reg is None else (reg.λ if isinstance(reg, L2Regularization) else float(reg))
    k0 = InterpTrajTime(kspha, dt, StartTime, datatime).T  # (nTerm, nSample) at τ = 0
    op = HighOrderExplicitOp(gridding, k0, datatime, fieldmap=np.asarray(fieldmap).reshape(gridding.nX, gridding.nY, 1),
                             csm=np.asarray(csm).reshape(gridding.nX, gridding.nY, 1, nCha),
                             recon_terms=recon_terms, engine=engine or DEFAULT_ENGINE)
    try:
        d = _device_vector(op, data, nSample, nCha, "data")
        w = None if weights is None else _device_vector(op, weights, nSample, 1, "weights")
        traj, _, _ = _colmajor(kspha, "kspha")
        x = torch.empty(op.ncol, dtype=torch.complex64, device=op.torch_device)
        mask_c = (ctypes.c_double * nTerm)(*mask)
        p = _lib.HoeDelayParams(float(StartTime), float(dt), float(dtau_min), float(JumpFact), float(lam),
                                ctypes.cast(mask_c, ctypes.POINTER(ctypes.c_double)), int(iter_max), int(max_outer))
        res = _lib.HoeDelayResult()
        _lib.check(_lib.load().hoe_find_delay(op._handle(), ctypes.byref(p), d.data_ptr(),
                                              None if w is None else w.data_ptr(), traj.data_ptr(), nField,
                                              x.data_ptr(), ctypes.byref(res), op._stream()), op._h)
        info = {"tau_last": res.tau_last, "dtau": res.dtau, "jump": res.jump, "iterations": res.iterations,
                "status": STATUS.get(res.status, res.status),
                "image": x.cpu().numpy().reshape(gridding.matrixSize, order="F")}
    finally:
        op.close()
    return (res.tau, info) if return_info else res.tau


def FindDelay_multishot(gridding: Grid, data, kspha, datatime, StartTime, dt: float, *, JumpFact: float = 3,
                        dtau_min: float = 5e-9, fieldmap=None, csm=None, recon_terms: str = "111",
                        iter_max: int = 10, reg=None, weights=None, max_outer: int = 50, engine: str | None = None,
                        return_info: bool = False):
    """One synchronisation delay τ (seconds) shared by all shots of a 2-D image
    (FindDelay_multishot.jl:65-158), on the device (hoe_find_delay_multishot).

    data (nShot*nSPI, nCha) with the samples of a shot consecutive; kspha
    (nShot, nField, nTerm); datatime (nShot, nSPI) ADC times, or None for
    dt*(0:nField-1) in every shot (the overload without datatime,
    FindDelay_multishot.jl:161-189); StartTime (nShot,).  As in the reference,
    the per-shot residual and derivative products use the first shot's ADC
    times (an operator on those times is built when the shots' times differ
    and the fieldmap is not zero).  Density weights are the fixed ``weights``."""
    from .operator import DEFAULT_ENGINE, HighOrderExplicitOp
    from .recon import _device_vector
    torch = _torch()
    if gridding.nZ != 1:
        raise ArgumentError("FindDelay_multishot needs a two-dimensional grid (nZ == 1)")
    data = np.asarray(data) if not isinstance(data, torch.Tensor) else data
    nSample, nCha = tuple(data.shape)
    kspha = np.asarray(kspha, dtype=np.float64)
    if kspha.ndim != 3:
        raise DimensionMismatch("kspha must be (nShot, nFieldSample, nTerm)")
    nShot, nField, nTerm = kspha.shape
    if datatime is None:
        datatime = np.tile(dt * np.arange(nField), (nShot, 1))
    datatime = np.asarray(datatime, dtype=np.float64)
    if datatime.ndim != 2 or datatime.shape[0] != nShot:
        raise DimensionMismatch("kspha and datatime must have the same number of shots")
    nSPI = datatime.shape[1]
    if nShot * nSPI != nSample:
        raise DimensionMismatch(f"data has {nSample} samples, expected nShot*nSPI = {nShot * nSPI}")
    start = np.asarray(StartTime, dtype=np.float64).reshape(-1)
    if start.size != nShot:
        raise DimensionMismatch("StartTime must have one entry per shot")
    mask = term_mask(recon_terms, nTerm)
    if fieldmap is None:
        fieldmap = np.zeros((gridding.nX, gridding.nY))
    if csm is None:
        csm = np.ones((gridding.nX, gridding.nY, 1), dtype=np.complex128)
    if np.asarray(csm).shape[-1] != nCha:
        raise DimensionMismatch("data and csm must have the same number of coil channels")
    lam = 0.0 if reg is None else (reg.λ if isinstance(reg, L2Regularization) else float(reg))
    k0 = np.concatenate([InterpTrajTime(kspha[s], dt, start[s], datatime[s]) for s in range(nShot)], axis=0).T
    kw = dict(fieldmap=np.asarray(fieldmap).reshape(gridding.nX, gridding.nY, 1),
              csm=np.asarray(csm).reshape(gridding.nX, gridding.nY, 1, nCha), recon_terms=recon_terms,
              engine=engine or DEFAULT_ENGINE)
    op = HighOrderExplicitOp(gridding, k0, datatime.reshape(-1), **kw)
    opr = None
    try:
        if np.any(np.asarray(fieldmap) != 0) and np.any(datatime != datatime[0]):
            opr = HighOrderExplicitOp(gridding, k0, np.tile(datatime[0], nShot), **kw)
        d = _device_vector(op, data, nSample, nCha, "data")
        w = None if weights is None else _device_vector(op, weights, nSample, 1, "weights")
        traj = torch.from_numpy(np.concatenate([kspha[s].reshape(-1, order="F") for s in range(nShot)])).to(
            op.torch_device)
        x = torch.empty(op.ncol, dtype=torch.complex64, device=op.torch_device)
        mask_c = (ctypes.c_double * nTerm)(*mask)
        start_c = (ctypes.c_double * nShot)(*start)
        p = _lib.HoeDelayParams(0.0, float(dt), float(dtau_min), float(JumpFact), float(lam),
                                ctypes.cast(mask_c, ctypes.POINTER(ctypes.c_double)), int(iter_max), int(max_outer))
        res = _lib.HoeDelayResult()
        _lib.check(_lib.load().hoe_find_delay_multishot(
            op._handle(), None if opr is None else opr._handle(), ctypes.byref(p), nShot,
            ctypes.cast(start_c, ctypes.POINTER(ctypes.c_double)), d.data_ptr(),
            None if w is None else w.data_ptr(), traj.data_ptr(), nField, x.data_ptr(), ctypes.byref(res),
            op._stream()), op._h)
        info = {"tau_last": res.tau_last, "dtau": res.dtau, "jump": res.jump, "iterations": res.iterations,
                "status": STATUS.get(res.status, res.status), "resid_operator": opr is not None,
                "image": x.cpu().numpy().reshape(gridding.matrixSize, order="F")}
    finally:
        op.close()
        if opr is not None:
            opr.close()
    return (res.tau, info) if return_info else res.tau


def set_kspha(op, kspha, kspha_dt=None) -> None:
    """Replace the operator's coefficients on the device (hoe_set_kspha):
    kspha (nTermEff, nSam) prepared as at construction, kspha_dt (nTerm, nSam)."""
    torch = _torch()
    k = _vec64(np.asarray(kspha, dtype=np.float64).reshape(-1, order="F")
               if isinstance(kspha, np.ndarray) else kspha.t().contiguous(), "kspha")
    if k.numel() != op.nTermEff * op.nSam:
        raise DimensionMismatch("kspha must be (nTermEff, nSam)")
    kd = None
    if kspha_dt is not None:
        kd = _vec64(np.asarray(kspha_dt, dtype=np.float64).reshape(-1, order="F")
                    if isinstance(kspha_dt, np.ndarray) else kspha_dt.t().contiguous(), "kspha_dt")
        if kd.numel() != op.nTerm * op.nSam:
            raise DimensionMismatch("kspha_dt must be (nTerm, nSam)")
    _lib.check(_lib.load().hoe_set_kspha(op._handle(), k.data_ptr(), None if kd is None else kd.data_ptr(),
                                         op._stream()), op._h)
    op._kspha_inputs = (k, kd)
    if kd is not None:
        op.derivative_capable = True
    del torch
