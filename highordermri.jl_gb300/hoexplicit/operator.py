"""The GB300 explicit encoding operator: host-side mirror of the reference's
``HighOrderExplicitOp`` surface over the C ABI of libhoexplicit.so.

Reference surface mirrored (paths inside HighOrderMRI.jl):
  * constructor and validation — HighOrderExplicitOp.jl:44-51,
    explicit_gpu_operator.jl:299-392, array_operator.jl:83-181
  * ``op * x`` (prod!), ``adjoint(op) * y`` (ctprod!) — explicit_gpu_operator.jl:387-397
  * ``normalOperator(op, D)`` with its weight checks — explicit_gpu_operator.jl:399-416
  * ``explicit_gpu_normal(op; weights)`` — explicit_gpu_operator.jl:431-433
  * ``close(op)``: idempotent, use after close raises ArgumentError — :40-44, :435-446
  * ``kspha_dt`` derivative mode of the forward product — array_operator.jl:153-166

Solver vectors are torch CUDA complex64 tensors on the operator's device
(the counterpart of ``CuVector{ComplexF32}``, storage_type at
explicit_gpu_operator.jl:115).  numpy arrays are also accepted: they are
copied to the device and the result is copied back (host round trip).  The
in-place products ``prod_``/``ctprod_`` (the reference's ``mul!``) also take
host tensors: with page-locked memory they queue the copies and kernels on
the current stream and return without waiting.
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np

from . import _lib
from ._lib import ArgumentError, DimensionMismatch
from .model import Grid, basisfunc_spha, prep_concomitant, prep_kspha

ENGINES = {"fp32": _lib.HOE_ENGINE_FP32_SIMT, "simt": _lib.HOE_ENGINE_FP32_SIMT,
           "tc": _lib.HOE_ENGINE_TC_BF16X3, "bf16x3": _lib.HOE_ENGINE_TC_BF16X3,
           "auto": _lib.HOE_ENGINE_AUTO}
# the tensor-core engine on a GB300, the FP32 engine where it is unavailable
# (another device, more than 64 coils); ``op.engine`` reports the choice
DEFAULT_ENGINE = "auto"
_ENGINE_NAMES = {_lib.HOE_ENGINE_FP32_SIMT: "fp32", _lib.HOE_ENGINE_TC_BF16X3: "tc"}


def _torch():
    import torch  # device memory and streams only
    return torch


def _fortran_flat(a):
    return np.asarray(a).reshape(-1, order="F")


def _dptr(arr):
    return arr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if arr is not None else None


class _Vec:
    """Normalises a solver vector to a contiguous complex64 CUDA tensor."""

    def __init__(self, op, v, n, name):
        torch = _torch()
        self.host = None
        if isinstance(v, np.ndarray):
            self.host = "numpy"
            v = torch.from_numpy(np.ascontiguousarray(v.reshape(-1), dtype=np.complex64))
        if not isinstance(v, torch.Tensor):
            raise ArgumentError(f"{name} must be a torch tensor or numpy array")
        if v.numel() != n:
            raise DimensionMismatch(f"{name} has length {v.numel()}, expected {n}")
        self.pinned = False
        if v.device.type != "cuda":
            if self.host is None:
                self.host = "cpu"
                self.pinned = bool(v.is_pinned())
            # a page-locked source is copied on the current stream without a
            # host wait: the call's kernels follow on the same stream, and the
            # call waits for its result before returning
            v = v.to(device=op.torch_device, non_blocking=self.pinned)
        elif v.device.index != op.device:
            raise ArgumentError(f"{name} is on cuda:{v.device.index}, operator on cuda:{op.device}")
        if v.dtype != torch.complex64:
            v = v.to(torch.complex64)
        self.t = v.reshape(-1).contiguous()

    def out_like(self, result):
        if self.host == "numpy":
            return result.cpu().numpy()
        if self.host == "cpu":
            if self.pinned:  # page-locked in, page-locked out (direct DMA, no staging copy)
                out = _torch().empty(result.shape, dtype=result.dtype, pin_memory=True)
                out.copy_(result)
                return out
            return result.cpu()
        return result


# The tensor-core engine's execution plans (hoe_desc.tc_plan, hoe_autotune);
# plans 1-4 exist up to 16 coils.
TC_PLANS = {
    0: "default: 3 groups of 4 phase warps, deepest stage ring, flush every 32 stages",
    1: "2 groups of 4 phase warps",
    2: "4 groups of 4 phase warps",
    3: "stage ring of 4",
    4: "accumulator flush every 16 stages",
}


def build_desc(grid: Grid, kspha, times, *, fieldmap=None, csm=None, mask=None, concomitant=None,
               recon_terms=None, k_nominal=None, kspha_dt=None, kdot=None, engine=DEFAULT_ENGINE,
               device=0, split_hint=0, tc_plan=0):
    """Validate the constructor inputs (reference rules) and build the C
    descriptor.  Returns (desc, keep, meta); ``keep`` holds the host arrays the
    descriptor points to and must outlive every use of ``desc``."""
    if engine not in ENGINES:
        raise ArgumentError(f"unknown engine {engine!r}; choose one of {sorted(ENGINES)}")
    kspha = np.asarray(kspha)
    if kspha.ndim != 2:
        raise DimensionMismatch("kspha must be (nTerm, nSam)")
    nTerm, nSam = kspha.shape
    if nTerm not in (9, 16):
        raise ArgumentError("kspha requires 9 or 16 terms")
    times = np.asarray(times, dtype=np.float64).reshape(-1)
    if times.size != nSam:
        raise DimensionMismatch("times and kspha")
    nFull = grid.nX * grid.nY * grid.nZ
    mask = np.ones(nFull, dtype=bool) if mask is None else _fortran_flat(mask).astype(bool)
    if mask.size != nFull:
        raise DimensionMismatch("mask and grid")
    fieldmap = np.zeros(nFull) if fieldmap is None else _fortran_flat(fieldmap).astype(np.float64)
    if fieldmap.size != nFull:
        raise DimensionMismatch("fieldmap and mask")
    if csm is None:
        csm_flat = np.ones((nFull, 1), dtype=np.complex128)
    else:
        csm = np.asarray(csm)
        nCha_ = csm.shape[-1]
        if csm.size != nFull * nCha_:
            raise DimensionMismatch("csm and grid")
        csm_flat = csm.reshape(nFull, nCha_, order="F").astype(np.complex128)
    nCha = csm_flat.shape[1]
    idx = np.flatnonzero(mask)
    nVox = idx.size
    if nVox == 0:
        raise ArgumentError("mask must contain voxels")
    if nSam <= 0 or nCha <= 0:
        raise ArgumentError("samples and coils must be positive")
    if k_nominal is None:
        k_nominal = kspha[1:4, :]
    k_nominal = np.asarray(k_nominal, dtype=np.float64)
    if k_nominal.shape[0] != 3:
        raise ArgumentError("k_nominal must have 3 terms (row) for kx, ky, kz")

    prepared = prep_kspha(kspha, k_nominal, nTerm, recon_terms)
    xm, ym, zm = grid.x[idx], grid.y[idx], grid.z[idx]
    bf = basisfunc_spha(xm, ym, zm, list(range(1, nTerm + 1)))
    derivative_mode = kspha_dt is not None
    # the derivative mode ignores concomitant terms (array_operator.jl:139)
    bf, prepared = prep_concomitant(bf, prepared, xm, ym, zm,
                                    None if derivative_mode else concomitant)
    has_conc = int(prepared.shape[0] != nTerm)
    kd = kspha_dt if kspha_dt is not None else kdot
    if kd is not None:
        kd = np.asfortranarray(kd, dtype=np.float64)
        if kd.shape != (nTerm, nSam):
            raise ArgumentError("kspha_dt must have same size as kspha")

    keep = dict(
        mask_idx=np.ascontiguousarray(idx, dtype=np.int32),
        bf=np.asfortranarray(bf, dtype=np.float64),
        kspha=np.asfortranarray(prepared, dtype=np.float64),
        times=np.ascontiguousarray(times),
        fieldmap=np.ascontiguousarray(fieldmap[idx]),
        csm=np.asfortranarray(csm_flat[idx, :]),
        kspha_dt=kd,
    )
    k = keep
    desc = _lib.HoeDesc()
    desc.abi_version = _lib.HOE_ABI_VERSION
    desc.nX, desc.nY, desc.nZ = grid.nX, grid.nY, grid.nZ
    desc.nSam, desc.nCha, desc.nTerm = nSam, nCha, nTerm
    desc.has_concomitant = has_conc
    desc.nVox = nVox
    desc.engine = ENGINES[engine]
    desc.device = device
    desc.split_hint = int(split_hint)
    desc.tc_plan = int(tc_plan)
    desc.mask_idx = k["mask_idx"].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    desc.bf = _dptr(k["bf"])
    desc.kspha = _dptr(k["kspha"])
    desc.times = _dptr(k["times"])
    desc.fieldmap = _dptr(k["fieldmap"])
    desc.csm = k["csm"].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    desc.kspha_dt = _dptr(kd)
    meta = dict(nSam=nSam, nCha=nCha, nVox=nVox, nTerm=nTerm, nTermEff=prepared.shape[0], nFull=nFull,
                mask=mask, derivative_mode=derivative_mode)
    return desc, keep, meta


def plan(grid: Grid, kspha, times, **kwargs) -> dict:
    """Host-side plan of the operator (hoe_plan): tiles, residual rank and
    width, residual phase bound.  Needs no GPU."""
    desc, keep, meta = build_desc(grid, kspha, times, **kwargs)
    inf = _lib.HoeInfo()
    _lib.check(_lib.load().hoe_plan(ctypes.byref(desc), ctypes.byref(inf)))
    return {name: getattr(inf, name) for name, _ in inf._fields_}


def sfu_rate(stream=None) -> float:
    """sin/cos rate of the special-function unit of the current CUDA device
    (hoe_sfu_rate), in lane operations per clock per SM: the denominator of
    the phase generator's ceiling (2 operations per voxel-sample pair)."""
    torch = _torch()
    st = stream if stream is not None else torch.cuda.current_stream()
    out = ctypes.c_double(0.0)
    _lib.check(_lib.load().hoe_sfu_rate(ctypes.byref(out), ctypes.c_void_p(st.cuda_stream)))
    return float(out.value)


class ExplicitGB300Op:
    """Resident explicit encoding operator on one GB300 (the ``:gb300`` backend).

    Size ``(nSam*nCha, prod(grid.matrixSize))``, element type ComplexF32.
    Not reentrant: the operator owns scratch space on its device.
    """

    symmetric = False
    hermitian = False

    def __init__(self, grid: Grid, kspha, times, *, fieldmap=None, csm=None, mask=None,
                 concomitant=None, recon_terms=None, k_nominal=None, kspha_dt=None, kdot=None,
                 engine: str = DEFAULT_ENGINE, gpus=None, split_hint: int = 0, tc_plan: int = 0):
        lib = _lib.load()
        torch = _torch()
        if not torch.cuda.is_available():
            raise _lib.HoeError("the :gb300 explicit operator requires a CUDA device")
        if gpus is not None:
            ids = [int(g) for g in gpus]
            if len(ids) != 1:
                raise ArgumentError("the :gb300 operator uses exactly one GPU")
            if not 0 <= ids[0] < torch.cuda.device_count():
                raise ArgumentError("invalid visible GPU ID")
            device = ids[0]
        else:
            device = torch.cuda.current_device()

        desc, self._keep, meta = build_desc(
            grid, kspha, times, fieldmap=fieldmap, csm=csm, mask=mask, concomitant=concomitant,
            recon_terms=recon_terms, k_nominal=k_nominal, kspha_dt=kspha_dt, kdot=kdot,
            engine=engine, device=device, split_hint=split_hint, tc_plan=tc_plan)
        self.derivative_mode = meta["derivative_mode"]
        nSam, nCha, nVox, nTerm = meta["nSam"], meta["nCha"], meta["nVox"], meta["nTerm"]
        nFull, mask = meta["nFull"], meta["mask"]
        handle = ctypes.c_void_p()
        torch.cuda.init()
        _lib.check(lib.hoe_create(ctypes.byref(handle), ctypes.byref(desc)))
        self._h = handle
        self._finalizer = weakref.finalize(self, lib.hoe_free, handle)

        self.grid = grid
        self.device = device
        self.torch_device = torch.device("cuda", device)
        self.nSam, self.nCha, self.nVox, self.nTerm = nSam, nCha, nVox, nTerm
        self.nTermEff = meta["nTermEff"]
        self.nrow = nSam * nCha
        self.ncol = nFull
        self.shape = (self.nrow, self.ncol)
        self.mask = mask
        self.engine = _ENGINE_NAMES[self.info()["engine"]]
        self.nprod = self.ntprod = self.nctprod = 0
        self.tprod = None
        self._stage = {}   # device buffers for host operands of prod_/ctprod_, per (stream, role, length)

    # ------------------------------------------------------------------ misc
    def _handle(self):
        if self._h is None or _lib.load().hoe_is_closed(self._h):
            raise ArgumentError("operator is closed")
        return self._h

    def _stream(self):
        return _torch().cuda.current_stream(self.device).cuda_stream

    def info(self) -> dict:
        inf = _lib.HoeInfo()
        _lib.check(_lib.load().hoe_get_info(self._handle(), ctypes.byref(inf)), self._h)
        return {name: getattr(inf, name) for name, _ in inf._fields_}

    def set_timing(self, enable: bool = True) -> None:
        """Enable CUDA-event tracing of forward/adjoint calls (hoe_set_timing)."""
        _lib.check(_lib.load().hoe_set_timing(self._handle(), int(bool(enable))), self._h)

    def timings(self) -> dict:
        """Durations (ms) of the last traced calls and the launch count."""
        t = _lib.HoeTimings()
        _lib.check(_lib.load().hoe_get_timings(self._handle(), ctypes.byref(t)), self._h)
        return {name: getattr(t, name) for name, _ in t._fields_}

    def check(self) -> None:
        """Wait for the operator's stream and raise if a kernel reported a
        bounded-wait timeout (hoe_check)."""
        _lib.check(_lib.load().hoe_check(self._handle(), self._stream()), self._h)

    def autotune(self, reps: int = 5) -> dict:
        """Time forward+adjoint for each execution plan and keep the fastest
        (hoe_autotune): the FP32 engine at three split-K factors and the
        tensor-core engine's plans (five up to 16 coils: phase-warp groups,
        stage-ring depth, accumulator flush interval; TC_PLANS)."""
        r = _lib.HoeTuneResult()
        _lib.check(_lib.load().hoe_autotune(self._handle(), int(reps), ctypes.byref(r), self._stream()), self._h)
        names = _ENGINE_NAMES
        self.engine = names[r.engine]
        return {"engine": self.engine, "split_forward": r.split_forward, "split_adjoint": r.split_adjoint,
                "tc_plan": r.tc_plan,
                "candidates": [{"engine": names[r.cand_engine[i]], "split": r.cand_split[i],
                                "plan": r.cand_plan[i], "ms": r.cand_ms[i]}
                               for i in range(r.candidates)]}

    def set_engine(self, engine: str) -> None:
        if engine not in ENGINES:
            raise ArgumentError(f"unknown engine {engine!r}")
        _lib.check(_lib.load().hoe_set_engine(self._handle(), ENGINES[engine]), self._h)
        self.engine = _ENGINE_NAMES[self.info()["engine"]]

    def close(self) -> None:
        """Release device resources; idempotent (explicit_gpu_operator.jl:435-446)."""
        if self._h is not None:
            _lib.load().hoe_close(self._h)

    @property
    def closed(self) -> bool:
        return self._h is None or bool(_lib.load().hoe_is_closed(self._h))

    # ------------------------------------------------------------ products
    def _io(self, t, n, name, role, torch, stream):
        """Device view of an in-place product operand.  A CUDA tensor is used
        as is; a host tensor goes through a device buffer that the operator
        keeps per (stream, role, length), reused in stream order.  Returns
        (device tensor, host tensor to copy the result into or None, pinned)."""
        if not isinstance(t, torch.Tensor) or t.dtype != torch.complex64 or not t.is_contiguous():
            raise ArgumentError(f"{name} must be a contiguous complex64 torch tensor")
        if t.numel() != n:
            raise DimensionMismatch(f"{name} has length {t.numel()}, expected {n}")
        if t.is_cuda:
            if t.get_device() != self.device:
                raise ArgumentError(f"{name} is on cuda:{t.get_device()}, operator on cuda:{self.device}")
            return t, None, False
        key = (stream, role, n)
        buf = self._stage.get(key)
        if buf is None:
            buf = torch.empty(n, dtype=torch.complex64, device=self.torch_device)
            self._stage[key] = buf
        return buf, t, t.is_pinned()

    def _product(self, fn, out, v, nout, nin, counter):
        """Queue out = op(v) on the current stream.  Host operands are copied
        in and out around the kernels; with page-locked host memory nothing
        waits, so `out` holds the result once the stream has been synchronised
        (as with torch's non_blocking copies).  Other host memory is copied
        synchronously.  The library checks that the operator is open."""
        if self._h is None:
            raise ArgumentError("operator is closed")
        torch = _torch()
        st = torch.cuda.current_stream(self.device).cuda_stream
        dv, hv, pv = self._io(v, nin, "input", 0, torch, st)
        dout, hout, pout = self._io(out, nout, "out", 1, torch, st)
        if hv is not None:
            dv.copy_(hv, non_blocking=pv)
        rc = fn(self._h, dv.data_ptr(), dout.data_ptr(), st)
        if rc:
            _lib.check(rc, self._h)
        if hout is not None:
            hout.copy_(dout, non_blocking=pout)
        setattr(self, counter, getattr(self, counter) + 1)
        return out

    def prod_(self, out, x):
        """In-place forward: out = E x (or B x in the kspha_dt mode), the
        reference's mul!(out, op, x).  CUDA or host tensors (complex64,
        contiguous); queued on the current stream."""
        fn = _lib.load().hoe_derivative if self.derivative_mode else _lib.load().hoe_forward
        return self._product(fn, out, x, self.nrow, self.ncol, "nprod")

    def ctprod_(self, out, y):
        """In-place adjoint: out = E^H y (zeros outside the mask), the
        reference's mul!(out, adjoint(op), y).  CUDA or host tensors
        (complex64, contiguous); queued on the current stream."""
        return self._product(_lib.load().hoe_adjoint, out, y, self.ncol, self.nrow, "nctprod")

    def forward(self, x):
        v = _Vec(self, x, self.ncol, "x")
        self._handle()
        out = _torch().empty(self.nrow, dtype=_torch().complex64, device=self.torch_device)
        return v.out_like(self.prod_(out, v.t))

    def adjoint_apply(self, y):
        v = _Vec(self, y, self.nrow, "y")
        self._handle()
        out = _torch().empty(self.ncol, dtype=_torch().complex64, device=self.torch_device)
        return v.out_like(self.ctprod_(out, v.t))

    def __mul__(self, x):
        return self.forward(x)

    __matmul__ = __mul__

    @property
    def H(self):
        return AdjointOp(self)

    def backward(self, x, r, *, kspha=True, fieldmap=True, t0_b0=True, t0_coef=False):
        """Gradient of L = 0.5*||E x - y||^2 given the residual r = E x - y.

        Returns (dL/dkspha (nTermEff, nSam) float32 tensor, dL/dfieldmap
        (nFull,) float32 tensor zero outside the mask, dL/dt0 float64 tensor of
        one element); unrequested outputs are None.  ``t0_coef`` needs
        ``kspha_dt`` or ``kdot`` at construction.  The tensor-core engine forms
        the gradient on the tensor cores for up to 16 coils with residual widths
        up to 24 (``info()["residual_width"]``) and up to 32 coils with widths up
        to 16; otherwise the FP32 kernel does (up to 16 coils).
        """
        torch = _torch()
        xv = _Vec(self, x, self.ncol, "x")
        rv = _Vec(self, r, self.nrow, "r")
        flags = ((_lib.HOE_GRAD_KSPHA if kspha else 0) | (_lib.HOE_GRAD_FIELDMAP if fieldmap else 0)
                 | (_lib.HOE_GRAD_T0_B0 if t0_b0 else 0) | (_lib.HOE_GRAD_T0_COEF if t0_coef else 0))
        dk = torch.empty((self.nSam, self.nTermEff), dtype=torch.float32, device=self.torch_device) if kspha else None
        ddf = torch.empty(self.ncol, dtype=torch.float32, device=self.torch_device) if fieldmap else None
        dt0 = torch.zeros(1, dtype=torch.float64, device=self.torch_device) if (t0_b0 or t0_coef) else None
        p = lambda t: t.data_ptr() if t is not None else None
        _lib.check(_lib.load().hoe_backward(self._handle(), xv.t.data_ptr(), rv.t.data_ptr(),
                                            p(dk), p(ddf), p(dt0), flags, self._stream()), self._h)
        return (dk.t() if dk is not None else None), ddf, dt0


class AdjointOp:
    """``adjoint(op)``: prod and ctprod swapped (explicit_gpu_operator.jl:394-397)."""

    def __init__(self, op: ExplicitGB300Op):
        self.op = op
        self.nrow, self.ncol = op.ncol, op.nrow
        self.shape = (self.nrow, self.ncol)

    def __mul__(self, y):
        return self.op.adjoint_apply(y)

    __matmul__ = __mul__

    def prod_(self, out, y):
        return self.op.ctprod_(out, y)

    def ctprod_(self, out, x):
        return self.op.prod_(out, x)

    @property
    def H(self):
        return self.op


class WeightingOp:
    """Diagonal weighting W with raw complex sample weights repeated ``rep``
    times (LinearOperatorCollection WeightingOp as used by recon_HOOp.jl:77)."""

    def __init__(self, weights, rep: int = 1):
        self.weights = np.tile(np.asarray(weights).reshape(-1), rep)
        self.rep = rep


class WeightedOp:
    """``W ∘ op`` (recon_HOOp.jl:78)."""

    def __init__(self, W: WeightingOp, op: ExplicitGB300Op):
        if W.weights.size != op.nrow:
            raise DimensionMismatch("weights and operator rows")
        self.W, self.op = W, op
        self.nrow, self.ncol = op.nrow, op.ncol


def compose(W: WeightingOp, op: ExplicitGB300Op) -> WeightedOp:
    return WeightedOp(W, op)


class NormalOp:
    """``E^H D E`` sharing its parent's workspace and lifetime."""

    hermitian = True

    def __init__(self, op: ExplicitGB300Op, D: np.ndarray):
        torch = _torch()
        self.op = op
        self.nrow = self.ncol = op.ncol
        self.shape = (self.ncol, self.ncol)
        self.D = torch.from_numpy(np.ascontiguousarray(D, dtype=np.float32)).to(op.torch_device)

    def prod_(self, out, x):
        op = self.op
        _lib.check(_lib.load().hoe_normal(op._handle(), self.D.data_ptr(), x.data_ptr(),
                                          out.data_ptr(), op._stream()), op._h)
        return out

    def __mul__(self, x):
        v = _Vec(self.op, x, self.ncol, "x")
        self.op._handle()
        out = _torch().empty(self.ncol, dtype=_torch().complex64, device=self.op.torch_device)
        return v.out_like(self.prod_(out, v.t))

    __matmul__ = __mul__


def normal_diagonal(weights, nSam: int, nCha: int) -> np.ndarray:
    """Validate and expand normal weights to the real diagonal D (length
    nSam*nCha), with the rules of explicit_gpu_operator.jl:402-412."""
    if isinstance(weights, WeightingOp):
        weights = np.abs(weights.weights) ** 2
    if weights is None:
        D = np.ones(nSam * nCha)
    else:
        if hasattr(weights, "detach"):
            weights = weights.detach().cpu().numpy()
        D = np.asarray(weights).reshape(-1)
    if D.size == nSam:
        D = np.tile(D, nCha)
    if D.size != nSam * nCha:
        raise DimensionMismatch("normal weights")
    if not np.all(np.isfinite(D)):
        raise ArgumentError("normal weights must be finite")
    eps = float(np.finfo(np.float32).eps)
    if np.iscomplexobj(D):
        if np.max(np.abs(D.imag)) > 10 * eps * max(1.0, float(np.max(np.abs(D)))):
            raise ArgumentError("normal weights must already be real nonnegative WᴴW")
        D = D.real
    if np.min(D) < 0:
        raise ArgumentError("normal weights must be nonnegative")
    return D.astype(np.float64)


def normalOperator(op, weights=None):
    """Data normal ``A^H D A``; ``weights`` is the already squared real
    non-negative diagonal D (length nSam or nSam*nCha), a WeightingOp (whose
    raw weights are squared once), or None for unit weights.  A ``W ∘ op``
    argument supplies W^H W (explicit_gpu_operator.jl:399-416)."""
    if isinstance(op, WeightedOp):
        return normalOperator(op.op, np.abs(op.W.weights) ** 2)
    if not isinstance(op, ExplicitGB300Op):
        raise ArgumentError("normalOperator expects the :gb300 operator")
    op._handle()
    return NormalOp(op, normal_diagonal(weights, op.nSam, op.nCha))


def explicit_gpu_normal(op, weights=None):
    """``A^H D A`` with ``D = abs2.(weights)`` from raw sample weights
    (explicit_gpu_operator.jl:431-433)."""
    if weights is None:
        return normalOperator(op, None)
    if hasattr(weights, "detach"):
        weights = weights.detach().cpu().numpy()
    return normalOperator(op, np.abs(np.asarray(weights)) ** 2)


_KERNEL_OPTIONS = dict(backend="legacy", block_size=320, phase_backend="kernel", gemm_backend="cublas",
                       phase_cache_bytes=0, forward_threads=256, adjoint_threads=512)


def check_kernel_options(kspha_dt=None, **opts) -> None:
    """The reference's validation of its CUDA implementation's execution
    keywords (kernel_operator.jl:223-236, explicit_gpu_operator.jl:313-320),
    with the same ArgumentError messages.  They choose among that
    implementation's execution strategies (direct kernels, blocked phase
    tiles with a kernel- or GEMM-generated phase, a cached phase matrix),
    which the GB300 engine replaces: they are checked for drop-in use and do
    not change the arithmetic."""
    o = dict(_KERNEL_OPTIONS, **opts)
    sym = lambda v: str(v).lstrip(":")  # noqa: E731
    backend = sym(o["backend"])
    if backend != "legacy":
        if backend not in ("direct", "blocked", "cached", "cached_full"):
            raise ArgumentError(f"unknown explicit backend {backend}")
        if kspha_dt is not None:
            raise ArgumentError("kspha_dt requires backend=:legacy")
        if int(o["phase_cache_bytes"]) < 0:
            raise ArgumentError("phase_cache_bytes must be nonnegative")
        if int(o["phase_cache_bytes"]) != 0 and backend != "blocked":
            raise ArgumentError("phase_cache_bytes applies to backend=:blocked; cached backends already retain "
                                "the complete phase matrix")
        if sym(o["phase_backend"]) not in ("kernel", "gemm"):
            raise ArgumentError(f"unknown phase backend {sym(o['phase_backend'])}")
        if sym(o["gemm_backend"]) not in ("cublas", "auto"):
            raise ArgumentError("gemm_backend must be :cublas or :auto")
        if int(o["block_size"]) <= 0:
            raise ArgumentError("block_size must be positive")
        if int(o["forward_threads"]) not in (64, 128, 256, 512):
            raise ArgumentError("unsupported forward_threads")
        if int(o["adjoint_threads"]) not in (64, 128, 256, 512):
            raise ArgumentError("unsupported adjoint_threads")
    elif int(o["phase_cache_bytes"]) != 0:
        raise ArgumentError("phase_cache_bytes requires backend=:blocked")


def HighOrderExplicitOp(grid: Grid, kspha, times, *, implementation: str = "gb300", **kwargs):
    """Construct the explicit encoding operator (HighOrderExplicitOp.jl:44-51).

    This package provides the ``:gb300`` implementation only; the reference's
    ``:array`` and ``:kernel`` implementations are not part of it.  Their
    execution keywords are accepted so that a call written for either works
    unchanged: ``arrayType``, ``nBlock`` and ``verbose`` (the Array path) are
    ignored; ``backend``, ``block_size``, ``phase_backend``, ``gemm_backend``,
    ``phase_cache_bytes``, ``forward_threads`` and ``adjoint_threads`` (the
    CUDA path) get the reference's validation (check_kernel_options).
    """
    impl = str(implementation).lstrip(":")
    if impl != "gb300":
        raise ArgumentError("implementation must be :gb300 (this package has no :array or :kernel backend)")
    kwargs.pop("arrayType", None)
    kwargs.pop("nBlock", None)
    kwargs.pop("verbose", None)
    opts = {k: kwargs.pop(k) for k in list(kwargs) if k in _KERNEL_OPTIONS}
    check_kernel_options(kspha_dt=kwargs.get("kspha_dt"), **opts)
    return ExplicitGB300Op(grid, kspha, times, **kwargs)


def close(op) -> None:
    op.close()
