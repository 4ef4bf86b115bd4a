"""Batches of :gb300 operators (the slices of a multi-slice scan) over
``hoe_batch_*``.

The reference builds one operator per slice and calls its products and
``recon_HOOp`` slice by slice (explicit_gpu_operator.jl:299-392,
recon_HOOp.jl:52-88).  ``OperatorBatch`` applies all slices together: with
the tensor-core engine each direction of every slice runs in one persistent
launch, and ``recon`` solves every slice's weighted CGNR in lockstep inside
one CUDA graph.
"""
from __future__ import annotations

import ctypes
import weakref

from . import _lib
from ._lib import ArgumentError, DimensionMismatch
from .recon import DEFAULT_ITERATIONS, DEFAULT_REL_TOL, STATUS, _device_vector


def _ptrs(ts):
    return (ctypes.c_void_p * len(ts))(*[None if t is None else t.data_ptr() for t in ts])


class OperatorBatch:
    """Members share one device; the batch borrows them (close it first)."""

    def __init__(self, ops):
        ops = list(ops)
        if not ops:
            raise ArgumentError("a batch needs at least one operator")
        lib = _lib.load()
        self.ops = ops
        hs = (ctypes.c_void_p * len(ops))(*[op._handle().value for op in ops])
        h = ctypes.c_void_p()
        _lib.check(lib.hoe_batch_create(ctypes.byref(h), hs, len(ops)))
        self._b = h
        self._finalizer = weakref.finalize(self, lib.hoe_batch_free, h)
        self.device = ops[0].device
        self.torch_device = ops[0].torch_device

    def _batch(self):
        if self._b is None:
            raise ArgumentError("batch is closed")
        return self._b

    def _stream(self):
        return self.ops[0]._stream()

    def _vecs(self, vs, lens, name):
        import torch
        if len(vs) != len(self.ops):
            raise DimensionMismatch(f"{name}: {len(vs)} vectors for {len(self.ops)} members")
        out = []
        for v, n, op in zip(vs, lens, self.ops):
            if not isinstance(v, torch.Tensor):
                v = torch.from_numpy(v)
            if v.numel() != n:
                raise DimensionMismatch(f"{name} has length {v.numel()}, expected {n}")
            out.append(v.to(device=op.torch_device, dtype=torch.complex64).reshape(-1).contiguous())
        return out

    def info(self) -> dict:
        inf = _lib.HoeBatchInfo()
        _lib.check(_lib.load().hoe_batch_get_info(self._batch(), ctypes.byref(inf)), batch=self._b)
        return {name: getattr(inf, name) for name, _ in inf._fields_}

    def forward(self, xs):
        import torch
        x = self._vecs(xs, [op.ncol for op in self.ops], "x")
        y = [torch.empty(op.nrow, dtype=torch.complex64, device=op.torch_device) for op in self.ops]
        _lib.check(_lib.load().hoe_batch_forward(self._batch(), _ptrs(x), _ptrs(y), self._stream()),
                   batch=self._b)
        return y

    def adjoint(self, ys):
        import torch
        y = self._vecs(ys, [op.nrow for op in self.ops], "y")
        x = [torch.empty(op.ncol, dtype=torch.complex64, device=op.torch_device) for op in self.ops]
        _lib.check(_lib.load().hoe_batch_adjoint(self._batch(), _ptrs(y), _ptrs(x), self._stream()),
                   batch=self._b)
        return x

    def normal(self, xs, D=None):
        """out_i = E_iᴴ diag(D_i) E_i x_i; D: None or per-member float32 device
        tensors of length nSam*nCha (None entries: ones)."""
        import torch
        x = self._vecs(xs, [op.ncol for op in self.ops], "x")
        out = [torch.empty(op.ncol, dtype=torch.complex64, device=op.torch_device) for op in self.ops]
        d = None if D is None else _ptrs(list(D))
        _lib.check(_lib.load().hoe_batch_normal(self._batch(), d, _ptrs(x), _ptrs(out), self._stream()),
                   batch=self._b)
        return out

    def recon(self, datas, weights=None, *, iterations: int = DEFAULT_ITERATIONS,
              rel_tol: float = DEFAULT_REL_TOL, lam: float = 0.0, use_graph: bool = True, out=None,
              stats: bool = True):
        """recon_HOOp's weighted CGNR for every member (data i: (nSam_i, nCha))."""
        import torch
        d = [_device_vector(op, v, op.nSam, op.nCha, "Data") for op, v in zip(self.ops, datas)]
        if weights is None:
            w = [None] * len(self.ops)
        else:
            w = [None if v is None else _device_vector(op, v, op.nSam, 1, "weight")
                 for op, v in zip(self.ops, weights)]
        if out is None:
            out = [torch.empty(op.ncol, dtype=torch.complex64, device=op.torch_device) for op in self.ops]
        p = _lib.HoeCgParams(int(iterations), int(bool(use_graph)), float(rel_tol), float(lam))
        st = (_lib.HoeCgStats * len(self.ops))()
        _lib.check(_lib.load().hoe_batch_recon(self._batch(), _ptrs(d), _ptrs(w), _ptrs(out), ctypes.byref(p),
                                               st if stats else None, self._stream()), batch=self._b)
        self._inputs = (d, w)
        if not stats:
            return out, None
        return out, [{"iterations": s.iterations, "status": STATUS.get(s.status, s.status),
                      "residual0": s.residual0, "residual": s.residual} for s in st]

    def check(self) -> None:
        _lib.check(_lib.load().hoe_batch_check(self._batch(), self._stream()), batch=self._b)

    def close(self) -> None:
        if self._b is not None:
            self._finalizer()
            self._b = None
