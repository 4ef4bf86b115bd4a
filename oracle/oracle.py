"""TEST INFRASTRUCTURE ONLY — ctypes wrapper of the C FP64 oracle (hoe_oracle.c).

Each function restates the reference's CPU Array path; see the header of
``hoe_oracle.c`` for the reference file:line each one follows.  Arrays use the
reference's (Julia column-major) conventions: ``bf`` is ``(nVox, R)``,
``kspha`` is ``(R, nSam)``, ``csm`` is ``(nVox, nCha)``, data is flattened with
samples fastest.  Inputs are numpy arrays; complex arrays are complex128.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"

_lib = None


def build_oracle() -> Path:
    """Compile liboracle.so with the committed Makefile (gcc, OpenMP)."""
    src = HERE / "hoe_oracle.c"
    if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        _lib = ctypes.CDLL(str(LIB_PATH))
        D = ctypes.POINTER(ctypes.c_double)
        I64 = ctypes.c_int64
        _lib.oracle_forward.argtypes = [I64, I64, I64, I64, D, D, D, D, D, D, I64, D]
        _lib.oracle_adjoint.argtypes = [I64, I64, I64, I64, D, D, D, D, D, D, I64, D]
        _lib.oracle_derivative.argtypes = [I64, I64, I64, I64, I64, D, D, D, D, D, D, D, D]
        _lib.oracle_backward.argtypes = [I64, I64, I64, I64, I64, D, D, D, D, D, D, D, D, D, D, D]
        _lib.oracle_grid.argtypes = [I64, I64, I64, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, D, D, D]
        _lib.oracle_basis.argtypes = [I64, D, D, D, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_int), D]
        _lib.oracle_basis.restype = ctypes.c_int
        _lib.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib.oracle_max_threads.restype = ctypes.c_int
    return _lib


def _p(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _c128(a):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def grid(nX, nY, nZ, dx, dy, dz):
    n = nX * nY * nZ
    x, y, z = (np.empty(n) for _ in range(3))
    lib().oracle_grid(nX, nY, nZ, dx, dy, dz, _p(x), _p(y), _p(z))
    return x, y, z


def basis(x, y, z, terms):
    x, y, z = _f64(x), _f64(y), _f64(z)
    terms = np.ascontiguousarray(terms, dtype=np.int32)
    out = np.empty((len(terms), len(x)))  # row l contiguous == column-major (nVox, nT)
    rc = lib().oracle_basis(len(x), _p(x), _p(y), _p(z), len(terms),
                            terms.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _p(out))
    if rc != 0:
        raise ValueError("Basis function undefined.")
    return out.T  # (nVox, nTerm) view with column-major layout


class Model:
    """Prepared model arrays in the reference layout (FP64)."""

    def __init__(self, bf, kspha, times, fieldmap, csm, nTerm=None):
        self.bf = np.asfortranarray(bf, dtype=np.float64)          # (nVox, R)
        self.kspha = np.asfortranarray(kspha, dtype=np.float64)    # (R, nSam)
        self.times = _f64(times)
        self.fieldmap = None if fieldmap is None else _f64(fieldmap)
        self.csm = None if csm is None else np.asfortranarray(csm, dtype=np.complex128)  # (nVox, nCha)
        self.nVox, self.R = self.bf.shape
        self.nSam = self.kspha.shape[1]
        self.nCha = 1 if csm is None else self.csm.shape[1]
        self.nTerm = self.R if nTerm is None else nTerm

    def _args(self):
        # both arrays are Fortran-contiguous: element (v,l) at v + l*nVox, (l,s) at l + s*R
        return (_p(self.bf), _p(self.kspha), _p(self.times), _p(self.fieldmap),
                None if self.csm is None else self.csm.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))


def forward(m: Model, xm, nBlock: int = 50):
    """y = E xm (xm: masked image, complex); returns complex128 [nSam*nCha]."""
    xm = _c128(xm)
    y = np.empty(m.nSam * m.nCha, dtype=np.complex128)
    bf, k, t, f, c = m._args()
    lib().oracle_forward(m.nVox, m.nSam, m.nCha, m.R, bf, k, t, f, c,
                         xm.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nBlock,
                         y.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return y


def adjoint(m: Model, y, nBlock: int = 50):
    """xm = E^H y on the masked voxels; returns complex128 [nVox]."""
    y = _c128(y)
    xm = np.empty(m.nVox, dtype=np.complex128)
    bf, k, t, f, c = m._args()
    lib().oracle_adjoint(m.nVox, m.nSam, m.nCha, m.R, bf, k, t, f, c,
                         y.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), nBlock,
                         xm.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return xm


def derivative(m: Model, kspha_dt, xm):
    xm = _c128(xm)
    kd = np.asfortranarray(kspha_dt, dtype=np.float64)
    y = np.empty(m.nSam * m.nCha, dtype=np.complex128)
    bf, k, t, f, c = m._args()
    lib().oracle_derivative(m.nVox, m.nSam, m.nCha, m.R, kd.shape[0], bf, k, _p(kd), t, f, c,
                            xm.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                            y.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return y


def backward(m: Model, xm, r, kspha_dt=None):
    """Returns (dk (R, nSam), ddf (nVox,), dt0_b0, dt0_coef)."""
    xm, r = _c128(xm), _c128(r)
    kd = None if kspha_dt is None else np.asfortranarray(kspha_dt, dtype=np.float64)
    # the coefficient part of dL/dt0 runs over the rows of kspha_dt (no concomitant rows)
    nT = m.nTerm if kd is None else kd.shape[0]
    if kd is not None and (kd.ndim != 2 or kd.shape[1] != m.nSam or nT > m.R):
        raise ValueError(f"kspha_dt must be (nTerm <= {m.R}, {m.nSam}), got {kd.shape}")
    dk = np.zeros((m.R, m.nSam), order="F")
    ddf = np.zeros(m.nVox)
    parts = np.zeros(2)
    bf, k, t, f, c = m._args()
    lib().oracle_backward(m.nVox, m.nSam, m.nCha, m.R, nT, bf, k, _p(kd), t, f, c,
                          xm.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                          r.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                          _p(dk), _p(ddf), _p(parts))
    return dk, ddf, parts[0], parts[1]


def scatter(xm, mask_flat):
    """Masked vector -> full grid with zeros outside the mask (array_operator.jl:345-346)."""
    out = np.zeros(mask_flat.size, dtype=np.complex128)
    out[mask_flat] = xm
    return out
