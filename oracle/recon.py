"""TEST INFRASTRUCTURE ONLY — FP64 restatement of the weighted CGNR solve of
recon_HOOp (src/Recon/recon_HOOp.jl:73-81) over the oracle's operator.

recon_HOOp weights the data and the operator with the raw sample weights
repeated over coils (:75-77) and runs RegularizedLeastSquares 0.16.12 ``CGNR``
(not vendored in the reference tree) with ``AHA = EᴴE`` and
``L2Regularization(λ)``.  The published conjugate-gradient recurrence on the
normal equations ``(EᴴE + λI) x = Eᴴ b`` from ``x = 0`` is restated here:

    z₀ = Eᴴb, p₀ = z₀;  q = (EᴴE+λI)p;  α = ‖z‖²/Re(pᴴq);  x += αp;  z −= αq;
    β = ‖z_new‖²/‖z‖²;  p = z + βp;  stop after ``iterations`` updates or once
    ‖z‖ ≤ rel_tol·‖z₀‖.

Vectors live on the masked voxels: outside the mask the adjoint is zero, so
the full-grid iterates are zero there and the two forms are the same solve.
"""
from __future__ import annotations

import numpy as np

from . import oracle as _o

ITERATION_LIMIT, CONVERGED, STOPPED = 0, 1, 2


def cgnr(normal, rhs, iterations: int, rel_tol: float = 0.0, lam: float = 0.0):
    """CG on (N + λI) x = rhs with N Hermitian PSD; returns (x, stats)."""
    x = np.zeros_like(rhs, dtype=np.complex128)
    z = np.array(rhs, dtype=np.complex128)
    p = z.copy()
    zz0 = zz = float(np.vdot(z, z).real)
    status = CONVERGED if zz == 0.0 else 0
    done = 0
    for _ in range(iterations):
        if status != 0:
            break
        q = normal(p) + lam * p
        pq = float(np.vdot(p, q).real)
        if not (pq > 0.0 and np.isfinite(pq)):
            status = STOPPED
            break
        alpha = zz / pq
        x += alpha * p
        z -= alpha * q
        zz_new = float(np.vdot(z, z).real)
        done += 1
        p = z + (zz_new / zz) * p
        zz = zz_new
        if zz <= rel_tol * rel_tol * zz0:
            status = CONVERGED
    return x, {"iterations": done, "status": status, "residual0": np.sqrt(zz0), "residual": np.sqrt(zz)}


def recon(m: "_o.Model", data, weights, iterations: int, rel_tol: float = 0.0, lam: float = 0.0,
          nBlock: int = 50):
    """Masked-voxel image of recon_HOOp's weighted CGNR in FP64.

    ``data``: complex (nSam*nCha,) samples fastest; ``weights``: complex
    (nSam,) raw sample weights or None (ones).
    """
    data = np.asarray(data, dtype=np.complex128).reshape(-1)
    if weights is None:
        d2 = np.ones(m.nSam * m.nCha)
    else:
        d2 = np.tile(np.abs(np.asarray(weights, dtype=np.complex128)) ** 2, m.nCha)
    rhs = _o.adjoint(m, d2 * data, nBlock)
    normal = lambda v: _o.adjoint(m, d2 * _o.forward(m, v, nBlock), nBlock)  # noqa: E731
    return cgnr(normal, rhs, iterations, rel_tol, lam)
