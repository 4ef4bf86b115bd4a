"""TEST INFRASTRUCTURE ONLY — independent FP64 dense-matrix oracle for tiny cases.

Restates the structure of the reference's independent oracle
(``test/test_explicit_gpu.jl:8-35``): hand-written basis polynomials and
scalar FP64 loops, ``cis(2*pi*phi)/sqrt(nVox)``, rows ordered samples fastest
then coils, zero columns outside the mask; and the concomitant dense encoding
of ``test/test_Concomitant.jl:26-50``.  It shares no code with the C oracle or
with the product's host-side preparation.
"""
from __future__ import annotations

import math

import numpy as np


def reference_basis(x: float, y: float, z: float):
    """The 16 unnormalised solid harmonics through third order, one point."""
    r2 = x * x + y * y + z * z
    return (1.0, x, y, z, x * y, z * y, 3 * z * z - r2, x * z, x * x - y * y,
            3 * y * x * x - y * y * y, x * y * z, (5 * z * z - r2) * y, 5 * z * z * z - 3 * z * r2,
            (5 * z * z - r2) * x, (x * x - y * y) * z, x * x * x - 3 * x * y * y)


def grid_coordinates(nX, nY, nZ, dx, dy, dz):
    """Centred coordinates, x index fastest (Grid.jl:78-82), as flat vectors."""
    i = np.arange(1, nX + 1)
    j = np.arange(1, nY + 1)
    k = np.arange(1, nZ + 1)
    K, J, I = np.meshgrid(k, j, i, indexing="ij")
    x = (I.ravel() - (nX + 1) / 2.0) * dx
    y = (J.ravel() - (nY + 1) / 2.0) * dy
    z = (K.ravel() - (nZ + 1) / 2.0) * dz
    return x, y, z


def reference_matrix(coords, kspha, times, fieldmap, csm, mask, concomitant=None):
    """Dense E (nSam*nCha x nFull), complex128.

    coords: (x, y, z) flat full-grid vectors (metres); kspha (nTerm, nSam) in
    cycles/m^p; times (nSam,) s; fieldmap (nFull,) Hz; csm (nFull, nCha);
    mask (nFull,) bool; concomitant (4, nSam) cycles/m^2 for [z^2, x^2+y^2, xz, yz].
    """
    x, y, z = (np.asarray(c, dtype=np.float64) for c in coords)
    kspha = np.asarray(kspha, dtype=np.float64)
    times = np.asarray(times, dtype=np.float64)
    fieldmap = np.asarray(fieldmap, dtype=np.float64)
    csm = np.asarray(csm, dtype=np.complex128)
    nTerm, ns = kspha.shape
    nc = csm.shape[1]
    idx = np.flatnonzero(mask)
    nvox = len(idx)
    A = np.zeros((ns * nc, len(mask)), dtype=np.complex128)
    for v in idx:
        b = reference_basis(float(x[v]), float(y[v]), float(z[v]))
        for s in range(ns):
            ph = float(times[s]) * float(fieldmap[v])
            for q in range(nTerm):
                ph += float(kspha[q, s]) * b[q]
            if concomitant is not None:
                ph += (concomitant[0, s] * z[v] ** 2 + concomitant[1, s] * (x[v] ** 2 + y[v] ** 2)
                       + concomitant[2, s] * x[v] * z[v] + concomitant[3, s] * y[v] * z[v])
            P = complex(math.cos(2 * math.pi * ph), math.sin(2 * math.pi * ph)) / math.sqrt(nvox)
            for c in range(nc):
                A[s + c * ns, v] = P * csm[v, c]
    return A


def rel(a, b) -> float:
    """Relative L2 error ||a-b|| / ||b|| (the reference's raw_complex_nrmse form)."""
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))
