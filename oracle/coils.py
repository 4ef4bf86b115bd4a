"""TEST INFRASTRUCTURE ONLY — FP64 numpy restatement of SVD coil compression
(src/Recon/CoilCompression.jl): covariance estimate (:127-148), whitening by
the inverse Cholesky factor scaled by sqrt(s) (:150-183), svd of the whitened
calibration matrix with rank by count or cumulative energy and compression
matrix W V[:, :rank] (:239-275), application along the coil axis (:289-301).
"""
from __future__ import annotations

import numpy as np


def coil_last(a, coil_dim=-1):
    a = np.asarray(a)
    d = coil_dim % a.ndim
    axes = [k for k in range(a.ndim) if k != d] + [d]
    t = np.transpose(a, axes)
    return t.reshape(-1, t.shape[-1], order="F"), t.shape, axes


def estimate_noise_covariance(noise, coil_dim=-1, center=True):
    m, _, _ = coil_last(noise, coil_dim)
    m = m.astype(np.complex128)
    if center:
        m = m - m.mean(axis=0, keepdims=True)
    c = m.conj().T @ m / (m.shape[0] - 1 if center else m.shape[0])
    return (c + c.conj().T) / 2


def fit(calibration, coil_dim=-1, n_virtual_coils=None, energy_threshold=None, noise_covariance=None, scale=1.0):
    """Returns (compression_matrix, singular_values, retained_energy)."""
    m, _, _ = coil_last(calibration, coil_dim)
    m = m.astype(np.complex128)
    n_coil = m.shape[1]
    if noise_covariance is None:
        W = np.eye(n_coil, dtype=np.complex128)
    else:
        psi = np.asarray(noise_covariance, dtype=np.complex128)
        psi = (psi + psi.conj().T) / 2
        U = np.linalg.cholesky(psi).conj().T   # psi = U^H U
        W = np.sqrt(scale) * np.linalg.inv(U)
    _, s, vh = np.linalg.svd(m @ W, full_matrices=False)
    energy = float(np.sum(s ** 2))
    if n_virtual_coils is not None:
        rank = int(n_virtual_coils)
    else:
        cum = np.cumsum(s ** 2)
        hit = np.flatnonzero(cum >= energy_threshold * energy)
        rank = int(hit[0]) + 1 if hit.size else s.size
    return W @ vh.conj().T[:, :rank], s, float(np.sum(s[:rank] ** 2) / energy)


def apply(array, matrix, coil_dim=-1):
    m, shape, axes = coil_last(array, coil_dim)
    out = (m @ matrix).reshape(shape[:-1] + (matrix.shape[1],), order="F")
    return np.transpose(out, np.argsort(axes))
