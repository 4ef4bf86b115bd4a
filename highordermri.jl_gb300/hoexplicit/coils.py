"""SVD coil compression on the GPU (src/Recon/CoilCompression.jl) over
libhoexplicit.so: the Gram matrix and the application run on the device, the
coil-sized algebra (whitening, Hermitian eigen-decomposition) on the host in
FP64.  Names, keywords and errors follow the reference:
``estimate_noise_covariance``, ``noise_prewhitening_scale_factor``,
``fit_coil_compression``, ``apply_coil_compression``, ``compress_coils`` and
``CoilCompressionTransform``.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import ArgumentError, DimensionMismatch


def _torch():
    import torch
    return torch


@dataclass
class CoilCompressionTransform:
    """``compression_matrix`` (input coils, virtual coils) acting on the coil
    dimension from the right; ``singular_values`` of the (whitened)
    calibration matrix; ``retained_energy`` kept by the virtual coils."""

    compression_matrix: np.ndarray
    singular_values: np.ndarray
    retained_energy: float
    noise_covariance: np.ndarray | None = None
    prewhitening_scale_factor: float = 1.0

    @property
    def shape(self):
        return self.compression_matrix.shape

    def __repr__(self):
        method = "SVD" if self.noise_covariance is None else "noise-whitened SVD"
        extra = "" if self.prewhitening_scale_factor == 1 else f", prewhitening_scale_factor={self.prewhitening_scale_factor}"
        return (f">>> CoilCompressionTransform <<<\n{self.shape[0]} => {self.shape[1]}\nmethod          : {method}\n"
                f"retained_energy : {self.retained_energy}{extra}")


def _coil_last(array, coil_dim):
    """(observations, coils) matrix with the coil dimension last, as a
    column-major device buffer; returns (buffer, n, nCoil, coil-last shape, axes)."""
    torch = _torch()
    t = array if isinstance(array, torch.Tensor) else torch.from_numpy(np.asarray(array))
    nd = t.dim()
    d = coil_dim if coil_dim >= 0 else nd + coil_dim
    if not 0 <= d < nd:
        raise ArgumentError(f"coil_dim={coil_dim} must be a dimension of the array")
    axes = [a for a in range(nd) if a != d] + [d]
    tp = t.permute(*axes)
    shape = tuple(tp.shape)
    nCoil = shape[-1]
    n = int(np.prod(shape[:-1])) if len(shape) > 1 else 1
    # Julia's reshape(coil_last, :, nCoil) is column-major: flatten the leading
    # dimensions with the first one fastest
    lead = tp.permute(*range(len(shape) - 2, -1, -1), len(shape) - 1) if len(shape) > 1 else tp
    mat = lead.reshape(n, nCoil)
    return mat, n, nCoil, shape, axes


def _device_colmajor(mat, dtype):
    torch = _torch()
    return mat.to(device="cuda", dtype=dtype).t().contiguous().reshape(-1)


def estimate_noise_covariance(noise_data, *, coil_dim: int = -1, center: bool = True) -> np.ndarray:
    """Complex receive-noise covariance (CoilCompression.jl:127-148)."""
    torch = _torch()
    mat, n, nCoil, _, _ = _coil_last(noise_data, coil_dim)
    if not bool(torch.isfinite(torch.view_as_real(mat.to(torch.complex128))).all()):
        raise ArgumentError("noise_data must contain only finite values")
    minimum = 2 if center else 1
    if n < minimum:
        raise ArgumentError(f"noise_data must contain at least {minimum} observations")
    buf = _device_colmajor(mat, torch.complex128)
    G = np.zeros((nCoil, nCoil), dtype=np.complex128, order="F")
    _lib.check(_lib.load().hoe_coil_gram(buf.data_ptr(), 1, n, nCoil, int(bool(center)),
                                         G.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                         torch.cuda.current_stream().cuda_stream))
    C = G / (n - 1 if center else n)
    return (C + C.conj().T) / 2


def noise_prewhitening_scale_factor(acquisition_dwell_time: float, noise_dwell_time: float, *,
                                    receiver_bandwidth_ratio: float = 1.0) -> float:
    """s = (T_acq / T_noise) * R_BW (CoilCompression.jl:100-112)."""
    a, b, r = float(acquisition_dwell_time), float(noise_dwell_time), float(receiver_bandwidth_ratio)
    if not (np.isfinite(a) and a > 0):
        raise ArgumentError("acquisition_dwell_time must be finite and positive")
    if not (np.isfinite(b) and b > 0):
        raise ArgumentError("noise_dwell_time must be finite and positive")
    if not (np.isfinite(r) and r > 0):
        raise ArgumentError("receiver_bandwidth_ratio must be finite and positive")
    s = (a / b) * r
    if not (np.isfinite(s) and s > 0):
        raise ArgumentError("the resulting prewhitening scale factor must be finite and positive")
    return s


def fit_coil_compression(calibration_data, *, coil_dim: int = -1, n_virtual_coils: int | None = None,
                         energy_threshold: float | None = None, noise_covariance=None,
                         prewhitening_scale_factor: float = 1.0) -> CoilCompressionTransform:
    """Fit the SVD coil-compression transform (CoilCompression.jl:239-275)."""
    torch = _torch()
    if (n_virtual_coils is None) == (energy_threshold is None):
        raise ArgumentError("specify exactly one of n_virtual_coils and energy_threshold")
    mat, n, nCoil, _, _ = _coil_last(calibration_data, coil_dim)
    if not bool(torch.isfinite(torch.view_as_real(mat.to(torch.complex128))).all()):
        raise ArgumentError("calibration_data must contain only finite values")
    cov = None
    if noise_covariance is not None:
        cov = np.asarray(noise_covariance, dtype=np.complex128)
        if cov.shape != (nCoil, nCoil):
            raise DimensionMismatch(f"noise_covariance must have size ({nCoil}, {nCoil})")
        cov = np.asfortranarray(cov)
    buf = _device_colmajor(mat, torch.complex128)
    M = np.zeros((nCoil, nCoil), dtype=np.complex128, order="F")
    sv = np.zeros(min(n, nCoil))
    rank = ctypes.c_int32(0)
    kept = ctypes.c_double(0.0)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    _lib.check(_lib.load().hoe_coil_fit(
        buf.data_ptr(), 1, n, nCoil, int(n_virtual_coils) if n_virtual_coils is not None else 0,
        float(energy_threshold) if energy_threshold is not None else 0.0,
        None if cov is None else dp(cov), float(prewhitening_scale_factor), dp(M), dp(sv),
        ctypes.byref(rank), ctypes.byref(kept), torch.cuda.current_stream().cuda_stream))
    return CoilCompressionTransform(np.array(M[:, :rank.value]), sv, kept.value,
                                    None if cov is None else np.array(cov), float(prewhitening_scale_factor))


def apply_coil_compression(array, transform: CoilCompressionTransform, *, coil_dim: int = -1):
    """Apply along ``coil_dim`` (CoilCompression.jl:289-301); returns the same
    kind of array (numpy in, numpy out; torch in, CUDA torch out)."""
    torch = _torch()
    is_numpy = not isinstance(array, torch.Tensor)
    mat, n, nCoil, shape, axes = _coil_last(array, coil_dim)
    Mt = transform.compression_matrix
    if nCoil != Mt.shape[0]:
        raise DimensionMismatch(f"array has {nCoil} coils but transform expects {Mt.shape[0]}")
    nVirt = Mt.shape[1]
    a = _device_colmajor(mat, torch.complex64)
    M = torch.from_numpy(np.asfortranarray(Mt, dtype=np.complex64).reshape(-1, order="F")).cuda()
    out = torch.empty(n * nVirt, dtype=torch.complex64, device="cuda")
    _lib.check(_lib.load().hoe_coil_apply(a.data_ptr(), n, nCoil, M.data_ptr(), nVirt, out.data_ptr(),
                                          torch.cuda.current_stream().cuda_stream))
    # column-major (n, nVirt) -> coil-last array with the original leading shape
    lead = shape[:-1]
    res = out.reshape(nVirt, n).t()                              # (n, nVirt), row r = observation r
    res = res.reshape(*lead[::-1], nVirt) if lead else res.reshape(nVirt)
    res = res.permute(*range(len(lead) - 1, -1, -1), len(lead)) if lead else res
    inv = np.argsort(axes)
    res = res.permute(*inv)
    return res.cpu().numpy() if is_numpy else res


def compress_coils(data, csm, *, data_coil_dim: int = -1, csm_coil_dim: int = -1,
                   n_virtual_coils: int | None = None, energy_threshold: float | None = None,
                   noise_covariance=None, prewhitening_scale_factor: float = 1.0):
    """Fit on ``data`` and apply to both ``data`` and ``csm`` (CoilCompression.jl:303-353)."""
    t = fit_coil_compression(data, coil_dim=data_coil_dim, n_virtual_coils=n_virtual_coils,
                             energy_threshold=energy_threshold, noise_covariance=noise_covariance,
                             prewhitening_scale_factor=prewhitening_scale_factor)
    return (apply_coil_compression(data, t, coil_dim=data_coil_dim),
            apply_coil_compression(csm, t, coil_dim=csm_coil_dim), t)
