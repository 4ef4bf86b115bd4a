"""SVD coil compression (src/Recon/CoilCompression.jl) on the GPU.

Restates test/test_CoilCompression.jl ("rank and energy selection", "noise
covariance and prewhitening") with numpy seeds in place of Julia's, and
compares the device fit and application with the numpy oracle
(oracle/coils.py).  Singular vectors are defined up to a phase per column,
so compression matrices are compared through their projectors C C^H.
"""
import numpy as np
import pytest

from oracle import coils as oc


def test_oracle_restates_reference_rank_and_energy_case():
    cal = np.diag([4, 3, 1, 0.1]).astype(np.complex128)
    C, s, kept = oc.fit(cal, coil_dim=1, n_virtual_coils=2)
    assert C.shape == (4, 2)
    assert np.allclose(C.conj().T @ C, np.eye(2))
    assert np.isclose(kept, 25 / 26.01)
    assert np.allclose(s, [4, 3, 1, 0.1])
    _, _, kept_e = oc.fit(cal, energy_threshold=0.95)
    assert kept_e >= 0.95


torch = pytest.importorskip("torch")

from hoexplicit import (ArgumentError, DimensionMismatch, apply_coil_compression, compress_coils,  # noqa: E402
                        estimate_noise_covariance, fit_coil_compression, noise_prewhitening_scale_factor)


def test_scale_factor_host_side():
    assert np.isclose(noise_prewhitening_scale_factor(4e-6, 2e-6), 2.0)
    assert np.isclose(noise_prewhitening_scale_factor(4e-6, 2e-6, receiver_bandwidth_ratio=0.8), 1.6)
    for args, kw in [((0.0, 2e-6), {}), ((4e-6, -2e-6), {}), ((4e-6, 2e-6), {"receiver_bandwidth_ratio": np.inf})]:
        with pytest.raises(ArgumentError):
            noise_prewhitening_scale_factor(*args, **kw)


@pytest.mark.gpu
def test_rank_and_energy_selection():
    cal = np.diag([4, 3, 1, 0.1]).astype(np.complex128)
    t = fit_coil_compression(cal, coil_dim=1, n_virtual_coils=2)
    assert t.shape == (4, 2)
    assert np.allclose(t.compression_matrix.conj().T @ t.compression_matrix, np.eye(2))
    assert np.isclose(t.retained_energy, 25 / 26.01)
    assert np.allclose(t.singular_values, [4, 3, 1, 0.1], rtol=1.5e-8)
    assert "4 => 2" in repr(t)
    e = fit_coil_compression(cal, energy_threshold=0.95)
    assert e.shape == (4, 2) and e.retained_energy >= 0.95
    with pytest.raises(ArgumentError):
        fit_coil_compression(cal)
    with pytest.raises(ArgumentError):
        fit_coil_compression(cal, n_virtual_coils=2, energy_threshold=0.95)
    with pytest.raises(ArgumentError):
        fit_coil_compression(cal, n_virtual_coils=0)
    with pytest.raises(ArgumentError):
        fit_coil_compression(cal, energy_threshold=1.1)
    with pytest.raises(ArgumentError):
        fit_coil_compression(np.zeros((8, 4), dtype=np.complex128), n_virtual_coils=2)


@pytest.mark.gpu
def test_noise_covariance_and_prewhitening():
    rng = np.random.default_rng(20260805)
    noise = rng.standard_normal((101, 3)) + 1j * rng.standard_normal((101, 3))
    cov = estimate_noise_covariance(noise, coil_dim=1)
    centered = noise - noise.mean(axis=0, keepdims=True)
    assert np.allclose(cov, centered.conj().T @ centered / 100)
    assert np.allclose(cov, cov.conj().T)
    cal = rng.standard_normal((40, 3)) + 1j * rng.standard_normal((40, 3))
    psi = np.array([[4.0, 0.7 + 0.2j, 0.1 - 0.1j], [0.7 - 0.2j, 2.0, 0.3 + 0.05j], [0.1 + 0.1j, 0.3 - 0.05j, 1.0]])
    t = fit_coil_compression(cal, n_virtual_coils=2, noise_covariance=psi)
    C = t.compression_matrix
    assert np.allclose(C.conj().T @ psi @ C, np.eye(2))
    assert np.allclose(t.noise_covariance, psi)
    assert "noise-whitened SVD" in repr(t)
    Cr, sr, kr = oc.fit(cal, n_virtual_coils=2, noise_covariance=psi)
    assert np.allclose(t.singular_values, sr)
    assert np.allclose(C @ C.conj().T, Cr @ Cr.conj().T)
    s = noise_prewhitening_scale_factor(4e-6, 2e-6, receiver_bandwidth_ratio=0.8)
    tc = fit_coil_compression(cal, n_virtual_coils=2, noise_covariance=psi, prewhitening_scale_factor=s)
    assert np.allclose(tc.compression_matrix.conj().T @ (psi / s) @ tc.compression_matrix, np.eye(2))
    assert np.allclose(tc.compression_matrix.conj().T @ psi @ tc.compression_matrix, s * np.eye(2))
    assert np.isclose(tc.prewhitening_scale_factor, s) and "prewhitening_scale_factor" in repr(tc)
    assert np.allclose(tc.singular_values, oc.fit(cal, n_virtual_coils=2, noise_covariance=psi, scale=s)[1])
    assert np.isclose(tc.retained_energy, t.retained_energy)
    with pytest.raises(DimensionMismatch):
        fit_coil_compression(cal, n_virtual_coils=2, noise_covariance=np.eye(2))
    with pytest.raises(ArgumentError):
        fit_coil_compression(cal, n_virtual_coils=2, noise_covariance=np.array([[1, 1, 0], [0, 1, 0], [0, 0, 1]]))
    with pytest.raises(ArgumentError):
        fit_coil_compression(cal, n_virtual_coils=2, noise_covariance=np.zeros((3, 3)))
    with pytest.raises(ArgumentError):
        fit_coil_compression(cal, n_virtual_coils=2, prewhitening_scale_factor=2)
    with pytest.raises(ArgumentError):
        fit_coil_compression(cal, n_virtual_coils=2, noise_covariance=psi, prewhitening_scale_factor=0)
    with pytest.raises(ArgumentError):
        estimate_noise_covariance(np.zeros((1, 3), dtype=np.complex128))


@pytest.mark.gpu
def test_compress_data_and_maps_like_the_oracle():
    # 32 ring coils compressed to 16, as the 200x200 spiral workload does
    from hoexplicit import workloads
    rng = np.random.default_rng(7)
    w = workloads.small(seed=3, shape=(24, 20, 1), nSam=900, nCha=32)
    csm = np.asarray(w.csm)                                 # (24, 20, 1, 32)
    data = rng.standard_normal((900, 32)) @ (rng.standard_normal((32, 32)) * np.linspace(1, 0.01, 32)) \
        + 1j * rng.standard_normal((900, 32))
    d2, c2, t = compress_coils(data, csm, n_virtual_coils=16)
    Cr, sr, kr = oc.fit(data, n_virtual_coils=16)
    assert np.allclose(t.singular_values, sr, rtol=1e-10)
    assert np.isclose(t.retained_energy, kr)
    P = t.compression_matrix @ t.compression_matrix.conj().T
    assert np.allclose(P, Cr @ Cr.conj().T, atol=1e-9)
    assert d2.shape == (900, 16) and c2.shape == (24, 20, 1, 16)
    rel = lambda a, b: np.linalg.norm(a - b) / np.linalg.norm(b)  # noqa: E731
    assert rel(d2, oc.apply(data, t.compression_matrix)) < 1e-6          # complex64 application
    assert rel(c2, oc.apply(csm, t.compression_matrix)) < 1e-6
    # torch input on the device, coil axis first
    ct = torch.from_numpy(np.moveaxis(csm, -1, 0).astype(np.complex64)).cuda()
    c3 = apply_coil_compression(ct, t, coil_dim=0)
    assert c3.shape == (16, 24, 20, 1) and c3.is_cuda
    assert rel(np.moveaxis(c3.cpu().numpy(), 0, -1), oc.apply(csm, t.compression_matrix)) < 1e-6
    with pytest.raises(DimensionMismatch):
        apply_coil_compression(np.zeros((5, 7), dtype=np.complex64), t)
