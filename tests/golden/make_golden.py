"""Generate the golden fixtures in tests/golden/ (committed .npz files).

The fixture problems restate the reference's own test problems:
  * ``fixture_highorder``: explicit_highorder_test_problem of
    test/test_HighOrderExplicit.jl:3-59 (4x3x2 grid, spacing (0.7,0.9,1.2) m,
    7 samples, 16 terms from range/sin/cos, fieldmap range(-25,20), 3
    analytic coils, voxels (1,1,1) and (end,end,end) masked out, image and
    probe from ranges).  Float32-rounded inputs, as in the reference test.
  * ``zero_phase``: the known-answer case of test/test_explicit_gpu.jl:109-113
    (2x2 grid, 9 zero terms, zero times: E*ones(4) == fill(2,3)) and the
    unit-weight normal of test/test_explicit_multi_gpu.jl:72-77 (== fill(3,4)).
  * ``gpu_case_*``: the shapes/terms/coils of test/test_explicit_gpu.jl:104-107
    with that file's input construction (ns=11, times range(0.001,0.009),
    fieldmap range(-37,49), spacing (0.07,0.08,0.09), masked voxels 1 and
    end-1, weights w + 0.7) drawn from numpy seeds (Julia's MersenneTwister
    streams are not reproducible here).
  * ``concomitant``: a concomitant-phase case in the style of
    test/test_Concomitant.jl:3-50.
Outputs are computed with the independent FP64 dense oracle (oracle/dense.py).

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import dense  # noqa: E402

OUT = Path(__file__).resolve().parent


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def jrange(a, b, n):
    return f32(np.linspace(a, b, n))


def fixture_highorder():
    nx, ny, nz = 4, 3, 2
    ns, nt, nc = 7, 16, 3
    dx, dy, dz = (float(np.float32(v)) for v in (0.7, 0.9, 1.2))
    x, y, z = dense.grid_coordinates(nx, ny, nz, dx, dy, dz)
    x, y, z = f32(x), f32(y), f32(z)
    times = jrange(0.0, 1.3e-3, ns)
    k = np.zeros((nt, ns))
    k[0] = jrange(-0.01, 0.015, ns)
    k[1] = jrange(-0.08, 0.07, ns)
    k[2] = jrange(0.06, -0.05, ns)
    k[3] = jrange(-0.03, 0.04, ns)
    for term in range(5, 10):
        k[term - 1] = f32(np.float32(4e-4 * (term - 4)) * np.sin(np.linspace(0, np.pi, ns, dtype=np.float32)))
    for term in range(10, 17):
        k[term - 1] = f32(np.float32(2e-5 * (term - 9)) * np.cos(np.linspace(0, np.pi, ns, dtype=np.float32)))
    fieldmap = jrange(-25, 20, nx * ny * nz)
    nxn, nyn, nzn = x / np.max(np.abs(x)), y / np.max(np.abs(y)), z / np.max(np.abs(z))
    csm = np.empty((nx * ny * nz, nc), dtype=np.complex128)
    for coil in range(1, nc + 1):
        ang = np.float32(2 * np.pi * (coil - 1) / nc)
        mag = 1 + np.float32(0.08) * (np.cos(ang) * nxn + np.sin(ang) * nyn)
        ph = np.float32(0.12 * coil) * (nyn - nzn)
        csm[:, coil - 1] = (mag * np.exp(1j * ph)).astype(np.complex64)
    mask = np.ones(nx * ny * nz, dtype=bool)
    mask[0] = False
    mask[-1] = False
    image = (jrange(0.1, 1.0, nx * ny * nz) + 1j * jrange(-0.2, 0.15, nx * ny * nz))
    probe = (jrange(-0.4, 0.5, ns * nc) + 1j * jrange(0.3, -0.2, ns * nc))
    A = dense.reference_matrix((x, y, z), k, times, fieldmap, csm, mask)
    return dict(shape=np.array([nx, ny, nz]), spacing=np.array([dx, dy, dz]), x=x, y=y, z=z,
                kspha=k, times=times, fieldmap=fieldmap, csm=csm, mask=mask, image=image,
                probe=probe, forward=A @ image, adjoint=A.conj().T @ probe)


def zero_phase():
    x, y, z = dense.grid_coordinates(2, 2, 1, 0.01, 0.01, 0.01)
    k = np.zeros((9, 3))
    times = np.zeros(3)
    csm = np.ones((4, 1), dtype=np.complex128)
    mask = np.ones(4, dtype=bool)
    A = dense.reference_matrix((x, y, z), k, times, np.zeros(4), csm, mask)
    ones = np.ones(4, dtype=np.complex128)
    return dict(shape=np.array([2, 2, 1]), spacing=np.array([0.01, 0.01, 0.01]), x=x, y=y, z=z,
                kspha=k, times=times, fieldmap=np.zeros(4), csm=csm, mask=mask, image=ones,
                forward=A @ ones, normal=A.conj().T @ (A @ ones))


def gpu_case(shape, nt, nc, seed):
    rng = np.random.default_rng(seed)
    nfull = int(np.prod(shape))
    x, y, z = dense.grid_coordinates(*shape, 0.07, 0.08, 0.09)
    ns = 11
    times = np.linspace(0.001, 0.009, ns)
    k = rng.standard_normal((nt, ns))
    fieldmap = np.linspace(-37, 49, nfull)
    csm = (rng.standard_normal((nfull, nc)) + 1j * rng.standard_normal((nfull, nc))) / np.sqrt(2)
    mask = np.ones(nfull, dtype=bool)
    mask[0] = False
    mask[nfull - 2] = False
    img = (rng.standard_normal(nfull) + 1j * rng.standard_normal(nfull)) / np.sqrt(2)
    data = (rng.standard_normal(ns * nc) + 1j * rng.standard_normal(ns * nc)) / np.sqrt(2)
    w = (rng.standard_normal(ns) + 1j * rng.standard_normal(ns)) / np.sqrt(2) + 0.7
    A = dense.reference_matrix((x, y, z), k, times, fieldmap, csm, mask)
    D = np.tile(np.abs(w) ** 2, nc)
    return dict(shape=np.array(shape), spacing=np.array([0.07, 0.08, 0.09]), x=x, y=y, z=z,
                kspha=k, times=times, fieldmap=fieldmap, csm=csm, mask=mask, image=img,
                probe=data, weights=w, forward=A @ img, adjoint=A.conj().T @ data,
                normal=A.conj().T @ (D * (A @ img)), rhs=A.conj().T @ (D * data))


def concomitant_case(seed=723):
    rng = np.random.default_rng(seed)
    shape = (6, 5, 3)
    nfull = int(np.prod(shape))
    x, y, z = dense.grid_coordinates(*shape, 0.008, 0.013, 0.011)
    ns, nt, nc = 9, 16, 2
    k = rng.standard_normal((nt, ns)) * 1e-5
    k[:4] *= 1000
    times = rng.random(ns) * 1e-3
    fieldmap = rng.standard_normal(nfull) * 5
    csm = rng.standard_normal((nfull, nc)) + 1j * rng.standard_normal((nfull, nc))
    conc = rng.standard_normal((4, ns)) * 1e-3 * 1e4
    mask = np.ones(nfull, dtype=bool)
    mask[0] = mask[-1] = False
    img = rng.standard_normal(nfull) + 1j * rng.standard_normal(nfull)
    data = rng.standard_normal(ns * nc) + 1j * rng.standard_normal(ns * nc)
    A = dense.reference_matrix((x, y, z), k, times, fieldmap, csm, mask, concomitant=conc)
    return dict(shape=np.array(shape), spacing=np.array([0.008, 0.013, 0.011]), x=x, y=y, z=z,
                kspha=k, times=times, fieldmap=fieldmap, csm=csm, mask=mask, concomitant=conc,
                image=img, probe=data, forward=A @ img, adjoint=A.conj().T @ data)


GPU_CASES = [((5, 4, 1), 9, 3), ((4, 3, 2), 16, 33), ((4, 5, 1), 16, 5), ((3, 4, 2), 9, 33)]


def main():
    np.savez_compressed(OUT / "fixture_highorder.npz", **fixture_highorder())
    np.savez_compressed(OUT / "zero_phase.npz", **zero_phase())
    for i, (shape, nt, nc) in enumerate(GPU_CASES):
        np.savez_compressed(OUT / f"gpu_case_{i}.npz", **gpu_case(shape, nt, nc, 1234 + nt + nc))
    np.savez_compressed(OUT / "concomitant.npz", **concomitant_case())
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
