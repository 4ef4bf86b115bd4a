"""The oracle against the reference's known-answer tests and golden vectors.

Pins the C FP64 restatement (oracle/hoe_oracle.c) and the dense restatement
(oracle/dense.py) to each other and to every known answer the reference's
test suite holds for this path.
"""
import numpy as np
import pytest

from oracle import dense, oracle
from tests.golden_util import load, model_from_golden

TOL64 = 1e-12


def test_basis_known_answer_term17():
    # test/test_Concomitant.jl:92  basisfunc_spha([1,2],[3,4],[5,6],17) == [-24,-96]
    bf = oracle.basis([1.0, 2.0], [3.0, 4.0], [5.0, 6.0], [17])
    assert np.array_equal(bf[:, 0], [-24.0, -96.0])


def test_basis_terms_match_dense_restatement():
    rng = np.random.default_rng(3)
    x, y, z = rng.standard_normal((3, 50))
    bf = oracle.basis(x, y, z, list(range(1, 17)))
    ref = np.array([dense.reference_basis(a, b, c) for a, b, c in zip(x, y, z)])
    assert np.allclose(bf, ref, rtol=1e-14, atol=1e-14)


def test_grid_coordinates():
    # Grid.jl:78-82: (j - (N+1)/2) * delta, x fastest
    x, y, z = oracle.grid(4, 3, 2, 0.7, 0.9, 1.2)
    xd, yd, zd = dense.grid_coordinates(4, 3, 2, 0.7, 0.9, 1.2)
    assert np.array_equal(x, xd) and np.array_equal(y, yd) and np.array_equal(z, zd)
    assert np.isclose(x[0], -1.5 * 0.7) and np.isclose(x[1], -0.5 * 0.7)
    assert np.isclose(y[4], -0.9 * 0.0 - 0.0 + (2 - 2) * 0.9)


def test_zero_phase_known_answers():
    # test/test_explicit_gpu.jl:109-113 op*ones == fill(2,3);
    # test/test_explicit_multi_gpu.jl:72-77 unit-weight normal == fill(3,4)
    g = load("zero_phase")
    m, mask = model_from_golden(g)
    y = oracle.forward(m, g["image"][mask])
    assert np.allclose(y, 2.0, atol=1e-15)
    xn = oracle.adjoint(m, y)
    assert np.allclose(xn, 3.0, atol=1e-15)
    assert np.allclose(g["forward"], 2.0) and np.allclose(g["normal"], 3.0)


@pytest.mark.parametrize("nblock", [1, 4, 50])
def test_fixture_highorder_forward_adjoint(nblock):
    # test/test_HighOrderExplicit.jl:94-128 (dense vs blocked, adjoint identity, mask zeros)
    g = load("fixture_highorder")
    m, mask = model_from_golden(g)
    y = oracle.forward(m, g["image"][mask], nBlock=nblock)
    xa = oracle.scatter(oracle.adjoint(m, g["probe"], nBlock=nblock), mask)
    assert dense.rel(y, g["forward"]) < TOL64
    assert dense.rel(xa, g["adjoint"]) < TOL64
    assert np.all(xa[~mask] == 0)
    lhs = np.vdot(g["probe"], y)
    rhs = np.vdot(xa, g["image"])
    assert abs(lhs - rhs) / abs(lhs) < TOL64


@pytest.mark.parametrize("case", range(4))
def test_gpu_case_shapes(case):
    # test/test_explicit_gpu.jl:104-107 shapes, dense vs blocked restatement
    g = load(f"gpu_case_{case}")
    m, mask = model_from_golden(g)
    y = oracle.forward(m, g["image"][mask], nBlock=4)
    assert dense.rel(y, g["forward"]) < TOL64
    xa = oracle.scatter(oracle.adjoint(m, g["probe"], nBlock=7), mask)
    assert dense.rel(xa, g["adjoint"]) < TOL64
    D = np.tile(np.abs(g["weights"]) ** 2, m.nCha)
    xn = oracle.scatter(oracle.adjoint(m, D * oracle.forward(m, g["image"][mask])), mask)
    assert dense.rel(xn, g["normal"]) < TOL64
    rhs = oracle.scatter(oracle.adjoint(m, D * g["probe"]), mask)
    assert dense.rel(rhs, g["rhs"]) < TOL64


def test_concomitant_case():
    # test/test_Concomitant.jl:93-107 (F64 at 1e-11)
    g = load("concomitant")
    m, mask = model_from_golden(g)
    y = oracle.forward(m, g["image"][mask], nBlock=3)
    xa = oracle.scatter(oracle.adjoint(m, g["probe"], nBlock=3), mask)
    assert dense.rel(y, g["forward"]) < 1e-11
    assert dense.rel(xa, g["adjoint"]) < 1e-11


def test_derivative_is_dphase_of_forward():
    # array_operator.jl:216-218: B x = d(E x)/dtau for a coefficient time shift
    g = load("gpu_case_2")
    m, mask = model_from_golden(g)
    rng = np.random.default_rng(0)
    kd = rng.standard_normal(m.kspha.shape)
    h = 1e-6
    mp = oracle.Model(m.bf, m.kspha + h * kd, m.times, m.fieldmap, m.csm)
    mn = oracle.Model(m.bf, m.kspha - h * kd, m.times, m.fieldmap, m.csm)
    xm = g["image"][mask]
    fd = (oracle.forward(mp, xm) - oracle.forward(mn, xm)) / (2 * h)
    b = oracle.derivative(m, kd, xm)
    assert dense.rel(b, fd) < 1e-7


def test_backward_matches_finite_differences():
    g = load("gpu_case_0")
    m, mask = model_from_golden(g)
    xm = g["image"][mask]
    y = g["probe"]
    rng = np.random.default_rng(1)
    kd = rng.standard_normal(m.kspha.shape) * 10

    def loss(kspha, fieldmap, t0):
        mm = oracle.Model(m.bf, kspha - t0 * kd, m.times, fieldmap, m.csm)
        # fieldmap part of t0: phase fieldmap*(t - t0)
        mm.times = m.times - t0
        r = oracle.forward(mm, xm) - y
        return 0.5 * np.vdot(r, r).real

    r = oracle.forward(m, xm) - y
    dk, ddf, t0b, t0c = oracle.backward(m, xm, r, kd)
    h = 1e-6
    for (l, s) in [(0, 0), (3, 5), (8, 10)]:
        kp = m.kspha.copy(); kp[l, s] += h
        kn = m.kspha.copy(); kn[l, s] -= h
        fd = (loss(kp, m.fieldmap, 0) - loss(kn, m.fieldmap, 0)) / (2 * h)
        assert abs(fd - dk[l, s]) <= 1e-6 * max(1, abs(fd))
    for v in [0, 5, 11]:
        fp = m.fieldmap.copy(); fp[v] += 1e-3
        fn = m.fieldmap.copy(); fn[v] -= 1e-3
        fd = (loss(m.kspha, fp, 0) - loss(m.kspha, fn, 0)) / 2e-3
        assert abs(fd - ddf[v]) <= 1e-6 * max(1, abs(fd))
    ht = 1e-9
    fd = (loss(m.kspha, m.fieldmap, ht) - loss(m.kspha, m.fieldmap, -ht)) / (2 * ht)
    assert abs(fd - (t0b + t0c)) <= 1e-5 * max(1, abs(fd))
