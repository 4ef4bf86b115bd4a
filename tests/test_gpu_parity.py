"""GPU parity of libhoexplicit.so against the FP64 oracle (through the C ABI).

Mirrors the reference's explicit-operator tests (test/test_HighOrderExplicit.jl,
test/test_explicit_gpu.jl, test/test_explicit_interface.jl,
test/test_Concomitant.jl) on the committed golden fixtures and on seeded
problems at sizes that are not multiples of the tiles.

Tolerances (relative L2 vs FP64): 1e-5 for the plain FP32 engine, 1e-4 for
the tensor-core engine.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from hoexplicit import (ArgumentError, DimensionMismatch, Grid, HighOrderExplicitOp,  # noqa: E402
                        OutOfMemoryError, WeightingOp, compose, explicit_gpu_normal, normalOperator,
                        workloads)
from oracle import dense, oracle  # noqa: E402
from tests.golden_util import load, model_from_golden  # noqa: E402

TOL = {"fp32": 1e-5, "tc": 1e-4}


def have_tc():
    g = load("zero_phase")
    try:
        op = op_from_golden(g, "tc")
        op.close()
        return True
    except Exception:
        return False


ENGINE_PARAMS = [pytest.param("fp32", id="fp32"), pytest.param("tc", id="tc")]


def maybe_skip(engine):
    if engine == "tc" and not have_tc():
        pytest.skip("tensor-core engine not available in this build")


def op_from_golden(g, engine, **kw):
    nx, ny, nz = (int(v) for v in g["shape"])
    dx, dy, dz = (float(v) for v in g["spacing"])
    grid = Grid(nx, ny, nz, dx, dy, dz, x=g["x"], y=g["y"], z=g["z"])
    sh = (nx, ny, nz)
    nc = g["csm"].shape[1]
    extra = {}
    if "concomitant" in g:
        extra["concomitant"] = g["concomitant"]
    return HighOrderExplicitOp(grid, g["kspha"], g["times"],
                               fieldmap=g["fieldmap"].reshape(sh, order="F"),
                               csm=g["csm"].reshape(sh + (nc,), order="F"),
                               mask=g["mask"].reshape(sh, order="F"), engine=engine, **extra, **kw)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex64)).cuda()


def host(t):
    return t.cpu().numpy().astype(np.complex128)


@pytest.mark.parametrize("engine", ENGINE_PARAMS)
def test_zero_phase_known_answer(engine):
    maybe_skip(engine)
    # test/test_explicit_gpu.jl:109-113 and test/test_explicit_multi_gpu.jl:72-77
    g = load("zero_phase")
    op = op_from_golden(g, engine)
    y = host(op * dev(np.ones(4)))
    assert np.allclose(y, 2.0, rtol=1e-6, atol=1e-6)
    n = host(normalOperator(op) * dev(np.ones(4)))
    assert np.allclose(n, 3.0, rtol=1e-6, atol=1e-6)
    op.close()


@pytest.mark.parametrize("engine", ENGINE_PARAMS)
def test_fixture_highorder(engine):
    maybe_skip(engine)
    # test/test_HighOrderExplicit.jl:94-128
    g = load("fixture_highorder")
    op = op_from_golden(g, engine)
    tol = TOL[engine]
    y = host(op * dev(g["image"]))
    xa = host(op.H * dev(g["probe"]))
    assert dense.rel(y, g["forward"]) < tol
    assert dense.rel(xa, g["adjoint"]) < tol
    assert np.all(xa[~g["mask"]] == 0)
    lhs, rhs = np.vdot(g["probe"], y), np.vdot(xa, g["image"])
    assert abs(lhs - rhs) / (np.linalg.norm(y) * np.linalg.norm(g["probe"])) < tol
    op.close()


@pytest.mark.parametrize("engine", ENGINE_PARAMS)
@pytest.mark.parametrize("case", range(4))
def test_reference_gpu_cases(engine, case):
    maybe_skip(engine)
    # test/test_explicit_gpu.jl:37-96 (forward, adjoint, weighted normal, RHS,
    # adjoint identity, mask zeros, linearity, zero input, non-negativity,
    # repeatability, invalid weights, close semantics)
    g = load(f"gpu_case_{case}")
    tol = TOL[engine]
    op = op_from_golden(g, engine)
    x, y, w = dev(g["image"]), dev(g["probe"]), g["weights"]
    nc = g["csm"].shape[1]
    fwd, bwd = host(op * x), host(op.H * y)
    assert dense.rel(fwd, g["forward"]) < tol
    assert dense.rel(bwd, g["adjoint"]) < tol
    assert abs(np.vdot(g["probe"], fwd) - np.vdot(bwd, g["image"])) / max(
        np.linalg.norm(fwd) * np.linalg.norm(g["probe"]), 1) < tol
    assert np.all(bwd[~g["mask"]] == 0)
    W = WeightingOp(w, nc)
    normal = normalOperator(compose(W, op))
    res = host(normal * x)
    assert dense.rel(res, g["normal"]) < tol
    assert dense.rel(host(explicit_gpu_normal(op, w) * x), g["normal"]) < tol
    D = np.tile(np.abs(w) ** 2, nc)
    assert dense.rel(host(normalOperator(op, D) * x), g["normal"]) < tol
    rhs = host(op.H * dev(np.tile(np.abs(w) ** 2, nc) * g["probe"]))
    assert dense.rel(rhs, g["rhs"]) < tol
    assert np.real(np.vdot(g["image"], res)) >= 0
    assert dense.rel(host(normal * (2 * x)), 2 * res) < 2 * tol
    assert np.linalg.norm(host(normal * torch.zeros_like(x))) == 0
    assert np.array_equal(host(normal * x), res)  # deterministic reductions
    with pytest.raises(ArgumentError):
        normalOperator(op, np.full(len(w), 1 + 1j))
    with pytest.raises(ArgumentError):
        normalOperator(op, np.full(len(w), -1.0))
    op.close()
    op.close()
    with pytest.raises(ArgumentError):
        normalOperator(op)
    with pytest.raises(ArgumentError):
        normal * x
    with pytest.raises(ArgumentError):
        op * x


@pytest.mark.parametrize("engine", ENGINE_PARAMS)
def test_concomitant_fixture(engine):
    maybe_skip(engine)
    # test/test_Concomitant.jl:93-107
    g = load("concomitant")
    op = op_from_golden(g, engine)
    tol = TOL[engine]
    assert dense.rel(host(op * dev(g["image"])), g["forward"]) < tol
    assert dense.rel(host(op.H * dev(g["probe"])), g["adjoint"]) < tol


def test_recon_terms_nominal_substitution():
    # test/test_explicit_interface.jl:24-30: "0011" with k_nominal equals the
    # operator built from the effective coefficients
    g = load("gpu_case_1")
    rng = np.random.default_rng(731)
    kn = rng.standard_normal((3, g["kspha"].shape[1]))
    eff = dict(g)
    eff["kspha"] = g["kspha"].copy()
    eff["kspha"][0] = 0
    eff["kspha"][1:4] = kn
    a = op_from_golden(g, "fp32", recon_terms="0011", k_nominal=kn)
    b = op_from_golden(eff, "fp32")
    x = dev(g["image"])
    assert np.array_equal(host(a * x), host(b * x))


SMALL = [
    dict(shape=(9, 7, 1), nSam=300, nCha=3, nTerm=16),
    dict(shape=(5, 6, 4), nSam=129, nCha=5, nTerm=9),
    dict(shape=(13, 11, 1), nSam=257, nCha=16, nTerm=16, conc=True),
    dict(shape=(17, 9, 2), nSam=200, nCha=1, nTerm=9),
    dict(shape=(12, 12, 1), nSam=131, nCha=33, nTerm=16),
    dict(shape=(14, 13, 1), nSam=333, nCha=24, nTerm=16, conc=True),
    # residual ranks 6 / 3 / 16 / 17: TF32 residual widths (tensor-core
    # instances) 8, 8, 16 and 24
    dict(shape=(9, 7, 1), nSam=300, nCha=3, nTerm=9),
    dict(shape=(12, 1, 1), nSam=300, nCha=3, nTerm=9),
    dict(shape=(6, 5, 4), nSam=300, nCha=3, nTerm=16),
    dict(shape=(6, 5, 4), nSam=300, nCha=3, nTerm=16, conc=True),
    dict(shape=(16, 16, 1), nSam=640, nCha=8, nTerm=16, masked=False),
    # degenerate sizes: one voxel and one sample, two samples, one sample of
    # a 3-D grid with concomitant terms, the tensor cores' largest coil count
    # (64) on one voxel row, fewer samples than one 64-column stage
    dict(shape=(1, 1, 1), nSam=1, nCha=1, nTerm=9, masked=False),
    dict(shape=(3, 1, 1), nSam=2, nCha=2, nTerm=16, masked=False),
    dict(shape=(2, 2, 2), nSam=1, nCha=8, nTerm=16, conc=True, masked=False),
    dict(shape=(1, 7, 1), nSam=65, nCha=64, nTerm=16),
    dict(shape=(5, 3, 1), nSam=63, nCha=17, nTerm=9),
]


def run_small(engine, params, seed=11):
    w = workloads.small(seed=seed, **params)
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine=engine, **w.op_kwargs())
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    m = oracle.Model(bf, k, t, f, c, nTerm=w.kspha.shape[0])
    mask = np.zeros(w.x.size, dtype=bool)
    mask[idx] = True
    rng = np.random.default_rng(seed + 1)
    y0 = rng.standard_normal(w.nSam * w.nCha) + 1j * rng.standard_normal(w.nSam * w.nCha)
    return op, m, mask, w, y0


@pytest.mark.parametrize("engine", ENGINE_PARAMS)
@pytest.mark.parametrize("params", SMALL, ids=lambda p: "x".join(map(str, p["shape"])) + f"-{p['nSam']}s-{p['nCha']}c"
                         + f"-{p['nTerm']}t" + ("-conc" if p.get("conc") else ""))
def test_small_problems_vs_oracle(engine, params):
    maybe_skip(engine)
    op, m, mask, w, y0 = run_small(engine, params)
    tol = TOL[engine]
    yo = oracle.forward(m, w.x[mask])
    xo = oracle.scatter(oracle.adjoint(m, y0), mask)
    yg = host(op * dev(w.x))
    xg = host(op.H * dev(y0))
    assert dense.rel(yg, yo) < tol
    assert dense.rel(xg, xo) < tol
    assert np.all(xg[~mask] == 0)
    no = oracle.scatter(oracle.adjoint(m, oracle.forward(m, w.x[mask])), mask)
    assert dense.rel(host(normalOperator(op) * dev(w.x)), no) < tol
    op.check()
    op.close()


@pytest.mark.parametrize("engine", ENGINE_PARAMS)
def test_config1_full_size_vs_oracle(engine):
    maybe_skip(engine)
    tol = TOL[engine]
    w = workloads.config1()
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine=engine, **w.op_kwargs())
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    m = oracle.Model(bf, k, t, f, c)
    yo = oracle.forward(m, w.x[idx])
    yg = host(op * dev(w.x))
    assert dense.rel(yg, yo) < tol
    rng = np.random.default_rng(5)
    y = yo + 0.01 * np.linalg.norm(yo) / np.sqrt(yo.size) * (rng.standard_normal(yo.size) + 1j * rng.standard_normal(yo.size))
    xo = oracle.adjoint(m, y)
    xg = host(op.H * dev(y))
    assert dense.rel(xg[idx], xo) < tol
    op.check()  # no bounded device wait ran out
    info = op.info()
    assert info["residual_phase_bound"] < 16.0  # worst-case bound of the FP32 residual phase (cycles)
    # 2-D slice: solid harmonics through third order span 9 directions, +1 fieldmap
    assert info["residual_rank"] <= 10 and info["residual_width"] == 12


def test_config2_full_size_properties():
    # the 200x200 / 12,000-sample / 16-coil workload at full size on the
    # tensor-core engine: FP64 spot check on sampled rows, agreement with the
    # FP32 engine, adjoint identity, linearity, bitwise repeatability, and the
    # fused normal against E^H (D * E x)
    maybe_skip("tc")
    w = workloads.config2()
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="tc", **w.op_kwargs())
    rng = np.random.default_rng(12)
    x = dev(w.x)
    y0 = op * x
    ynp = host(y0)
    # FP64 oracle on 48 sampled rows (all coils)
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    rows = np.sort(rng.choice(w.nSam, 48, replace=False))
    m = oracle.Model(bf, k[:, rows], t[rows], f, c, nTerm=w.kspha.shape[0])
    yo = oracle.forward(m, w.x[idx])
    assert dense.rel(ynp.reshape(w.nCha, w.nSam)[:, rows].reshape(-1), yo) < 1e-4
    # FP32 engine at full size
    op32 = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="fp32", **w.op_kwargs())
    y = dev(ynp + 0.05 * np.linalg.norm(ynp) / np.sqrt(ynp.size) * (rng.standard_normal(ynp.size) + 1j * rng.standard_normal(ynp.size)))
    assert dense.rel(ynp, host(op32 * x)) < 1e-4
    xa = op.H * y
    assert dense.rel(host(xa), host(op32.H * y)) < 1e-4
    # adjoint identity <y, E x> = <E^H y, x>
    lhs = np.vdot(host(y), ynp)
    rhs = np.vdot(host(xa), host(x))
    assert abs(lhs - rhs) / (np.linalg.norm(ynp) * np.linalg.norm(host(y))) < 1e-5
    # linearity
    x2 = dev(rng.standard_normal(op.ncol) + 1j * rng.standard_normal(op.ncol))
    a, b = 0.7 - 0.2j, -1.3 + 0.4j
    lin = host(op * (a * x + b * x2))
    assert dense.rel(lin, a * ynp + b * host(op * x2)) < 1e-5
    # repeatability (fixed reduction order)
    assert np.array_equal(host(op * x), ynp)
    # fused normal vs E^H (D * E x)
    D = np.tile(0.05 + rng.random(w.nSam), w.nCha)
    nrm = host(normalOperator(op, D) * x)
    ref = host(op.H * dev(D * ynp))
    assert dense.rel(nrm, ref) < 1e-4
    op.check()
    op32.close()
    op.close()


def test_derivative_mode_vs_oracle():
    # array_operator.jl:153-166 / 187-235: kspha_dt switches prod to B x
    w = workloads.small(seed=3, shape=(11, 10, 1), nSam=260, nCha=4, nTerm=16, conc=True)
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, kspha_dt=w.kspha_dt, engine="fp32", **w.op_kwargs())
    bf, k, t, f, c, idx = workloads.prepared_model(w, derivative=True)
    m = oracle.Model(bf, k, t, f, c)
    bo = oracle.derivative(m, w.kspha_dt, w.x[idx])
    bg = host(op * dev(w.x))
    assert dense.rel(bg, bo) < 1e-5


DERIV_CASES = [
    dict(shape=(11, 10, 1), nSam=260, nCha=4, nTerm=16, conc=True),   # one pass of 16 terms
    dict(shape=(12, 11, 1), nSam=300, nCha=8, nTerm=9),               # 8 terms, then 1
    dict(shape=(10, 12, 1), nSam=700, nCha=16, nTerm=16),             # four passes of 4 terms
    dict(shape=(9, 13, 1), nSam=333, nCha=20, nTerm=9),               # 3 terms of 20 coils per pass
    dict(shape=(10, 10, 1), nSam=280, nCha=10, nTerm=16),             # 6, 6, then 4 terms of 10 coils
]


@pytest.mark.parametrize("case", DERIV_CASES, ids=lambda c: f"{c['nCha']}c-{c['nTerm']}t")
def test_tc_derivative_vs_oracle(case):
    # the tensor-core derivative: B x = 2 pi i sum_l kdot[l,s] E(bf_l . x)
    # (array_operator.jl:187-235) from virtual-coil forward passes
    if not have_tc():
        pytest.skip("tensor-core engine unavailable")
    w = workloads.small(seed=11, **case)
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, kspha_dt=w.kspha_dt, engine="tc", **w.op_kwargs())
    op32 = HighOrderExplicitOp(w.grid, w.kspha, w.times, kspha_dt=w.kspha_dt, engine="fp32", **w.op_kwargs())
    bf, k, t, f, c, idx = workloads.prepared_model(w, derivative=True)
    bo = oracle.derivative(oracle.Model(bf, k, t, f, c), w.kspha_dt, w.x[idx])
    bg = host(op * dev(w.x))
    assert dense.rel(bg, bo) < 1e-4, dense.rel(bg, bo)
    assert dense.rel(bg, host(op32 * dev(w.x))) < 1e-4
    assert np.array_equal(host(op * dev(w.x)), bg)   # fixed reduction order
    op.check()
    op32.close()
    op.close()


def test_tc_derivative_config2_full_size():
    # B x at 200x200 / 12,000 samples / 16 coils / 16 terms (4 passes): FP64
    # spot check on sampled rows, agreement with the FP32 engine, linearity,
    # bitwise repeatability
    maybe_skip("tc")
    w = workloads.config2()
    kw = dict(kspha_dt=w.kspha_dt, **w.op_kwargs())
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="tc", **kw)
    rng = np.random.default_rng(13)
    x = dev(w.x)
    bnp = host(op * x)
    bf, k, t, f, c, idx = workloads.prepared_model(w, derivative=True)
    rows = np.sort(rng.choice(w.nSam, 48, replace=False))
    m = oracle.Model(bf, k[:, rows], t[rows], f, c, nTerm=w.kspha.shape[0])
    bo = oracle.derivative(m, np.asarray(w.kspha_dt)[:, rows], w.x[idx])
    assert dense.rel(bnp.reshape(w.nCha, w.nSam)[:, rows].reshape(-1), bo) < 1e-4
    op32 = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="fp32", **kw)
    assert dense.rel(bnp, host(op32 * x)) < 1e-4
    x2 = dev(rng.standard_normal(op.ncol) + 1j * rng.standard_normal(op.ncol))
    a, b = 0.6 + 0.3j, -1.1 + 0.2j
    assert dense.rel(host(op * (a * x + b * x2)), a * bnp + b * host(op * x2)) < 1e-4
    assert np.array_equal(host(op * x), bnp)
    op.check()
    op32.close()
    op.close()


# relative L2 tolerances of the backward vs the FP64 oracle's analytic gradient
BWD_TOL = {"fp32": 1e-4, "tc": 1e-3}


BWD_CASES = [
    dict(shape=(10, 9, 1), nSam=300, nCha=4, nTerm=16),            # residual width 16, 4 coils
    dict(shape=(11, 9, 1), nSam=300, nCha=8, nTerm=9),             # width 8, 8 coils
    dict(shape=(9, 8, 1), nSam=280, nCha=12, nTerm=9),             # width 8, 12 coils
    dict(shape=(7, 6, 3), nSam=260, nCha=6, nTerm=16, conc=True),  # width 24
]


@pytest.mark.parametrize("engine", ENGINE_PARAMS)
@pytest.mark.parametrize("case", range(len(BWD_CASES)))
def test_backward_vs_oracle_and_fd(engine, case):
    maybe_skip(engine)
    check_backward_vs_oracle(engine, BWD_CASES[case])


# 17-32 coils: the tensor-core backward only (KC = 64, 2-stage ring, 2-tile
# basis ring); the FP32 backward kernel stops at 16 coils
@pytest.mark.parametrize("params", [dict(shape=(10, 9, 1), nSam=300, nCha=24, nTerm=16),
                                    dict(shape=(9, 8, 1), nSam=280, nCha=32, nTerm=9),
                                    dict(shape=(64, 64, 1), nSam=6000, nCha=20, nTerm=16)],
                         ids=["24c", "32c", "20c-long"])
def test_tc_backward_many_coils_vs_oracle(params):
    maybe_skip("tc")
    check_backward_vs_oracle("tc", params)


def test_backward_coil_limits_raise():
    # beyond the kernels' coil counts the call fails cleanly (ArgumentError)
    maybe_skip("tc")
    for engine, nCha in (("fp32", 20), ("tc", 40)):
        w = workloads.small(seed=4, shape=(8, 8, 1), nSam=200, nCha=nCha, nTerm=9)
        op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine=engine, **w.op_kwargs())
        x = dev(w.x)
        with pytest.raises(ArgumentError):
            op.backward(x, op * x)
        op * x   # the operator stays usable
        op.check()
        op.close()


def check_backward_vs_oracle(engine, params):
    w = workloads.small(seed=4, **params)
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, kdot=w.kspha_dt, engine=engine, **w.op_kwargs())
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    # kspha_dt has the nTerm rows of kspha (no concomitant rows)
    m = oracle.Model(bf, k, t, f, c, nTerm=w.kspha.shape[0])
    rng = np.random.default_rng(9)
    y = oracle.forward(m, w.x[idx]) * 0.9 + 0.05 * (rng.standard_normal(w.nSam * w.nCha) + 1j * rng.standard_normal(w.nSam * w.nCha))
    r = oracle.forward(m, w.x[idx]) - y
    dk_o, ddf_o, t0b, t0c = oracle.backward(m, w.x[idx], r, w.kspha_dt)
    dk, ddf, dt0 = op.backward(dev(w.x), dev(r), t0_coef=True)
    dk = dk.cpu().numpy().astype(np.float64)
    ddf = ddf.cpu().numpy().astype(np.float64)
    tol = BWD_TOL[engine]
    assert dense.rel(dk, dk_o) < tol
    assert dense.rel(ddf[idx], ddf_o) < tol
    assert np.all(ddf[np.setdiff1d(np.arange(ddf.size), idx)] == 0)
    assert abs(dt0.item() - (t0b + t0c)) <= tol * abs(t0b + t0c)
    op.check()
    op.close()


def test_tc_backward_long_pipeline_matches_fp32_engine():
    # 200x200 spiral, 12,000 samples, 16 coils: ~387 stages per CTA, so the
    # dk accumulators are flushed every 32 stages and at row-tile ends
    maybe_skip("tc")
    w = workloads.config2()
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="tc", **w.op_kwargs())
    rng = np.random.default_rng(5)
    x = dev(w.x)
    r = op * x - dev(0.98 * (op * x).cpu().numpy() + 0.02 * (rng.standard_normal(op.nrow) + 1j * rng.standard_normal(op.nrow)))
    a = op.backward(x, r)
    op.set_engine("fp32")
    b = op.backward(x, r)
    for u, v in zip(a, b):
        u = u.cpu().numpy().astype(np.float64).ravel()
        v = v.cpu().numpy().astype(np.float64).ravel()
        assert np.all(np.isfinite(u))
        assert dense.rel(u, v) < 2e-3
    op.check()
    op.close()


@pytest.mark.parametrize("nCha", [8, 16])
def test_tc_backward_width24_matches_fp32_engine(nCha):
    # 3D grid with concomitant terms: residual rank 17-24, TF32 residual width
    # 24 (the 16-coil instance runs a 2-stage ring); tens of stages per CTA
    maybe_skip("tc")
    w = workloads.small(seed=8, shape=(24, 24, 8), nSam=3000, nCha=nCha, nTerm=16, conc=True)
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, kdot=w.kspha_dt, engine="tc", **w.op_kwargs())
    assert op.info()["residual_width"] == 24
    rng = np.random.default_rng(6)
    x = dev(w.x)
    r = op * x - dev(0.98 * (op * x).cpu().numpy() + 0.02 * (rng.standard_normal(op.nrow) + 1j * rng.standard_normal(op.nrow)))
    a = op.backward(x, r, t0_coef=True)
    op.set_engine("fp32")
    b = op.backward(x, r, t0_coef=True)
    for u, v in zip(a, b):
        u = u.cpu().numpy().astype(np.float64).ravel()
        v = v.cpu().numpy().astype(np.float64).ravel()
        assert np.all(np.isfinite(u))
        assert dense.rel(u, v) < 2e-3
    op.check()
    op.close()


def test_failure_injection_cleans_up():
    # host-side fault injection: the 3rd device allocation of create fails
    g = load("gpu_case_0")
    os.environ["HOE_INJECT_ALLOC_FAIL"] = "3"
    try:
        with pytest.raises(OutOfMemoryError):
            op_from_golden(g, "fp32")
    finally:
        del os.environ["HOE_INJECT_ALLOC_FAIL"]
    op = op_from_golden(g, "fp32")  # the next construction succeeds
    assert dense.rel(host(op * dev(g["image"])), g["forward"]) < 1e-5
    op.close()


def test_host_round_trip_numpy():
    g = load("gpu_case_2")
    op = op_from_golden(g, "fp32")
    y = op * g["image"].astype(np.complex64)
    assert isinstance(y, np.ndarray)
    assert dense.rel(y, g["forward"]) < 1e-5
    # page-locked host tensors come back page-locked
    xp = torch.from_numpy(g["image"].astype(np.complex64)).pin_memory()
    yp = op * xp
    assert yp.device.type == "cpu" and yp.is_pinned()
    assert dense.rel(yp.numpy(), g["forward"]) < 1e-5


@pytest.mark.parametrize("engine", ENGINE_PARAMS)
def test_in_place_products_with_host_buffers(engine):
    # mul!(y, op, x) / mul!(x, adjoint(op), y) with host tensors: page-locked
    # operands are queued without a host wait (valid after a synchronise);
    # back-to-back calls reuse the operator's device buffers in stream order
    maybe_skip(engine)
    g = load("gpu_case_2")
    op = op_from_golden(g, engine)
    tol = TOL[engine]
    x0 = torch.from_numpy(g["image"].astype(np.complex64))
    y0 = torch.from_numpy(g["probe"].astype(np.complex64))
    xs = [x0.pin_memory(), (x0 * (0.5 - 0.25j)).pin_memory()]
    yo = [torch.empty(op.nrow, dtype=torch.complex64, pin_memory=True) for _ in xs]
    for x, y in zip(xs, yo):
        assert op.prod_(y, x) is y
    xo = torch.empty(op.ncol, dtype=torch.complex64, pin_memory=True)
    op.H.prod_(xo, y0.pin_memory())
    torch.cuda.synchronize()
    assert dense.rel(yo[0].numpy(), g["forward"]) < tol
    assert dense.rel(yo[1].numpy(), (0.5 - 0.25j) * g["forward"]) < tol
    assert dense.rel(xo.numpy(), g["adjoint"]) < tol
    # pageable host memory: copied synchronously, same results
    yp = torch.empty(op.nrow, dtype=torch.complex64)
    op.prod_(yp, x0)
    assert dense.rel(yp.numpy(), g["forward"]) < tol
    # device output from a host input, host output from a device input
    yd = torch.empty(op.nrow, dtype=torch.complex64, device="cuda")
    op.prod_(yd, xs[0])
    xh = torch.empty(op.ncol, dtype=torch.complex64, pin_memory=True)
    op.ctprod_(xh, yd)
    torch.cuda.synchronize()
    assert dense.rel(host(yd), g["forward"]) < tol
    assert dense.rel(xh.numpy(), (op.H * dev(g["forward"])).cpu().numpy()) < tol
    # the adjoint writes every grid point: zeros outside the mask, whatever
    # the output buffer held
    mask = g["mask"].astype(bool)
    xf = torch.full((op.ncol,), 7 - 3j, dtype=torch.complex64, device="cuda")
    op.ctprod_(xf, dev(g["probe"]))
    xf = host(xf)
    assert not mask.all() and np.all(xf[~mask] == 0)
    assert dense.rel(xf, g["adjoint"]) < tol
    with pytest.raises(DimensionMismatch):
        op.prod_(torch.empty(op.nrow + 1, dtype=torch.complex64), x0)
    with pytest.raises(ArgumentError):
        op.prod_(yp, x0.to(torch.complex128))


def test_timing_trace():
    w = workloads.small(seed=2, shape=(16, 16, 1), nSam=512, nCha=8)
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="fp32", **w.op_kwargs())
    op.set_timing(True)
    y = op * dev(w.x)
    op.H * y
    t = op.timings()
    assert t["forward_kernel_ms"] > 0 and t["adjoint_kernel_ms"] > 0
    assert t["forward_total_ms"] >= t["forward_kernel_ms"]
    assert t["launches"] >= 6


def test_autotune_keeps_results_correct():
    w = workloads.small(seed=31, shape=(20, 17, 1), nSam=700, nCha=4)
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="fp32", **w.op_kwargs())
    r = op.autotune(reps=2)
    assert r["engine"] in ("fp32", "tc") and len(r["candidates"]) >= 2
    assert all(c["ms"] > 0 for c in r["candidates"])
    assert min(r["candidates"], key=lambda c: c["ms"])["engine"] == r["engine"]
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    m = oracle.Model(bf, k, t, f, c, nTerm=w.kspha.shape[0])
    assert dense.rel(host(op * dev(w.x)), oracle.forward(m, w.x[idx])) < TOL[r["engine"]]
    op.check()
    op.close()


def test_default_engine_is_chosen_by_the_device():
    # engine="auto" (the default): the tensor-core engine on a GB300 with at
    # most 64 coils, the FP32 engine otherwise; op.engine names the choice
    w = workloads.small(seed=33, shape=(16, 12, 1), nSam=500, nCha=3)
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, **w.op_kwargs())
    assert op.engine == ("tc" if have_tc() else "fp32")
    assert op.info()["engine"] == (1 if op.engine == "tc" else 0)
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    m = oracle.Model(bf, k, t, f, c, nTerm=w.kspha.shape[0])
    assert dense.rel(host(op * dev(w.x)), oracle.forward(m, w.x[idx])) < TOL[op.engine]
    op.set_engine("fp32")
    assert op.engine == "fp32"
    op.set_engine("auto")
    assert op.engine == ("tc" if have_tc() else "fp32")
    op.close()
    # more than 64 coils: the tensor-core engine is unavailable, AUTO takes FP32
    w = workloads.small(seed=34, shape=(6, 5, 1), nSam=140, nCha=66, nTerm=9)
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, **w.op_kwargs())
    assert op.engine == "fp32"
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    m = oracle.Model(bf, k, t, f, c, nTerm=w.kspha.shape[0])
    assert dense.rel(host(op * dev(w.x)), oracle.forward(m, w.x[idx])) < TOL["fp32"]
    with pytest.raises(ArgumentError):
        op.set_engine("tc")
    op.close()


def test_tc_many_coils_long_pipeline():
    # 40 coils use 64-coil MMA tiles; their shared-memory plan leaves a
    # one-deep residual-phase ring, so both phase-warp groups hand the same
    # tile buffer back and forth over ~8 stages per CTA in each direction
    maybe_skip("tc")
    w = workloads.small(seed=41, shape=(64, 48, 1), nSam=3000, nCha=40, nTerm=16)
    a = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="tc", **w.op_kwargs())
    b = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="fp32", **w.op_kwargs())
    x = dev(w.x)
    assert dense.rel(host(a * x), host(b * x)) < TOL["tc"]
    rng = np.random.default_rng(42)
    y = dev(rng.standard_normal(a.nrow) + 1j * rng.standard_normal(a.nrow))
    assert dense.rel(host(a.H * y), host(b.H * y)) < TOL["tc"]
    a.check()
    a.close()
    b.close()


@pytest.mark.parametrize("n,nSam,nCha", [(160, 9000, 8), (160, 9000, 24), (96, 6000, 40)],
                         ids=["8c-ring3", "24c-oneAbuf", "40c-twoAccSets"])
def test_tc_long_pipelines_match_fp32_engine(n, nSam, nCha):
    # each coil tile width has its own tensor-memory plan: 8 coils a three-deep
    # residual ring; 24 coils one A buffer and the 2N-wide product; 40 coils one
    # issuer, two alternating accumulator sets and a one-deep residual ring.
    # 40-190 stages per CTA run through many accumulator groups.
    maybe_skip("tc")
    w = workloads.spiral_slice(17, n, nSam, nCha, d=200e-3 / n)
    a = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="tc", **w.op_kwargs())
    b = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="fp32", **w.op_kwargs())
    x = dev(w.x)
    ya, yb = host(a * x), host(b * x)
    assert dense.rel(ya, yb) < TOL["tc"]
    y = dev(yb)
    assert dense.rel(host(a.H * y), host(b.H * y)) < TOL["tc"]
    a.check()
    a.close()
    b.close()


# Execution plans of the tensor-core contraction (hoe_desc.tc_plan, chosen by
# hoe_autotune): each plan is its own kernel instance, so each is held to the
# same tolerance against the FP64 oracle, at both coil widths (up to 8 and
# 9-16 coils) and the residual widths 8, 16 and 24
PLAN_CASES = [
    dict(shape=(13, 11, 1), nSam=257, nCha=6, nTerm=9),               # 8-coil tiles, width 8
    dict(shape=(9, 7, 1), nSam=300, nCha=3, nTerm=16),                # 8-coil tiles, width 16
    dict(shape=(14, 13, 1), nSam=333, nCha=12, nTerm=16, conc=True),  # 16-coil tiles, width 16
    dict(shape=(6, 5, 4), nSam=300, nCha=16, nTerm=16, conc=True),    # 16-coil tiles, width 24
]


@pytest.mark.parametrize("plan", range(5))
def test_tc_plans_vs_oracle(plan):
    maybe_skip("tc")
    for params in PLAN_CASES:
        w = workloads.small(seed=19, **params)
        op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="tc", tc_plan=plan, **w.op_kwargs())
        assert op.info()["tc_plan"] == plan
        bf, k, t, f, c, idx = workloads.prepared_model(w)
        m = oracle.Model(bf, k, t, f, c, nTerm=w.kspha.shape[0])
        mask = np.zeros(w.x.size, dtype=bool)
        mask[idx] = True
        yo = oracle.forward(m, w.x[idx])
        rng = np.random.default_rng(plan)
        y0 = rng.standard_normal(op.nrow) + 1j * rng.standard_normal(op.nrow)
        xo = oracle.scatter(oracle.adjoint(m, y0), mask)
        yg = host(op * dev(w.x))
        assert dense.rel(yg, yo) < TOL["tc"], (plan, params, dense.rel(yg, yo))
        assert dense.rel(host(op.H * dev(y0)), xo) < TOL["tc"]
        assert np.array_equal(host(op * dev(w.x)), yg)
        op.check()
        op.close()


@pytest.mark.parametrize("plan", range(5))
@pytest.mark.parametrize("nCha", [8, 16])
def test_tc_plans_long_pipeline(plan, nCha):
    # 160x160 spiral, 9,000 samples: ~150-190 stages per CTA in each direction,
    # so every plan wraps its stage ring and flushes its accumulators many times
    maybe_skip("tc")
    w = workloads.spiral_slice(23, 160, 9000, nCha, d=200e-3 / 160)
    a = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="tc", tc_plan=plan, **w.op_kwargs())
    b = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="fp32", **w.op_kwargs())
    x = dev(w.x)
    yb = host(b * x)
    assert dense.rel(host(a * x), yb) < TOL["tc"]
    y = dev(yb)
    assert dense.rel(host(a.H * y), host(b.H * y)) < TOL["tc"]
    a.check()
    a.close()
    b.close()


def test_autotune_times_every_tensor_core_plan():
    # up to 16 coils the autotuner times five tensor-core plans besides the
    # FP32 split factors, keeps the fastest and the products stay correct
    maybe_skip("tc")
    w = workloads.spiral_slice(29, 96, 4000, 12, d=200e-3 / 96)
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="tc", **w.op_kwargs())
    assert op.info()["tc_plans"] == 5
    r = op.autotune(reps=2)
    tc = [c for c in r["candidates"] if c["engine"] == "tc"]
    assert sorted(c["plan"] for c in tc) == [0, 1, 2, 3, 4]
    assert all(c["ms"] > 0 for c in r["candidates"])
    best_tc = min(tc, key=lambda c: c["ms"])
    assert r["tc_plan"] == best_tc["plan"] == op.info()["tc_plan"]
    assert min(r["candidates"], key=lambda c: c["ms"])["engine"] == r["engine"]
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    m = oracle.Model(bf, k, t, f, c, nTerm=w.kspha.shape[0])
    rows = np.sort(np.random.default_rng(1).choice(w.nSam, 64, replace=False))
    mr = oracle.Model(bf, k[:, rows], t[rows], f, c, nTerm=w.kspha.shape[0])
    y = host(op * dev(w.x)).reshape(w.nCha, w.nSam)[:, rows].reshape(-1)
    assert dense.rel(y, oracle.forward(mr, w.x[idx])) < TOL[r["engine"]]
    op.check()
    op.close()
    # more than 16 coils: the default plan only
    w = workloads.small(seed=5, shape=(10, 9, 1), nSam=300, nCha=20, nTerm=9)
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="tc", **w.op_kwargs())
    assert op.info()["tc_plans"] == 1
    with pytest.raises(ArgumentError):
        HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="tc", tc_plan=2, **w.op_kwargs())
    op.close()


def test_tc_bounded_wait_runs_out_and_the_operator_recovers():
    # failure detection without a GPU fault: HOE_INJECT_TC_STALL=4 makes the
    # first forward contraction of the operator skip fetching the operands of
    # CTA 0's fifth stage, with every wait limited to 1 ms.  The waits for that
    # stage run out, the kernel sets its abort flag, drains its own copies and
    # MMAs, frees tensor memory and returns; hoe_check reports HOE_ERR_TIMEOUT.
    # The injection is one-shot: the next products are correct.
    maybe_skip("tc")
    from hoexplicit import HoeError
    from hoexplicit import _lib as L
    w = workloads.small(seed=12, shape=(64, 64, 1), nSam=4000, nCha=8, nTerm=16)  # ~13 stages per CTA
    os.environ["HOE_INJECT_TC_STALL"] = "4"
    try:
        op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="tc", **w.op_kwargs())
    finally:
        del os.environ["HOE_INJECT_TC_STALL"]
    x = dev(w.x)
    op * x
    with pytest.raises(HoeError) as exc:
        op.check()
    assert f"[{L.HOE_ERR_TIMEOUT}]" in str(exc.value)
    op.check()   # the error word was cleared after reporting
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    m = oracle.Model(bf, k, t, f, c, nTerm=w.kspha.shape[0])
    rows = np.sort(np.random.default_rng(2).choice(w.nSam, 64, replace=False))
    mr = oracle.Model(bf, k[:, rows], t[rows], f, c, nTerm=w.kspha.shape[0])
    y_first = None
    for _ in range(2):
        yfull = host(op * x)
        y = yfull.reshape(w.nCha, w.nSam)[:, rows].reshape(-1)
        assert dense.rel(y, oracle.forward(mr, w.x[idx])) < TOL["tc"]
        if y_first is not None:
            assert np.array_equal(yfull, y_first)
        y_first = yfull
    op.check()
    op.close()


def test_sfu_rate_calibration():
    """hoe_sfu_rate: the special-function unit's sin/cos rate is a positive
    number of lane operations per clock per SM, at most one per lane of the
    SM's four 32-wide sub-partitions, and stable between calls."""
    from hoexplicit.operator import sfu_rate
    a, b = sfu_rate(), sfu_rate()
    assert 4.0 <= a <= 128.0, a
    assert abs(a - b) <= 0.1 * a, (a, b)
