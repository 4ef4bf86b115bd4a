"""recon_HOOp on the device (hoe_recon): weighted CGNR captured in a CUDA graph.

Restates test/test_ReconstructionStability.jl:25-76 ("Raw sample weights in
reconstruction": CGNR through recon_HOOp vs a QR solve of the materialised
weighted operator, F32 tolerance 3e-4, F64 1e-10) with numpy seeds in place
of Julia's Xoshiro stream, and compares the device solve with the oracle's
FP64 CGNR (oracle/recon.py) on the 64x64 spiral workload.
"""
import numpy as np
import pytest

from hoexplicit import recon as hrecon
from hoexplicit import ArgumentError, DimensionMismatch
from oracle import oracle
from oracle import recon as orecon
from oracle.dense import rel


def raw_weight_problem(seed=514):
    """3x3 grid, 37 samples, 2 coils, 9 terms: test_ReconstructionStability.jl:27-42."""
    rng = np.random.default_rng(seed)
    nSam, nCha = 37, 2
    data = rng.standard_normal((nSam, nCha)) + 1j * rng.standard_normal((nSam, nCha))
    weight = (0.5 + rng.random(nSam)) * np.exp(1j * rng.random(nSam))
    kspha = rng.standard_normal((9, nSam)) * 0.01
    j = np.arange(nSam)
    kspha[1] = (np.mod(j, 3) - 1) / 3.0
    kspha[2] = (np.mod(j // 3, 3) - 1) / 3.0
    kspha[3] = 0.0
    times = np.linspace(0.0, 1e-3, nSam)
    csm = np.exp(1j * rng.random((3, 3, 1, nCha))) / np.sqrt(nCha)
    return data, weight, kspha, times, csm


def raw_weight_oracle(kspha, times, csm):
    x, y, z = oracle.grid(3, 3, 1, 1.0, 1.0, 1.0)
    bf = oracle.basis(x, y, z, list(range(1, 10)))
    nCha = csm.shape[-1]
    return oracle.Model(bf, kspha, times, np.zeros(9), csm.reshape(9, nCha, order="F"))


def qr_solution(m, data, weight):
    """Materialise the unweighted operator column by column and solve the
    weighted least-squares problem by QR (test_ReconstructionStability.jl:49-57)."""
    nVox = m.nVox
    E = np.zeros((m.nSam * m.nCha, nVox), dtype=np.complex128)
    for v in range(nVox):
        e = np.zeros(nVox, dtype=np.complex128)
        e[v] = 1.0
        E[:, v] = oracle.forward(m, e)
    wr = np.tile(weight, m.nCha)
    b = data.reshape(-1, order="F") * wr
    q, r = np.linalg.qr(E * wr[:, None])
    return np.linalg.solve(r, q.conj().T @ b)


def test_oracle_cgnr_matches_qr_raw_weights():
    data, weight, kspha, times, csm = raw_weight_problem()
    m = raw_weight_oracle(kspha, times, csm)
    expected = qr_solution(m, data, weight)
    x, st = orecon.recon(m, data.reshape(-1, order="F"), weight, iterations=30, rel_tol=1e-10)
    assert rel(x, expected) < 1e-10  # the reference's Float64 tolerance
    assert st["iterations"] <= 30


def test_oracle_cgnr_regularised_normal_equations():
    # (EᴴWᴴWE + λI) x = EᴴWᴴW d solved exactly for a well-conditioned system
    data, weight, kspha, times, csm = raw_weight_problem(7)
    m = raw_weight_oracle(kspha, times, csm)
    E = np.stack([oracle.forward(m, np.eye(9)[v]) for v in range(9)], axis=1)
    d2 = np.tile(np.abs(weight) ** 2, m.nCha)
    lam = 0.05
    A = E.conj().T @ (d2[:, None] * E) + lam * np.eye(9)
    b = E.conj().T @ (d2 * data.reshape(-1, order="F"))
    x, _ = orecon.recon(m, data.reshape(-1, order="F"), weight, iterations=40, rel_tol=1e-13, lam=lam)
    assert rel(x, np.linalg.solve(A, b)) < 1e-10


def test_recon_parameter_validation_host_side():
    with pytest.raises(KeyError):
        hrecon._required({"solver": hrecon.CGNR}, "reg")
    assert hrecon._required({":reconSize": (3, 3)}, "reconSize") == (3, 3)
    assert hrecon._solver_ok(hrecon.CGNR) and hrecon._solver_ok("CGNR")
    assert not hrecon._solver_ok("admm")
    assert hrecon._reg_lambda(hrecon.L2Regularization(1e-9)) == 1e-9
    assert hrecon._reg_lambda([hrecon.L2Regularization(0.0)]) == 0.0
    with pytest.raises(ArgumentError):
        hrecon._reg_lambda("L1")
    with pytest.raises(ArgumentError):
        hrecon.L2Regularization(-1.0)
    with pytest.raises(ArgumentError):
        hrecon.recon_HOOp(object(), np.zeros((3, 1)), np.ones(3),
                          {"solver": hrecon.CGNR, "reg": hrecon.L2Regularization(0.0), "reconSize": (2, 2)})


# --------------------------------------------------------------------- GPU
torch = pytest.importorskip("torch")

from hoexplicit import Grid, HighOrderExplicitOp, workloads  # noqa: E402
from tests.test_gpu_parity import ENGINE_PARAMS, maybe_skip  # noqa: E402


def raw_weight_op(engine):
    data, weight, kspha, times, csm = raw_weight_problem()
    op = HighOrderExplicitOp(Grid(3, 3, 1, 1.0, 1.0, 1.0), kspha, times, csm=csm, engine=engine)
    return op, data, weight, kspha, times, csm


@pytest.mark.gpu
@pytest.mark.parametrize("engine", ENGINE_PARAMS)
def test_recon_raw_sample_weights_vs_qr(engine):
    maybe_skip(engine)
    op, data, weight, kspha, times, csm = raw_weight_op(engine)
    m = raw_weight_oracle(kspha, times, csm)
    expected = qr_solution(m, data, weight)
    data0, weight0 = data.copy(), weight.copy()
    params = {"solver": hrecon.CGNR, "reg": hrecon.L2Regularization(0.0),
              "reconSize": (3, 3, 1), "iterations": 30, "relTol": 1e-10}
    image, st = hrecon.recon_HOOp(op, data.astype(np.complex64), weight.astype(np.complex64), params,
                                  return_stats=True)
    assert image.dtype == np.complex64
    assert image.shape == (3, 3, 1)
    assert rel(image.reshape(-1, order="F").astype(np.complex128), expected) < 3e-4  # Float32 tolerance
    assert np.array_equal(data, data0) and np.array_equal(weight, weight0)
    assert 0 < st["iterations"] <= 30
    op.check()
    op.close()


@pytest.mark.gpu
def test_recon_docs_example_cartesian():
    # docs/src/reference/recon-hoop.md: full Cartesian 8x8, λ = 1e-3, 10 iterations
    nX = nY = 8
    grid = Grid(nX, nY, 1, 1e-3, 1e-3, 5e-3)
    nSam = nX * nY
    kspha = np.zeros((9, nSam))
    kspha[1] = np.tile(np.arange(-4, 4) / (nX * 1e-3), nY)
    kspha[2] = np.repeat(np.arange(-4, 4) / (nY * 1e-3), nX)
    op = HighOrderExplicitOp(grid, kspha, np.zeros(nSam), engine="fp32")
    reference = np.zeros((nX, nY, 1), dtype=np.complex64)
    reference[2:6, 2:6, 0] = 1
    samples = (op * reference.reshape(-1, order="F")).reshape(nSam, 1, order="F")
    params = {":reconSize": grid.matrixSize, ":solver": hrecon.CGNR,
              ":reg": hrecon.L2Regularization(1e-3), ":iterations": 10}
    image = hrecon.recon_HOOp(op, samples, np.ones(nSam, dtype=np.complex64), params)
    assert image.shape == grid.matrixSize and np.all(np.isfinite(image))
    # unitary DFT encoding: the regularised solution is reference/(1+λ)
    assert rel(image.astype(np.complex128), reference / (1 + 1e-3)) < 1e-4
    op.close()


def _config1_problem():
    w = workloads.config1()
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    m = oracle.Model(bf, k, t, f, c)
    rng = np.random.default_rng(11)
    y = oracle.forward(m, w.x[idx])
    y = y + 0.01 * np.linalg.norm(y) / np.sqrt(y.size) * (rng.standard_normal(y.size) + 1j * rng.standard_normal(y.size))
    # square-root density-like weights: larger at the periphery of the spiral
    kr = np.hypot(w.kspha[1], w.kspha[2])
    weight = np.sqrt(0.05 + kr / kr.max()) * np.exp(0.3j * rng.standard_normal(w.nSam))
    return w, m, idx, y, weight


@pytest.mark.gpu
@pytest.mark.parametrize("engine", ENGINE_PARAMS)
def test_recon_config1_vs_oracle_cgnr(engine):
    maybe_skip(engine)
    w, m, idx, y, weight = _config1_problem()
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine=engine, **w.op_kwargs())
    data = y.reshape(w.nCha, w.nSam).T  # (nSam, nCha), samples fastest in vec
    lam = 1e-9
    xo, so = orecon.recon(m, y, weight, iterations=20, rel_tol=0.0, lam=lam)
    x, st = hrecon.solve(op, data, weight, iterations=20, rel_tol=0.0, lam=lam)
    xg = x.cpu().numpy().astype(np.complex128)
    err = rel(xg[idx], xo)
    assert err < (1e-4 if engine == "fp32" else 1e-3), err
    assert np.all(xg[np.setdiff1d(np.arange(xg.size), idx)] == 0)
    assert st["iterations"] == 20 and st["status"] == "iterations"
    assert abs(st["residual0"] - so["residual0"]) < 1e-4 * so["residual0"]
    assert st["residual"] < st["residual0"]
    op.check()
    op.close()


@pytest.mark.gpu
def test_recon_graph_matches_direct_launches_bitwise():
    w, m, idx, y, weight = _config1_problem()
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="fp32", **w.op_kwargs())
    data = y.reshape(w.nCha, w.nSam).T
    a, _ = hrecon.solve(op, data, weight, iterations=8, use_graph=False)
    a = a.clone()
    out = torch.empty_like(a)
    b, sb = hrecon.solve(op, data, weight, iterations=8, use_graph=True, out=out)
    b1 = b.clone()
    c, sc = hrecon.solve(op, data, weight, iterations=8, use_graph=True, out=out)  # cached graph replay
    assert torch.equal(a, b1) and torch.equal(b1, c)
    assert sb == sc
    op.close()


@pytest.mark.gpu
def test_recon_early_convergence_and_regularisation():
    w, m, idx, y, weight = _config1_problem()
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="fp32", **w.op_kwargs())
    data = y.reshape(w.nCha, w.nSam).T
    x, st = hrecon.solve(op, data, weight, iterations=50, rel_tol=0.3)
    assert st["status"] == "converged" and st["iterations"] < 50
    assert st["residual"] <= 0.3 * st["residual0"]
    xo, so = orecon.recon(m, y, weight, iterations=50, rel_tol=0.3)
    assert so["iterations"] == st["iterations"]
    assert rel(x.cpu().numpy().astype(np.complex128)[idx], xo) < 1e-4
    # strong Tikhonov weight: compare with the oracle's regularised solve
    lam = 10.0 * so["residual0"] / max(np.linalg.norm(xo), 1e-30)
    xg, _ = hrecon.solve(op, data, weight, iterations=6, lam=lam)
    xo2, _ = orecon.recon(m, y, weight, iterations=6, lam=lam)
    assert rel(xg.cpu().numpy().astype(np.complex128)[idx], xo2) < 1e-4
    # zero data: x = 0, converged before the first update
    x0, s0 = hrecon.solve(op, np.zeros_like(data), weight, iterations=5)
    assert s0["iterations"] == 0 and s0["status"] == "converged" and not torch.any(x0 != 0)
    with pytest.raises(DimensionMismatch):
        hrecon.solve(op, data[:-1], weight)
    op.close()
    with pytest.raises(ArgumentError):
        hrecon.solve(op, data, weight)
