"""Batches of operators (hoe_batch_*): all slices in one persistent launch per
direction, and per-slice CGNR solves in lockstep inside one CUDA graph.

A batched product must give each member's own product: against the member
applied alone (same engine) and against the FP64 oracle.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from hoexplicit import ArgumentError, DimensionMismatch, HighOrderExplicitOp, OperatorBatch, workloads  # noqa: E402
from hoexplicit import recon as hrecon  # noqa: E402
from oracle import oracle  # noqa: E402
from oracle.dense import rel  # noqa: E402
from tests.test_gpu_parity import maybe_skip  # noqa: E402

SHAPES = [((9, 7, 1), 300), ((20, 13, 1), 517), ((16, 16, 1), 129), ((11, 5, 3), 260)]


def small_ops(engine, shapes=SHAPES, nCha=3, seed0=20):
    ws, ops = [], []
    for i, (shape, nSam) in enumerate(shapes):
        w = workloads.small(seed=seed0 + i, shape=shape, nSam=nSam, nCha=nCha)
        ws.append(w)
        ops.append(HighOrderExplicitOp(w.grid, w.kspha, w.times, engine=engine, **w.op_kwargs()))
    return ws, ops


def kp_of(op):
    rp = op.info()["residual_width"]
    return 8 if rp <= 8 else (16 if rp <= 16 else 24)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.complex64)).cuda()


def host(t):
    return t.cpu().numpy().astype(np.complex128)


@pytest.mark.parametrize("engine", ["tc", "fp32"])
def test_batch_products_match_members_and_oracle(engine):
    maybe_skip(engine)
    ws, ops = small_ops(engine)
    B = OperatorBatch(ops)
    info = B.info()
    assert info["n"] == len(ops)
    if engine == "tc":
        assert info["contraction_launches"] == len({kp_of(op) for op in ops})
    else:
        assert info["contraction_launches"] == len(ops)
    xs = [dev(w.x) for w in ws]
    rng = np.random.default_rng(3)
    ys = [dev(rng.standard_normal(op.nrow) + 1j * rng.standard_normal(op.nrow)) for op in ops]
    yb = B.forward(xs)
    xb = B.adjoint(ys)
    nb = B.normal(xs)
    tol = 1e-4 if engine == "tc" else 1e-5
    for w, op, x, y, a, b, c in zip(ws, ops, xs, ys, yb, xb, nb):
        ya, xa, na = op * x, op.H * y, hrecon_normal(op, x)
        if engine == "fp32":  # members applied one after another: the same launches
            assert torch.equal(a, ya) and torch.equal(b, xa) and torch.equal(c, na)
        else:
            assert rel(host(a), host(ya)) < 2e-6
            assert rel(host(b), host(xa)) < 2e-6
            assert rel(host(c), host(na)) < 2e-6
        bf, k, t, f, cs, idx = workloads.prepared_model(w)
        m = oracle.Model(bf, k, t, f, cs, nTerm=w.kspha.shape[0])
        assert rel(host(a), oracle.forward(m, w.x[idx])) < tol
        assert rel(host(b)[idx], oracle.adjoint(m, host(y))) < tol
    B.check()
    B.close()
    for op in ops:
        op.close()


def hrecon_normal(op, x):
    from hoexplicit import normalOperator
    return normalOperator(op) * x


def test_batch_more_slices_than_one_launch_holds():
    maybe_skip("tc")
    shapes = [((7 + (i % 5), 6 + (i % 3), 1), 150 + 7 * i) for i in range(34)]
    ws, ops = small_ops("tc", shapes, nCha=2, seed0=100)
    B = OperatorBatch(ops)
    kps = [kp_of(op) for op in ops]
    expect = sum((kps.count(k) + 31) // 32 for k in set(kps))
    assert B.info()["contraction_launches"] == expect >= 2
    xs = [dev(w.x) for w in ws]
    for op, x, a in zip(ops, xs, B.forward(xs)):
        assert rel(host(a), host(op * x)) < 2e-6
    B.check()
    B.close()
    for op in ops:
        op.close()


@pytest.mark.parametrize("engine", ["tc", "fp32"])
def test_batch_recon_matches_member_solves(engine):
    maybe_skip(engine)
    ws, ops = small_ops(engine)
    B = OperatorBatch(ops)
    rng = np.random.default_rng(9)
    datas, weights = [], []
    for w, op in zip(ws, ops):
        y = host(op * dev(w.x))
        y = y + 0.01 * np.linalg.norm(y) / np.sqrt(y.size) * rng.standard_normal(y.size)
        datas.append(y.reshape(op.nCha, op.nSam).T)
        weights.append((0.5 + rng.random(op.nSam)) * np.exp(1j * rng.random(op.nSam)))
    xb, sb = B.recon(datas, weights, iterations=12, rel_tol=0.0, lam=1e-6)
    xb = [x.clone() for x in xb]
    xb2, sb2 = B.recon(datas, weights, iterations=12, rel_tol=0.0, lam=1e-6)  # cached graph
    for a, b in zip(xb, xb2):
        assert torch.equal(a, b)
    assert sb == sb2
    for w, op, d, wt, a, s in zip(ws, ops, datas, weights, xb, sb):
        x1, s1 = hrecon.solve(op, d, wt, iterations=12, rel_tol=0.0, lam=1e-6)
        if engine == "fp32":
            assert torch.equal(a, x1)
        else:
            assert rel(host(a), host(x1)) < 1e-4
        assert s["iterations"] == 12 and s["status"] == "iterations"
    B.check()
    B.close()
    for op in ops:
        op.close()


def test_batch_errors():
    maybe_skip("tc")
    ws, ops = small_ops("tc", SHAPES[:2])
    with pytest.raises(ArgumentError):
        OperatorBatch([])
    with pytest.raises(ArgumentError):
        OperatorBatch([ops[0], ops[0]])
    B = OperatorBatch(ops)
    with pytest.raises(DimensionMismatch):
        B.forward([dev(ws[0].x)])
    ops[1].close()
    with pytest.raises(ArgumentError):
        B.forward([dev(w.x) for w in ws])
    B.close()
    with pytest.raises(ArgumentError):
        B.forward([dev(w.x) for w in ws])
    ops[0].close()


def test_config5_full_size_batch():
    # the 24-slice workload (160^2-224^2 voxels, 8,000-20,000 samples, 16
    # coils) in one persistent launch per direction: each member's product
    # as applied alone, and an FP64 spot check on sampled rows of two slices
    maybe_skip("tc")
    ws = workloads.config5()
    ops = [HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="tc", **w.op_kwargs()) for w in ws]
    B = OperatorBatch(ops)
    assert B.info()["n"] == len(ws) == 24
    rng = np.random.default_rng(55)
    xs = [dev(w.x) for w in ws]
    ys = [dev(rng.standard_normal(op.nrow) + 1j * rng.standard_normal(op.nrow)) for op in ops]
    yb = B.forward(xs)
    xb = B.adjoint(ys)
    for op, x, y, a, b in zip(ops, xs, ys, yb, xb):
        assert rel(host(a), host(op * x)) < 2e-6
        assert rel(host(b), host(op.H * y)) < 2e-6
    for i in (0, len(ws) - 1):
        w = ws[i]
        bf, k, t, f, cs, idx = workloads.prepared_model(w)
        rows = np.sort(rng.choice(w.nSam, 32, replace=False))
        m = oracle.Model(bf, k[:, rows], t[rows], f, cs, nTerm=w.kspha.shape[0])
        ya = host(yb[i]).reshape(w.nCha, w.nSam)[:, rows].reshape(-1)
        assert rel(ya, oracle.forward(m, w.x[idx])) < 1e-4
    B.check()
    B.close()
    for op in ops:
        op.close()
