"""Host-side logic of the product package (no GPU): grid, basis, order
selection, concomitant terms, normal-weight validation, workloads."""
import numpy as np
import pytest

from hoexplicit import ArgumentError, DimensionMismatch, Grid, basisfunc_spha, prep_concomitant, prep_kspha
from hoexplicit.operator import WeightingOp, normal_diagonal
from hoexplicit import workloads
from oracle import dense, oracle


def test_grid_matches_oracle_and_roundtrips():
    g = Grid(5, 4, 3, 0.7, 0.9, 1.2)
    x, y, z = oracle.grid(5, 4, 3, 0.7, 0.9, 1.2)
    assert np.allclose(g.x, x) and np.allclose(g.y, y) and np.allclose(g.z, z)
    g2 = Grid.from_dict(g.struct_to_dict())
    assert g2.matrixSize == g.matrixSize and np.array_equal(g2.x, g.x)


def test_grid_orientation_keywords():
    # Grid.jl:83-94: exchange_xy swaps the coordinate vectors, reverse_*
    # reverses one flattened vector; sizes and spacings are unchanged
    g = Grid(5, 4, 3, 0.7, 0.9, 1.2)
    e = Grid(5, 4, 3, 0.7, 0.9, 1.2, exchange_xy=True)
    assert np.array_equal(e.x, g.y) and np.array_equal(e.y, g.x) and np.array_equal(e.z, g.z)
    r = Grid(5, 4, 3, 0.7, 0.9, 1.2, reverse_x=True, reverse_z=True)
    assert np.array_equal(r.x, g.x[::-1]) and np.array_equal(r.y, g.y) and np.array_equal(r.z, g.z[::-1])
    b = Grid(5, 4, 3, 0.7, 0.9, 1.2, exchange_xy=True, reverse_y=True)
    assert np.array_equal(b.y, g.x[::-1]) and np.array_equal(b.x, g.y)
    assert b.matrixSize == (5, 4, 3) and b.resolution == (0.7, 0.9, 1.2)


def test_prep_kspha_three_dimensional():
    # prep_kspha.jl:59-73: (nTerm, nSam, nDyn) coefficients are prepared as
    # one column-major (nTerm, nSam*nDyn) matrix; each dynamic equals the
    # two-dimensional preparation of its own slab
    rng = np.random.default_rng(8)
    k = rng.standard_normal((16, 11, 3))
    kn = rng.standard_normal((3, 11, 3))
    out = prep_kspha(k, kn, 16, "0101")
    assert out.shape == k.shape
    for d in range(3):
        assert np.array_equal(out[:, :, d], prep_kspha(k[:, :, d], kn[:, :, d], 16, "0101"))
    with pytest.raises(DimensionMismatch):
        prep_kspha(k, kn[:, :, :2], 16, None)
    # concomitant rows for 3-D coefficients: (4, nSam, nDyn), or (4, nSam) for one dynamic
    x, y, z = rng.standard_normal((3, 6))
    bf = rng.standard_normal((6, 16))
    c = rng.standard_normal((4, 11, 3))
    b2, k2 = prep_concomitant(bf, out, x, y, z, c)
    assert b2.shape == (6, 20) and k2.shape == (20, 11, 3) and np.array_equal(k2[16:], c)
    b1, k1 = prep_concomitant(bf, out[:, :, :1], x, y, z, c[:, :, 0])
    assert k1.shape == (20, 11, 1) and np.array_equal(k1[16:, :, 0], c[:, :, 0])
    with pytest.raises(DimensionMismatch):
        prep_concomitant(bf, out, x, y, z, c[:, :, 0])


def test_basis_matches_oracle():
    rng = np.random.default_rng(1)
    x, y, z = rng.standard_normal((3, 40))
    assert np.allclose(basisfunc_spha(x, y, z, list(range(1, 17))),
                       oracle.basis(x, y, z, list(range(1, 17))), rtol=1e-14, atol=1e-14)
    assert np.allclose(basisfunc_spha(x, y, z, [4, 2]), oracle.basis(x, y, z, [4, 2]))
    with pytest.raises(ArgumentError):
        basisfunc_spha(x, y, z, [37])


def test_prep_kspha_flags_and_copy():
    # prep_kspha.jl:1-56 and test/test_explicit_interface.jl:24-30 ("0011" + k_nominal)
    rng = np.random.default_rng(2)
    k = rng.standard_normal((16, 13))
    kn = rng.standard_normal((3, 13))
    kc = k.copy()
    e = prep_kspha(k, kn, 16, "0011")
    assert np.array_equal(k, kc)  # never mutates its input
    assert np.all(e[0] == 0) and np.array_equal(e[1:4], kn) and np.array_equal(e[4:], k[4:])
    e = prep_kspha(k, kn, 16, "1100")
    assert np.all(e[4:] == 0) and np.array_equal(e[:4], k[:4])
    e9 = prep_kspha(k[:9], kn, 9, None)
    assert np.array_equal(e9, k[:9])
    for bad in ("111", "11111", "11a1"):
        with pytest.raises(ArgumentError):
            prep_kspha(k, kn, 16, bad)
    with pytest.raises(ArgumentError):
        prep_kspha(k[:10], kn, 10, None)


def test_prep_concomitant():
    rng = np.random.default_rng(3)
    x, y, z = rng.standard_normal((3, 7))
    bf = rng.standard_normal((7, 16))
    k = rng.standard_normal((16, 5))
    c = rng.standard_normal((4, 5))
    b2, k2 = prep_concomitant(bf, k, x, y, z, c)
    assert b2.shape == (7, 20) and k2.shape == (20, 5)
    assert np.allclose(b2[:, 16:], np.stack([z * z, x * x + y * y, x * z, y * z], 1))
    assert prep_concomitant(bf, k, x, y, z, None)[0] is bf
    with pytest.raises(DimensionMismatch):
        prep_concomitant(bf, k, x, y, z, c[:3])
    with pytest.raises(ArgumentError):
        prep_concomitant(bf, k, x, y, z, c.astype(complex))


def test_normal_weight_rules():
    # explicit_gpu_operator.jl:402-412
    ns, nc = 11, 3
    D = normal_diagonal(None, ns, nc)
    assert D.shape == (33,) and np.all(D == 1)
    D = normal_diagonal(np.arange(ns, dtype=float), ns, nc)
    assert D.shape == (33,) and np.array_equal(D[11:22], np.arange(ns))
    w = np.arange(1, ns + 1) * (1 + 1j)
    D = normal_diagonal(WeightingOp(w, nc), ns, nc)
    assert np.allclose(D, np.tile(2 * np.arange(1, ns + 1) ** 2, nc))
    with pytest.raises(ArgumentError):
        normal_diagonal(np.full(ns, 1 + 1j), ns, nc)
    with pytest.raises(ArgumentError):
        normal_diagonal(np.full(ns, -1.0), ns, nc)
    with pytest.raises(ArgumentError):
        normal_diagonal(np.full(ns, np.nan), ns, nc)
    with pytest.raises(DimensionMismatch):
        normal_diagonal(np.ones(ns + 1), ns, nc)


def test_workload_shapes():
    w = workloads.config1()
    assert w.kspha.shape == (16, 4096) and w.nCha == 8 and w.nVox == 64 * 64
    assert abs(w.times[1] - 2e-6) < 1e-15
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    assert bf.shape == (4096, 16) and c.shape == (4096, 8)
    w3 = workloads.config3()
    assert w3.kspha.shape[1] == 12000 and w3.nCha == 16


def test_host_plan_needs_no_device():
    # hoe_plan validates the descriptor and reports the tiling and the reduced
    # residual phase basis on the host; the default engine stays "auto" there
    from hoexplicit import _lib
    from hoexplicit.operator import plan
    w = workloads.config1()
    p = plan(w.grid, w.kspha, w.times, **w.op_kwargs())
    assert p["engine"] == _lib.HOE_ENGINE_AUTO
    assert (p["nSam"], p["nCha"], p["nVox"], p["nTermEff"]) == (4096, 8, 4096, 16)
    assert 1 <= p["residual_rank"] <= p["residual_width"] <= 24
    assert 0 < p["residual_phase_bound"] < 64 and p["device_bytes"] == 0
    assert plan(w.grid, w.kspha, w.times, engine="fp32", **w.op_kwargs())["engine"] == _lib.HOE_ENGINE_FP32_SIMT
    with pytest.raises(ArgumentError):
        plan(w.grid, w.kspha, w.times, engine="fp16", **w.op_kwargs())


def test_kernel_execution_keywords_get_the_reference_validation():
    """The CUDA implementation's execution keywords (kernel_operator.jl:223-236,
    explicit_gpu_operator.jl:313-320) are accepted by the :gb300 front with
    the reference's ArgumentErrors; valid ones reach the operator unchanged."""
    from hoexplicit import ArgumentError
    from hoexplicit.operator import check_kernel_options
    check_kernel_options()                                   # :legacy defaults
    check_kernel_options(backend=":blocked", phase_backend=":gemm", block_size=4, phase_cache_bytes=96)
    check_kernel_options(backend="cached_full", gemm_backend="auto", forward_threads=64, adjoint_threads=128)
    bad = [dict(backend=":blocked", phase_cache_bytes=-1),
           dict(backend=":direct", phase_cache_bytes=1),
           dict(backend=":cached", phase_cache_bytes=1),
           dict(phase_cache_bytes=1),                        # :legacy
           dict(backend=":fancy"),
           dict(backend=":blocked", phase_backend=":fft"),
           dict(backend=":blocked", gemm_backend=":cutlass"),
           dict(backend=":blocked", block_size=0),
           dict(backend=":blocked", forward_threads=96),
           dict(backend=":blocked", adjoint_threads=1024)]
    for kw in bad:
        with pytest.raises(ArgumentError):
            check_kernel_options(**kw)
    with pytest.raises(ArgumentError, match="kspha_dt requires backend=:legacy"):
        check_kernel_options(kspha_dt=np.zeros((9, 3)), backend=":blocked")


def test_basis_terms_17_to_36():
    """Fourth- and fifth-order terms of basisfunction.jl: the reference's
    known answer for term 17 (test_Concomitant.jl:92), and for every term the
    defining properties of a real solid harmonic: homogeneous of degree 4
    (terms 17-25) or 5 (26-36) with zero Laplacian, and each order's terms
    linearly independent (they span the 9- and 11-dimensional spaces)."""
    np.testing.assert_array_equal(basisfunc_spha([1.0, 2.0], [3.0, 4.0], [5.0, 6.0], 17).ravel(), [-24.0, -96.0])
    sp = pytest.importorskip("sympy")
    from hoexplicit.model import _term
    x, y, z = sp.symbols("x y z")
    for order, terms in ((4, range(17, 26)), (5, range(26, 37))):
        polys = []
        for t in terms:
            e = sp.expand(_term(t, x, y, z))
            P = sp.Poly(e, x, y, z)
            assert P.is_homogeneous and P.total_degree() == order, t
            assert sp.expand(sp.diff(e, x, 2) + sp.diff(e, y, 2) + sp.diff(e, z, 2)) == 0, t
            polys.append(P)
        monoms = sorted({m for P in polys for m in P.monoms()})
        A = sp.Matrix([[P.coeff_monomial(x ** m[0] * y ** m[1] * z ** m[2]) for m in monoms] for P in polys])
        assert A.rank() == 2 * order + 1
    with pytest.raises(ArgumentError):
        basisfunc_spha([0.0], [0.0], [0.0], 37)
