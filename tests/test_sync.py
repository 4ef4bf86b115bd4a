"""Delay synchronisation and trajectory preprocessing (FindDelay.jl, InterpTraj.jl).

The reference's suite has no test for FindDelay or InterpTrajTime.  The
oracle's Akima interpolant is pinned to scipy's independent implementation of
the same published method, its k̇ stencil to exact derivatives; the device
kernels are compared with the oracle, the device sample-side re-plan with a
freshly built operator, and the device FindDelay with the oracle's loop on a
problem with a known delay.
"""
import numpy as np
import pytest

from oracle import oracle
from oracle import sync as osync
from oracle.dense import rel


def test_oracle_akima_matches_scipy():
    Akima = pytest.importorskip("scipy.interpolate").Akima1DInterpolator
    rng = np.random.default_rng(0)
    for n in (3, 4, 9, 50):
        x = np.arange(n) * 2e-6 - 1.3e-6
        y = np.cumsum(rng.standard_normal(n))
        q = np.linspace(x[0] - 1e-6, x[-1] + 1e-6, 301)
        a = osync.akima_eval(x, y, osync.akima_tangents(x, y), q)
        inside = (q >= x[0]) & (q <= x[-1])
        assert np.max(np.abs(a[inside] - Akima(x, y)(q[inside]))) < 1e-12
        assert np.all(a[~inside] == 0.0)  # extrapolate(itp, 0)
    # knots are interpolated exactly and straight lines are reproduced
    x = np.arange(6) * 1.0
    assert np.allclose(osync.akima_eval(x, 3 * x - 1, osync.akima_tangents(x, 3 * x - 1), x + 0.3)[:-1],
                       3 * (x + 0.3)[:-1] - 1)


def test_oracle_kdot_stencil_is_exact_for_quadratics():
    j = np.arange(40.0)
    traj = np.stack([3.0 * j, j ** 2], axis=1)
    kd = osync.kdot_stencil(traj, 2e-6)
    assert np.allclose(kd[2:-2, 0], 3.0 / 2e-6)
    assert np.allclose(kd[2:-2, 1], 2 * j[2:-2] / 2e-6)
    # zero padding at the ends, as conv(...)[3:end-2]
    assert np.isclose(kd[0, 0], (0.125 * traj[2, 0] + 0.25 * traj[1, 0]) / 2e-6)


def delay_problem(n=24, nSam=1500, nCha=2, tau_true=3.7e-6, dt=2e-6, seed=3, margin=8):
    """Spiral slice whose data were acquired with the coefficient series
    shifted by tau_true (InterpTrajTime at StartTime + tau_true)."""
    from hoexplicit import workloads
    from hoexplicit.model import basisfunc_spha
    w = workloads.spiral_slice(seed, n, nSam, nCha, d=200e-3 / n, dwell=dt)
    k9 = w.kspha[:9]
    traj = np.concatenate([k9[:, :1].repeat(margin, 1), k9, k9[:, -1:].repeat(margin, 1)], axis=1).T.copy()
    start = margin * dt
    datatime = np.arange(nSam) * dt
    g = w.grid
    bf = basisfunc_spha(g.x, g.y, g.z, list(range(1, 10)))
    fm = np.asarray(w.fieldmap).reshape(-1, order="F")
    csm = np.asarray(w.csm).reshape(n * n, nCha, order="F")
    m = oracle.Model(bf, osync.interp_traj_time(traj, dt, start + tau_true, datatime).T, datatime, fm, csm, nTerm=9)
    y = oracle.forward(m, w.x)
    rng = np.random.default_rng(1)
    y = y + 0.001 * np.linalg.norm(y) / np.sqrt(y.size) * (rng.standard_normal(y.size) + 1j * rng.standard_normal(y.size))
    return dict(w=w, traj=traj, start=start, datatime=datatime, bf=bf, fm=fm, csm=csm, y=y, dt=dt, tau=tau_true)


def test_oracle_find_delay_recovers_a_known_delay():
    P = delay_problem()
    tau, info = osync.find_delay(P["bf"], P["fm"], P["csm"], P["y"], P["traj"], P["datatime"], P["start"], P["dt"],
                                 dtau_min=5e-9, iter_max=10)
    assert abs(tau - P["tau"]) < 0.1 * P["tau"]
    assert info["iterations"] < 50


def multishot_problem(n=24, nSPI=750, nShot=2, nCha=2, tau_true=3.7e-6, dt=2e-6, seed=5, margin=8, shift=0.0):
    """A spiral slice read in nShot consecutive shots, each with its own
    coefficient series (with margins), start time and ADC times (shot s at
    dt*(0:nSPI-1) + s*shift); the data were acquired at delay tau_true."""
    from hoexplicit import workloads
    from hoexplicit.model import basisfunc_spha
    w = workloads.spiral_slice(seed, n, nSPI * nShot, nCha, d=200e-3 / n, dwell=dt)
    k9 = w.kspha[:9]
    traj = np.stack([np.concatenate([k9[:, s * nSPI:s * nSPI + 1].repeat(margin, 1), k9[:, s * nSPI:(s + 1) * nSPI],
                                     k9[:, (s + 1) * nSPI - 1:(s + 1) * nSPI].repeat(margin, 1)], axis=1).T
                     for s in range(nShot)])
    start = margin * dt + 0.25 * dt * np.arange(nShot)
    datatime = np.stack([np.arange(nSPI) * dt + s * shift for s in range(nShot)])
    g = w.grid
    bf = basisfunc_spha(g.x, g.y, g.z, list(range(1, 10)))
    fm = np.asarray(w.fieldmap).reshape(-1, order="F")
    csm = np.asarray(w.csm).reshape(n * n, nCha, order="F")
    k_true = np.concatenate([osync.interp_traj_time(traj[s], dt, start[s] + tau_true, datatime[s])
                             for s in range(nShot)], axis=0).T
    m = oracle.Model(bf, k_true, datatime.reshape(-1), fm, csm, nTerm=9)
    y = oracle.forward(m, w.x)
    rng = np.random.default_rng(2)
    y = y + 0.001 * np.linalg.norm(y) / np.sqrt(y.size) * (rng.standard_normal(y.size) + 1j * rng.standard_normal(y.size))
    return dict(w=w, traj=traj, start=start, datatime=datatime, bf=bf, fm=fm, csm=csm, y=y, dt=dt, tau=tau_true)


def test_oracle_find_delay_multishot_recovers_a_known_delay():
    P = multishot_problem()
    # the shots' increments shrink by ~6% an iteration, so this estimator
    # needs a larger Δτ_min and more iterations than the single-shot problem
    tau, info = osync.find_delay_multishot(P["bf"], P["fm"], P["csm"], P["y"], P["traj"], P["datatime"], P["start"],
                                           P["dt"], dtau_min=1e-8, iter_max=10, max_outer=100)
    assert abs(tau - P["tau"]) < 0.1 * P["tau"], tau
    assert info["iterations"] < 100


def test_oracle_find_delay_multishot_with_one_shot_is_find_delay():
    P = delay_problem()
    a = osync.find_delay(P["bf"], P["fm"], P["csm"], P["y"], P["traj"], P["datatime"], P["start"], P["dt"],
                         dtau_min=5e-9, iter_max=10)
    b = osync.find_delay_multishot(P["bf"], P["fm"], P["csm"], P["y"], P["traj"][None], P["datatime"][None],
                                   [P["start"]], P["dt"], dtau_min=5e-9, iter_max=10)
    assert a[0] == b[0] and a[1]["history"] == b[1]["history"]


# --------------------------------------------------------------------- GPU
torch = pytest.importorskip("torch")

from hoexplicit import Grid, HighOrderExplicitOp, workloads  # noqa: E402
from hoexplicit import sync as hsync  # noqa: E402
from tests.test_gpu_parity import ENGINE_PARAMS, maybe_skip  # noqa: E402


@pytest.mark.gpu
def test_device_preprocessing_matches_oracle():
    rng = np.random.default_rng(4)
    traj = np.cumsum(rng.standard_normal((700, 16)), axis=0) * 0.3
    dt = 2e-6
    assert np.max(np.abs(hsync.kspha_dt(traj, dt) - osync.kdot_stencil(traj, dt))) < 1e-9 * np.max(np.abs(traj)) / dt
    datatime = np.sort(rng.uniform(-20e-6, 1420e-6, 999))
    for delTime in (0.0, 3.7e-6, -11.3e-6):
        a = hsync.InterpTrajTime(traj, dt, delTime, datatime)
        b = osync.interp_traj_time(traj, dt, delTime, datatime)
        assert a.shape == b.shape == (999, 16)
        assert np.max(np.abs(a - b)) < 1e-11 * np.max(np.abs(traj))
        assert np.all(a[(datatime < -delTime) | (datatime > 699 * dt - delTime)] == 0)


@pytest.mark.gpu
@pytest.mark.parametrize("engine", ENGINE_PARAMS)
def test_set_kspha_matches_a_new_operator(engine):
    maybe_skip(engine)
    w = workloads.config1()
    w2 = workloads.config1(seed=2001)  # another trajectory of the same shape
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine=engine, **w.op_kwargs())
    hsync.set_kspha(op, w2.kspha, w2.kspha_dt)
    ref = HighOrderExplicitOp(w.grid, w2.kspha, w.times, engine=engine, **w.op_kwargs())
    x = torch.from_numpy(w.x.astype(np.complex64)).cuda()
    tol = 1e-5 if engine == "fp32" else 1e-4
    bf, k, t, f, c, idx = workloads.prepared_model(w)
    _, k2, _, _, _, _ = workloads.prepared_model(w2)
    m2 = oracle.Model(bf, k2, t, f, c)
    yo = oracle.forward(m2, w.x[idx])
    ya = (op * x).cpu().numpy()
    assert rel(ya, yo) < tol
    assert rel(ya, (ref * x).cpu().numpy()) < 2 * tol
    xo = oracle.adjoint(m2, yo)
    xa = (op.H * torch.from_numpy(yo.astype(np.complex64)).cuda()).cpu().numpy()
    assert rel(xa[idx], xo) < tol
    # derivative mode uses the new kspha_dt
    from hoexplicit import _lib
    yd = torch.empty(op.nrow, dtype=torch.complex64, device="cuda")
    _lib.check(_lib.load().hoe_derivative(op._handle(), x.data_ptr(), yd.data_ptr(), op._stream()), op._h)
    assert rel(yd.cpu().numpy(), oracle.derivative(m2, w2.kspha_dt, w.x[idx])) < tol
    op.check()
    op.close()
    ref.close()


@pytest.mark.gpu
@pytest.mark.parametrize("engine", ENGINE_PARAMS)
def test_find_delay_matches_oracle(engine):
    maybe_skip(engine)
    P = delay_problem()
    n, nCha = P["w"].grid.nX, P["csm"].shape[1]
    data = P["y"].reshape(nCha, -1).T
    tau, info = hsync.FindDelay(P["w"].grid, data.astype(np.complex64), P["traj"], P["datatime"], P["start"], P["dt"],
                                dtau_min=5e-9, fieldmap=P["fm"].reshape(n, n, order="F"),
                                csm=P["csm"].reshape(n, n, nCha, order="F"), recon_terms="111", iter_max=10,
                                engine=engine, return_info=True)
    to, oinfo = osync.find_delay(P["bf"], P["fm"], P["csm"], P["y"], P["traj"], P["datatime"], P["start"], P["dt"],
                                 dtau_min=5e-9, iter_max=10)
    assert info["status"] == "converged"
    # The loop stops once one increment falls under dtau_min while still
    # creeping towards its fixed point (a few ns per update), so arithmetic
    # that differs slightly (the split-BF16 engine) stops a little earlier or later.
    assert abs(tau - to) < (0.02 if engine == "fp32" else 0.05) * P["tau"], (tau, to)
    assert abs(tau - P["tau"]) < 0.1 * P["tau"]
    assert info["image"].shape == (n, n, 1)


def _multishot_device(P, engine, **kw):
    n, nCha = P["w"].grid.nX, P["csm"].shape[1]
    data = P["y"].reshape(nCha, -1).T
    return hsync.FindDelay_multishot(P["w"].grid, data.astype(np.complex64), P["traj"], P["datatime"], P["start"],
                                     P["dt"], dtau_min=1e-8, fieldmap=P["fm"].reshape(n, n, order="F"),
                                     csm=P["csm"].reshape(n, n, nCha, order="F"), recon_terms="111", iter_max=10,
                                     max_outer=100, engine=engine, return_info=True, **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("engine", ENGINE_PARAMS)
def test_find_delay_multishot_matches_oracle(engine):
    maybe_skip(engine)
    P = multishot_problem()
    tau, info = _multishot_device(P, engine)
    to, _ = osync.find_delay_multishot(P["bf"], P["fm"], P["csm"], P["y"], P["traj"], P["datatime"], P["start"],
                                       P["dt"], dtau_min=1e-8, iter_max=10, max_outer=100)
    assert info["status"] == "converged" and not info["resid_operator"]
    assert abs(tau - to) < (0.02 if engine == "fp32" else 0.05) * P["tau"], (tau, to)
    assert abs(tau - P["tau"]) < 0.1 * P["tau"]
    assert info["image"].shape == (P["w"].grid.nX, P["w"].grid.nY, 1)


@pytest.mark.gpu
@pytest.mark.parametrize("engine", ENGINE_PARAMS)
def test_find_delay_multishot_residuals_on_the_first_shots_times(engine):
    """Shot 2 acquired 6 us later than shot 1 with a fieldmap: the image update
    uses each shot's times, the residual and derivative products the first
    shot's (an operator on those times), as in the reference."""
    maybe_skip(engine)
    P = multishot_problem(shift=6e-6)
    tau, info = _multishot_device(P, engine)
    to, _ = osync.find_delay_multishot(P["bf"], P["fm"], P["csm"], P["y"], P["traj"], P["datatime"], P["start"],
                                       P["dt"], dtau_min=1e-8, iter_max=10, max_outer=100)
    assert info["resid_operator"] and info["status"] == "converged"
    assert abs(tau - to) < (0.02 if engine == "fp32" else 0.05) * P["tau"], (tau, to)


@pytest.mark.gpu
def test_find_delay_multishot_with_one_shot_is_find_delay():
    P = delay_problem()
    n, nCha = P["w"].grid.nX, P["csm"].shape[1]
    data = (P["y"].reshape(nCha, -1).T).astype(np.complex64)
    kw = dict(dtau_min=5e-9, fieldmap=P["fm"].reshape(n, n, order="F"), csm=P["csm"].reshape(n, n, nCha, order="F"),
              recon_terms="111", iter_max=10, engine="fp32", return_info=True)
    a, ia = hsync.FindDelay(P["w"].grid, data, P["traj"], P["datatime"], P["start"], P["dt"], **kw)
    b, ib = hsync.FindDelay_multishot(P["w"].grid, data, P["traj"][None], P["datatime"][None], [P["start"]], P["dt"],
                                      **kw)
    assert a == b and ia["iterations"] == ib["iterations"]
    np.testing.assert_array_equal(ia["image"], ib["image"])


def test_find_delay_multishot_argument_checks():
    from hoexplicit import ArgumentError, DimensionMismatch
    P = multishot_problem(nSPI=100)
    n, nCha = P["w"].grid.nX, P["csm"].shape[1]
    data = np.zeros((200, nCha), np.complex64)
    with pytest.raises(DimensionMismatch):
        hsync.FindDelay_multishot(P["w"].grid, data, P["traj"], P["datatime"][:1], P["start"], P["dt"])
    with pytest.raises(DimensionMismatch):
        hsync.FindDelay_multishot(P["w"].grid, data[:150], P["traj"], P["datatime"], P["start"], P["dt"])
    with pytest.raises(DimensionMismatch):
        hsync.FindDelay_multishot(P["w"].grid, data, P["traj"], P["datatime"], P["start"][:1], P["dt"])
    with pytest.raises(DimensionMismatch):
        hsync.FindDelay_multishot(P["w"].grid, data, P["traj"][0], P["datatime"], P["start"], P["dt"])
    with pytest.raises(ArgumentError):
        hsync.FindDelay_multishot(P["w"].grid, data, P["traj"], P["datatime"], P["start"], P["dt"], recon_terms="11")


@pytest.mark.gpu
def test_interp_traj_time_per_shot_overload():
    """InterpTrajTime of a (nShot, nField, nTerm) series: each shot with its own
    delay and ADC times (InterpTraj.jl:79-99), against the oracle per shot."""
    rng = np.random.default_rng(4)
    traj = np.cumsum(rng.standard_normal((3, 60, 4)), axis=1)
    dt = 2e-6
    delTime = np.array([3e-6, 7.5e-6, -1e-6])
    datatime = np.stack([np.arange(50) * dt + s * 0.3e-6 for s in range(3)])
    out = hsync.InterpTrajTime(traj, dt, delTime, datatime)
    assert out.shape == (3, 50, 4)
    for s in range(3):
        ref = osync.interp_traj_time(traj[s], dt, delTime[s], datatime[s])
        assert np.max(np.abs(out[s] - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_interp_traj_time_per_shot_argument_checks():
    from hoexplicit import ArgumentError, DimensionMismatch
    traj = np.zeros((2, 10, 3))
    with pytest.raises(DimensionMismatch):
        hsync.InterpTrajTime(traj, 1e-6, np.zeros(3), np.zeros((2, 5)))
    with pytest.raises(DimensionMismatch):
        hsync.InterpTrajTime(traj, 1e-6, np.zeros(2), np.zeros((3, 5)))
    with pytest.raises(ArgumentError):
        hsync.InterpTrajTime(traj, 1e-6, np.zeros(2))
