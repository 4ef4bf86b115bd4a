"""TEST INFRASTRUCTURE ONLY — FP64 restatement of the delay estimator and its
preprocessing (src/Synchronization/FindDelay.jl, InterpTraj.jl).

* ``kdot_stencil`` — FindDelay.jl:179-180: ``conv(kspha, [1/8 1/4 0 -1/4 -1/8]')[3:end-2,:]/dt``,
  column by column, zero outside the series.
* ``interp_traj_time`` — InterpTraj.jl:18-40: coefficient sample j at time
  ``(j-1)*dt - delTime``, Akima interpolation per column, zero outside the
  shifted interval.  The interpolant is Akima's (1970) piecewise cubic
  Hermite: slopes m_i of the knot intervals, extended past both ends by linear
  extrapolation (m_{-1} = 2m_0 - m_1, ...), knot tangents
  t_i = (|m_{i+1}-m_i| m_{i-1} + |m_{i-1}-m_{i-2}| m_i) / (|m_{i+1}-m_i| + |m_{i-1}-m_{i-2}|)
  (the mean of m_{i-1}, m_i where both weights vanish).  The reference calls
  Interpolations.jl (AkimaMonotonicInterpolation; not vendored in the
  reference tree) for this published method.
* ``find_delay`` — FindDelay.jl:139-214: alternate the weighted CGNR image
  reconstruction with the scalar update Δτ = J·Re(y2 \\ y1), y1 = data − E x,
  y2 = B x (B: the kspha_dt derivative operator), halving J after a sign
  change, until |Δτ| ≤ Δτ_min; return τ − Δτ/J·(J−1).  The density weights
  are a fixed input here (the reference recomputes them with NFFT's density
  compensation at every τ).
* ``find_delay_multishot`` — FindDelay_multishot.jl:65-158: one delay for
  several shots.  Each shot's series and its own k̇ are interpolated at its ADC
  times and delay StartTime[s] + τ; the image update uses all shots with the
  concatenated times; the per-shot residual and derivative products are built
  on the concatenated time vector, so every shot gets the first shot's ADC
  times (FindDelay_multishot.jl:111-116), as restated here.
"""
from __future__ import annotations

import numpy as np

from . import oracle as _o
from . import recon as _r

KDOT_KERNEL = np.array([1 / 8, 1 / 4, 0.0, -1 / 4, -1 / 8])


def kdot_stencil(traj, dt):
    """traj: (nField, nTerm) -> d traj/dt (nField, nTerm)."""
    traj = np.asarray(traj, dtype=np.float64)
    n = traj.shape[0]
    out = np.empty_like(traj)
    for l in range(traj.shape[1]):
        full = np.convolve(traj[:, l], KDOT_KERNEL)  # length n + 4
        out[:, l] = full[2:2 + n] / dt
    return out


def akima_tangents(x, y):
    """Knot tangents of Akima's interpolant (uniform or not)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = x.size
    m = np.diff(y) / np.diff(x)
    if n == 2:
        return np.full(2, m[0])
    mm = np.empty(n + 3)
    mm[2:n + 1] = m
    mm[1] = 2 * mm[2] - mm[3]
    mm[0] = 2 * mm[1] - mm[2]
    mm[n + 1] = 2 * mm[n] - mm[n - 1]
    mm[n + 2] = 2 * mm[n + 1] - mm[n]
    t = np.empty(n)
    for i in range(n):
        # m_{i-2}, m_{i-1}, m_i, m_{i+1} = mm[i], mm[i+1], mm[i+2], mm[i+3]
        w1 = abs(mm[i + 3] - mm[i + 2])
        w2 = abs(mm[i + 1] - mm[i])
        if w1 + w2 > 0.0:
            t[i] = (w1 * mm[i + 1] + w2 * mm[i + 2]) / (w1 + w2)
        else:
            t[i] = 0.5 * (mm[i + 1] + mm[i + 2])
    return t


def akima_eval(x, y, t, xq):
    """Cubic Hermite evaluation with tangents t; zero outside [x0, x_{n-1}]."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    xq = np.asarray(xq, dtype=np.float64)
    out = np.zeros(xq.size)
    inside = (xq >= x[0]) & (xq <= x[-1])
    q = xq[inside]
    j = np.clip(np.searchsorted(x, q, side="right") - 1, 0, x.size - 2)
    h = x[j + 1] - x[j]
    s = (q - x[j]) / h
    h00 = (1 + 2 * s) * (1 - s) ** 2
    h10 = s * (1 - s) ** 2
    h01 = s * s * (3 - 2 * s)
    h11 = s * s * (s - 1)
    out[inside] = h00 * y[j] + h10 * h * t[j] + h01 * y[j + 1] + h11 * h * t[j + 1]
    return out


def interp_traj_time(traj, dt, delTime, datatime):
    """(nField, nTerm) coefficient series -> (nData, nTerm) at ``datatime``."""
    traj = np.asarray(traj, dtype=np.float64)
    n, nTerm = traj.shape
    knots = dt * np.arange(n) - delTime
    out = np.empty((np.asarray(datatime).size, nTerm))
    for l in range(nTerm):
        out[:, l] = akima_eval(knots, traj[:, l], akima_tangents(knots, traj[:, l]), datatime)
    return out


def find_delay(bf, fieldmap, csm, data, traj, datatime, start_time, dt, *, weights=None, jump_fact=3,
               dtau_min=5e-9, iter_max=10, lam=0.0, term_mask=None, max_outer=50, nBlock=50):
    """Delay estimate τ (seconds) and its history.

    bf (nVox, nTerm) basis of the masked voxels, fieldmap (nVox,) Hz, csm
    (nVox, nCha), data (nSam*nCha,) samples fastest, traj (nField, nTerm).
    """
    traj = np.asarray(traj, dtype=np.float64)
    nTerm = traj.shape[1]
    mask = np.ones(nTerm) if term_mask is None else np.asarray(term_mask, dtype=np.float64)
    kd_full = kdot_stencil(traj, dt)
    tau, J, n_iter = 0.0, float(jump_fact), 1
    dtau_prev = dtau = np.inf
    hist = [tau]
    while abs(dtau) > dtau_min and n_iter <= max_outer:
        k_tau = interp_traj_time(traj, dt, tau + start_time, datatime).T * mask[:, None]
        kd_tau = interp_traj_time(kd_full, dt, tau + start_time, datatime).T * mask[:, None]
        m = _o.Model(bf, k_tau, datatime, fieldmap, csm, nTerm=nTerm)
        x, _ = _r.recon(m, data, weights, iter_max, 0.0, lam, nBlock)
        y1 = data - _o.forward(m, x, nBlock)
        y2 = _o.derivative(m, kd_tau, x)
        dtau = J * float(np.real(np.vdot(y2, y1) / np.vdot(y2, y2)))
        tau += dtau
        if n_iter > 1 and np.sign(dtau_prev) != np.sign(dtau):
            J = max(1.0, J / 2)
        dtau_prev = dtau
        n_iter += 1
        hist.append(tau)
    return tau - dtau / J * (J - 1), {"history": hist, "iterations": n_iter - 1, "jump": J}


def find_delay_multishot(bf, fieldmap, csm, data, traj, datatime, start_times, dt, *, weights=None, jump_fact=3,
                         dtau_min=5e-9, iter_max=10, lam=0.0, term_mask=None, max_outer=50, nBlock=50):
    """Delay estimate τ (seconds) shared by all shots, and its history.

    traj (nShot, nField, nTerm), datatime (nShot, nSPI) ADC times per shot,
    start_times (nShot,), data (nShot*nSPI*nCha,) samples fastest with the
    samples of a shot consecutive (sample j of shot s at s*nSPI + j).
    """
    traj = np.asarray(traj, dtype=np.float64)
    datatime = np.asarray(datatime, dtype=np.float64)
    start_times = np.asarray(start_times, dtype=np.float64).reshape(-1)
    nShot, _, nTerm = traj.shape
    mask = np.ones(nTerm) if term_mask is None else np.asarray(term_mask, dtype=np.float64)
    kd_full = np.stack([kdot_stencil(traj[s], dt) for s in range(nShot)])
    times = datatime.reshape(-1)
    times_res = np.tile(datatime[0], nShot)   # the per-shot operators' times

    def series(src, tau):
        return np.concatenate([interp_traj_time(src[s], dt, tau + start_times[s], datatime[s])
                               for s in range(nShot)], axis=0).T * mask[:, None]

    tau, J, n_iter = 0.0, float(jump_fact), 1
    dtau_prev = dtau = np.inf
    hist = [tau]
    while abs(dtau) > dtau_min and n_iter <= max_outer:
        k_tau, kd_tau = series(traj, tau), series(kd_full, tau)
        m = _o.Model(bf, k_tau, times, fieldmap, csm, nTerm=nTerm)
        x, _ = _r.recon(m, data, weights, iter_max, 0.0, lam, nBlock)
        mr = _o.Model(bf, k_tau, times_res, fieldmap, csm, nTerm=nTerm)
        y1 = data - _o.forward(mr, x, nBlock)
        y2 = _o.derivative(mr, kd_tau, x)
        dtau = J * float(np.real(np.vdot(y2, y1) / np.vdot(y2, y2)))
        tau += dtau
        if n_iter > 1 and np.sign(dtau_prev) != np.sign(dtau):
            J = max(1.0, J / 2)
        dtau_prev = dtau
        n_iter += 1
        hist.append(tau)
    return tau - dtau / J * (J - 1), {"history": hist, "iterations": n_iter - 1, "jump": J}
