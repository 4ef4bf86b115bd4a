"""Seeded synthetic workloads with the shapes and value distributions of the
five benchmark configurations (no public dataset is involved; the reference's
demo data are not used).

Each generator returns a ``Workload`` with host numpy arrays in the reference
layouts: ``kspha`` (nTerm, nSam) in cycles/m^p, ``times`` (nSam,) s,
``fieldmap``/``mask`` (nX, nY[, nZ]), ``csm`` (nX, nY[, nZ], nCha), image ``x``
flattened in Fortran order, optional ``concomitant`` (4, nSam) cycles/m^2.
Seeds are ``numpy.random.default_rng(1000 + config)``.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .model import Grid, basisfunc_spha

GAMMA = 42.577478e6  # Hz/T


@dataclass
class Workload:
    name: str
    grid: Grid
    kspha: np.ndarray
    times: np.ndarray
    fieldmap: np.ndarray
    csm: np.ndarray
    mask: np.ndarray
    x: np.ndarray
    concomitant: np.ndarray | None = None
    kspha_dt: np.ndarray | None = None
    dwell: float = 1e-6

    @property
    def nSam(self):
        return self.kspha.shape[1]

    @property
    def nCha(self):
        return self.csm.shape[-1]

    @property
    def nVox(self):
        return int(np.count_nonzero(self.mask))

    def op_kwargs(self):
        kw = dict(fieldmap=self.fieldmap, csm=self.csm, mask=self.mask)
        if self.concomitant is not None:
            kw["concomitant"] = self.concomitant
        return kw


def _smooth_poly(rng, t, degree=5):
    """Smooth random polynomial in normalised time, unit peak."""
    u = (t - t.min()) / max(t.max() - t.min(), 1e-30)
    c = rng.standard_normal(degree + 1)
    p = np.polynomial.polynomial.polyval(u, c)
    return p / max(np.max(np.abs(p)), 1e-30)


def _ellipse_phantom(rng, grid: Grid, n_ell=8):
    x = grid.x / max(np.max(np.abs(grid.x)), 1e-30)
    y = grid.y / max(np.max(np.abs(grid.y)), 1e-30)
    img = np.zeros(x.size, dtype=np.complex128)
    img[(x / 0.85) ** 2 + (y / 0.95) ** 2 <= 1] = 1.0
    for _ in range(n_ell):
        cx, cy = rng.uniform(-0.5, 0.5, 2)
        ax, ay = rng.uniform(0.08, 0.35, 2)
        th = rng.uniform(0, np.pi)
        xr = (x - cx) * np.cos(th) + (y - cy) * np.sin(th)
        yr = -(x - cx) * np.sin(th) + (y - cy) * np.cos(th)
        val = rng.uniform(-0.4, 0.6) * np.exp(1j * rng.uniform(-np.pi, np.pi))
        img[(xr / ax) ** 2 + (yr / ay) ** 2 <= 1] += val
    return img


def _gauss_fieldmap(rng, grid: Grid, n=3, peak=50.0):
    x = grid.x / max(np.max(np.abs(grid.x)), 1e-30)
    y = grid.y / max(np.max(np.abs(grid.y)), 1e-30)
    f = np.zeros(x.size)
    for _ in range(n):
        cx, cy = rng.uniform(-0.6, 0.6, 2)
        w = rng.uniform(0.15, 0.5)
        f += rng.uniform(-1, 1) * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * w * w))
    return f / max(np.max(np.abs(f)), 1e-30) * peak


def _ring_coils(rng, grid: Grid, nCha, fov):
    x, y = grid.x, grid.y
    R = 0.6 * fov / 2
    sig = 0.35 * fov
    coils = np.empty((x.size, nCha), dtype=np.complex128)
    for c in range(nCha):
        a = 2 * np.pi * c / nCha
        cx, cy = R * np.cos(a), R * np.sin(a)
        mag = np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * sig * sig))
        ph = rng.uniform(-np.pi, np.pi) + 2 * np.pi * 0.5 * (x * np.cos(a) + y * np.sin(a)) / fov
        coils[:, c] = mag * np.exp(1j * ph)
    return coils


def _higher_orders(rng, grid: Grid, mask_flat, kspha, t, linear_peak, frac=0.5, orders=(0, 2, 3)):
    """Fill zeroth/second/third-order rows with smooth polynomials scaled so
    that max |k_l(t) b_l(r)| = frac * linear_peak (cycles)."""
    nTerm = kspha.shape[0]
    idx = np.flatnonzero(mask_flat)
    bf = basisfunc_spha(grid.x[idx], grid.y[idx], grid.z[idx], list(range(1, nTerm + 1)))
    rows = []
    if 0 in orders:
        rows += [0]
    if 2 in orders:
        rows += list(range(4, 9))
    if 3 in orders and nTerm == 16:
        rows += list(range(9, 16))
    for l in rows:
        bmax = np.max(np.abs(bf[:, l]))
        if bmax <= 0:
            continue
        kspha[l] = _smooth_poly(rng, t) * (frac * linear_peak / bmax)
    return kspha


def config1(seed: int = 1001) -> Workload:
    """64x64, 3.125 mm, single-shot Archimedean spiral, 4096 samples, 2 us
    dwell, kmax = 160 cycles/m; 16 terms; +-50 Hz fieldmap; 8 ring coils."""
    rng = np.random.default_rng(seed)
    n, d, nSam, dwell, nCha = 64, 3.125e-3, 4096, 2e-6, 8
    grid = Grid(n, n, 1, d, d, d)
    fov = n * d
    kmax = 1.0 / (2 * d)
    t = np.arange(nSam) * dwell
    u = np.arange(nSam) / (nSam - 1)
    turns = fov * kmax / 2
    k = kmax * u * np.exp(2j * np.pi * turns * u)
    kspha = np.zeros((16, nSam))
    kspha[1], kspha[2] = k.real, k.imag
    mask = np.ones(n * n, dtype=bool)
    lin_peak = kmax * np.max(np.hypot(grid.x, grid.y))
    _higher_orders(rng, grid, mask, kspha, t, lin_peak)
    fm = _gauss_fieldmap(rng, grid, 3, 50.0)
    csm = _ring_coils(rng, grid, nCha, fov)
    x = _ellipse_phantom(rng, grid)
    return Workload("cfg1-spiral-64x64-4096s-8c-16t", grid, kspha, t,
                    fm.reshape(n, n, order="F"), csm.reshape(n, n, nCha, order="F"),
                    mask.reshape(n, n, order="F"), x, dwell=dwell,
                    kspha_dt=np.gradient(kspha, dwell, axis=1))


def _svd_compress(csm, n_out):
    """Global SVD coil compression of coil maps (nVox, nIn) -> (nVox, n_out)."""
    u, s, vh = np.linalg.svd(csm, full_matrices=False)
    return csm @ vh.conj().T[:, :n_out]


def config2(seed: int = 1002, n: int = 200, interleaves: int = 4, per: int = 3000,
            coils_in: int = 32, coils_out: int = 16, z_offset: float = 0.015) -> Workload:
    """200x200, 1 mm, variable-density spiral R=4 (4 x 3000 samples, 1 us),
    32 coils compressed to 16; 16 terms + 4 concomitant terms at 7 T;
    +-100 Hz smooth fieldmap."""
    rng = np.random.default_rng(seed)
    d, dwell = 1e-3, 1e-6
    grid = Grid(n, n, 1, d, d, d)
    grid.z = np.full(grid.x.size, z_offset)  # slice offset so z-dependent terms act
    fov = n * d
    kmax = 1.0 / (2 * d)
    R = 4
    turns = fov * kmax / (interleaves * R)
    u = np.arange(per) / (per - 1)
    rad = kmax * u ** 1.4
    ang = 2 * np.pi * turns * u ** 0.8
    ks, ts = [], []
    for i in range(interleaves):
        ks.append(rad * np.exp(1j * (ang + 2 * np.pi * i / interleaves)))
        ts.append(np.arange(per) * dwell)
    k = np.concatenate(ks)
    t = np.concatenate(ts)
    nSam = k.size
    kspha = np.zeros((16, nSam))
    kspha[1], kspha[2] = k.real, k.imag
    mask = np.ones(n * n, dtype=bool)
    lin_peak = kmax * np.max(np.hypot(grid.x, grid.y))
    _higher_orders(rng, grid, mask, kspha, t, lin_peak)
    # Maxwell (concomitant) coefficient for z^2 from the in-plane gradients at B0 = 7 T
    B0 = 7.0
    conc = np.zeros((4, nSam))
    for i in range(interleaves):
        sl = slice(i * per, (i + 1) * per)
        gx = np.gradient(kspha[1, sl], dwell) / GAMMA
        gy = np.gradient(kspha[2, sl], dwell) / GAMMA
        conc[0, sl] = np.cumsum(GAMMA * (gx ** 2 + gy ** 2) / (2 * B0)) * dwell
    fm = _gauss_fieldmap(rng, grid, 4, 100.0)
    csm = _svd_compress(_ring_coils(rng, grid, coils_in, fov), coils_out)
    csm /= np.max(np.sqrt(np.sum(np.abs(csm) ** 2, axis=1)))
    x = _ellipse_phantom(rng, grid)
    return Workload(f"cfg2-vdspiral-{n}x{n}-{nSam}s-{coils_out}c-16t+conc", grid, kspha, t,
                    fm.reshape(n, n, order="F"), csm.reshape(n, n, coils_out, order="F"),
                    mask.reshape(n, n, order="F"), x, concomitant=conc, dwell=dwell,
                    kspha_dt=np.gradient(kspha, dwell, axis=1))


def config3(seed: int = 1003, n: int = 200, lines: int = 50, per_line: int = 200,
            ramp: int = 20, nCha: int = 16) -> Workload:
    """200x200 single-shot blipped EPI, R=4 (50 lines x 200 samples plus ramp
    samples, 12,000 total, 2.5 us dwell); eddy-current-like exponential terms
    (tau 0.1-2 ms, <= 5% of the gradient) on every coefficient."""
    rng = np.random.default_rng(seed)
    d, dwell = 1e-3, 2.5e-6
    grid = Grid(n, n, 1, d, d, d)
    fov = n * d
    kmax = 1.0 / (2 * d)
    dk = 4.0 / fov
    kx, ky = [], []
    for ln in range(lines):
        sgn = 1 if ln % 2 == 0 else -1
        ramp_up = np.linspace(0, 1, ramp, endpoint=False) ** 2
        flat = np.linspace(-kmax, kmax, per_line)
        line = np.concatenate([-kmax - (1 - ramp_up) * 0, flat, kmax + ramp_up[::-1] * 0])[: per_line + 2 * ramp]
        kx.append(sgn * line)
        ky.append(np.full(line.size, -kmax + (ln + 0.5) * dk * (2 * kmax / (lines * dk))))
    kx = np.concatenate(kx)
    ky = np.concatenate(ky)
    nSam = kx.size
    t = np.arange(nSam) * dwell
    kspha = np.zeros((16, nSam))
    kspha[1], kspha[2] = kx, ky
    g = np.gradient(kx, dwell)
    for l in range(16):
        acc = np.zeros(nSam)
        for _ in range(2):
            tau = rng.uniform(1e-4, 2e-3)
            a = rng.uniform(-0.05, 0.05)
            h = np.exp(-np.arange(nSam) * dwell / tau)
            acc += a * np.convolve(g, h)[:nSam] * dwell / tau
        scale = 1.0 if l in (1, 2, 3) else (1.0 / (fov / 2)) ** (0 if l == 0 else (2 if l < 9 else 3)) * (fov / 2)
        kspha[l] += np.cumsum(acc) * dwell * scale / max(1, nSam * dwell / 1e-3)
    mask = np.ones(n * n, dtype=bool)
    fm = _gauss_fieldmap(rng, grid, 4, 100.0)
    csm = _ring_coils(rng, grid, nCha, fov)
    x = _ellipse_phantom(rng, grid)
    return Workload(f"cfg3-epi-{n}x{n}-{nSam}s-{nCha}c-16t", grid, kspha, t,
                    fm.reshape(n, n, order="F"), csm.reshape(n, n, nCha, order="F"),
                    mask.reshape(n, n, order="F"), x, dwell=dwell,
                    kspha_dt=np.gradient(kspha, dwell, axis=1))


def spiral_slice(seed, n: int, nSam: int, nCha: int = 16, d: float = 1e-3, dwell: float = 2e-6,
                 name: str = "slice") -> Workload:
    """One slice seeded as the 64x64 spiral workload, scaled to an n x n grid
    at spacing d: single-shot Archimedean spiral of nSam samples to
    kmax = 1/(2d), zeroth/second/third-order terms, +-50 Hz fieldmap, ring coils."""
    rng = np.random.default_rng(seed)
    grid = Grid(n, n, 1, d, d, d)
    fov = n * d
    kmax = 1.0 / (2 * d)
    t = np.arange(nSam) * dwell
    u = np.arange(nSam) / (nSam - 1)
    turns = fov * kmax / 2
    k = kmax * u * np.exp(2j * np.pi * turns * u)
    kspha = np.zeros((16, nSam))
    kspha[1], kspha[2] = k.real, k.imag
    mask = np.ones(n * n, dtype=bool)
    lin_peak = kmax * np.max(np.hypot(grid.x, grid.y))
    _higher_orders(rng, grid, mask, kspha, t, lin_peak)
    fm = _gauss_fieldmap(rng, grid, 3, 50.0)
    csm = _ring_coils(rng, grid, nCha, fov)
    x = _ellipse_phantom(rng, grid)
    return Workload(f"{name}-{n}x{n}-{nSam}s-{nCha}c-16t", grid, kspha, t,
                    fm.reshape(n, n, order="F"), csm.reshape(n, n, nCha, order="F"),
                    mask.reshape(n, n, order="F"), x, dwell=dwell,
                    kspha_dt=np.gradient(kspha, dwell, axis=1))


def volume3d(seed: int = 1006, shape=(64, 64, 32), d: float = 3.125e-3, parts: int = 8,
             per: int = 1024, nCha: int = 8, frac: float = 0.5, df_peak: float = 300.0,
             dwell: float = 2e-6) -> Workload:
    """3-D volume (default 64x64x32 at 3.125 mm) read by a stack of spirals:
    ``parts`` kz partitions (R = nZ/parts along z) of ``per`` samples each.
    Zeroth/second/third-order coefficients are smooth polynomials scaled to
    ``frac`` x the peak linear phase (as in the 64x64 spiral workload, whose
    factor is 0.5); the fieldmap is a sum of 3-D Gaussians scaled to
    +-``df_peak`` Hz; ring coils.  A large volume with strong higher orders
    is the shape with the largest phase per (sample, voxel) pair."""
    rng = np.random.default_rng(seed)
    nX, nY, nZ = shape
    grid = Grid(nX, nY, nZ, d, d, d)
    fovx, fovz = nX * d, nZ * d
    kmax = 1.0 / (2 * d)
    u = np.arange(per) / (per - 1)
    turns = fovx * kmax / 2
    kxy, kz, t = [], [], []
    for pz in range(parts):
        kxy.append(kmax * u * np.exp(1j * (2 * np.pi * turns * u + 2 * np.pi * pz / parts)))
        kz.append(np.full(per, (pz - parts / 2 + 0.5) * 2 * kmax / parts))
        t.append(np.arange(per) * dwell)
    kxy = np.concatenate(kxy)
    kspha = np.zeros((16, kxy.size))
    kspha[1], kspha[2], kspha[3] = kxy.real, kxy.imag, np.concatenate(kz)
    t = np.concatenate(t)
    mask = np.ones(nX * nY * nZ, dtype=bool)
    lin_peak = kmax * np.max(np.sqrt(grid.x ** 2 + grid.y ** 2 + grid.z ** 2))
    _higher_orders(rng, grid, mask, kspha, t, lin_peak, frac=frac)
    xs = grid.x / max(np.max(np.abs(grid.x)), 1e-30)
    ys = grid.y / max(np.max(np.abs(grid.y)), 1e-30)
    zs = grid.z / max(np.max(np.abs(grid.z)), 1e-30)
    fm = np.zeros(xs.size)
    for _ in range(4):
        cx, cy, cz = rng.uniform(-0.6, 0.6, 3)
        wd = rng.uniform(0.2, 0.5)
        fm += rng.uniform(-1, 1) * np.exp(-((xs - cx) ** 2 + (ys - cy) ** 2 + (zs - cz) ** 2) / (2 * wd * wd))
    fm *= df_peak / max(np.max(np.abs(fm)), 1e-30)
    csm = _ring_coils(rng, grid, nCha, fovx)
    x = _ellipse_phantom(rng, grid) * (np.abs(zs) <= 0.9)
    sh = (nX, nY, nZ)
    return Workload(f"vol3d-{nX}x{nY}x{nZ}-{kxy.size}s-{nCha}c-16t-f{frac:g}", grid, kspha, t,
                    fm.reshape(sh, order="F"), csm.reshape(sh + (nCha,), order="F"),
                    mask.reshape(sh, order="F"), x, dwell=dwell,
                    kspha_dt=np.gradient(kspha, dwell, axis=1))


def config5(seed: int = 1005, slices: int = 24, nCha: int = 16):
    """24 slices of 160^2-224^2 voxels (steps of 8) with 8,000-20,000 samples
    each (uneven), 16 coils: a list of Workloads."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(20, 29, slices) * 8
    nsams = rng.integers(8000, 20001, slices)
    return [spiral_slice(seed * 100 + i, int(sizes[i]), int(nsams[i]), nCha, name=f"cfg5-s{i:02d}")
            for i in range(slices)]


def small(seed: int = 7, shape=(9, 7, 1), nSam=300, nCha=3, nTerm=16, conc=False,
          masked=True) -> Workload:
    """Small random problem for parity tests at odd (non tile-multiple) sizes."""
    rng = np.random.default_rng(seed)
    nX, nY, nZ = shape
    grid = Grid(nX, nY, nZ, 0.011, 0.013, 0.017)
    nFull = nX * nY * nZ
    dwell = 4e-6
    t = 1e-3 + np.arange(nSam) * dwell
    u = np.arange(nSam) / max(nSam - 1, 1)
    kspha = np.zeros((nTerm, nSam))
    kspha[0] = 0.3 * np.sin(3 * u)
    kspha[1] = 40 * u * np.cos(9 * u)
    kspha[2] = 40 * u * np.sin(9 * u)
    kspha[3] = 10 * u
    for l in range(4, nTerm):
        kspha[l] = rng.standard_normal() * 300 * (1 + u) * np.cos((l + 1) * u)
    mask = np.ones(nFull, dtype=bool)
    if masked:
        mask[0] = False
        mask[nFull - 2] = False
    fm = rng.uniform(-40, 40, nFull)
    csm = (rng.standard_normal((nFull, nCha)) + 1j * rng.standard_normal((nFull, nCha)))
    x = rng.standard_normal(nFull) + 1j * rng.standard_normal(nFull)
    conc_arr = rng.standard_normal((4, nSam)) * 5.0 if conc else None
    sh = (nX, nY, nZ)
    return Workload(f"small-{nX}x{nY}x{nZ}-{nSam}s-{nCha}c-{nTerm}t", grid, kspha, t,
                    fm.reshape(sh, order="F"), csm.reshape(sh + (nCha,), order="F"),
                    mask.reshape(sh, order="F"), x, concomitant=conc_arr, dwell=dwell,
                    kspha_dt=np.gradient(kspha, dwell, axis=1) if nSam > 1 else np.zeros_like(kspha))


def prepared_model(w: Workload, derivative=False):
    """Masked FP64 model arrays (bf, kspha, times, fieldmap, csm) as the
    operator prepares them; used to drive the oracle on identical inputs."""
    from .model import prep_concomitant, prep_kspha
    mask = np.asarray(w.mask).reshape(-1, order="F").astype(bool)
    idx = np.flatnonzero(mask)
    nTerm = w.kspha.shape[0]
    k = prep_kspha(w.kspha, w.kspha[1:4], nTerm)
    g = w.grid
    bf = basisfunc_spha(g.x[idx], g.y[idx], g.z[idx], list(range(1, nTerm + 1)))
    bf, k = prep_concomitant(bf, k, g.x[idx], g.y[idx], g.z[idx],
                             None if derivative else w.concomitant)
    fm = np.asarray(w.fieldmap).reshape(-1, order="F")[idx]
    nCha = w.csm.shape[-1]
    csm = np.asarray(w.csm).reshape(-1, nCha, order="F")[idx]
    return bf, k, np.asarray(w.times, dtype=np.float64), fm, csm, idx
