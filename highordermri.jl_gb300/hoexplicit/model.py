"""Host-side model preparation: grid, solid-harmonic basis, order selection,
concomitant terms.  These run once per operator on the host, as in the
reference (array_operator.jl:121-139; explicit_gpu_operator.jl:355-360).

Arrays follow the reference's Julia conventions.  Spatial arrays are shaped
``(nX, nY, nZ)`` (or ``(nX, nY)`` when nZ == 1) and flattened in Fortran order
(x fastest); ``kspha`` is ``(nTerm, nSam)``; ``csm`` is ``(nX, nY[, nZ], nCha)``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from ._lib import ArgumentError, DimensionMismatch


@dataclass
class Grid:
    """Centred Cartesian grid (src/Grid/Grid.jl:18-30, constructor :65-96).

    ``r[j] = (j - (N+1)/2) * delta`` for 1-based j, x index fastest in the
    flattened coordinate vectors, metres.  As in the reference constructor,
    ``exchange_xy`` swaps the x and y coordinate vectors and each
    ``reverse_*`` reverses one flattened coordinate vector (Grid.jl:83-94);
    neither permutes image, mask, field-map or coil arrays.  They apply only
    when the coordinates are generated, not to explicit ``x``/``y``/``z``.
    """

    nX: int
    nY: int
    nZ: int
    dx: float = 1.0
    dy: float = 1.0
    dz: float = 1.0
    x: np.ndarray = field(default=None, repr=False)
    y: np.ndarray = field(default=None, repr=False)
    z: np.ndarray = field(default=None, repr=False)
    exchange_xy: bool = field(default=False, repr=False)
    reverse_x: bool = field(default=False, repr=False)
    reverse_y: bool = field(default=False, repr=False)
    reverse_z: bool = field(default=False, repr=False)

    def __post_init__(self):
        if self.x is None:
            i = np.arange(1, self.nX + 1, dtype=np.float64)
            j = np.arange(1, self.nY + 1, dtype=np.float64)
            k = np.arange(1, self.nZ + 1, dtype=np.float64)
            ii = np.tile(i, self.nY * self.nZ)
            jj = np.tile(np.repeat(j, self.nX), self.nZ)
            kk = np.repeat(k, self.nX * self.nY)
            x = (ii - (self.nX + 1) / 2.0) * self.dx
            y = (jj - (self.nY + 1) / 2.0) * self.dy
            z = (kk - (self.nZ + 1) / 2.0) * self.dz
            if self.exchange_xy:
                x, y = y, x
            self.x = x[::-1].copy() if self.reverse_x else x
            self.y = y[::-1].copy() if self.reverse_y else y
            self.z = z[::-1].copy() if self.reverse_z else z

    @property
    def matrixSize(self):
        return (self.nX, self.nY, self.nZ)

    @property
    def resolution(self):
        return (self.dx, self.dy, self.dz)

    def struct_to_dict(self):
        """Dictionary form of Grid.jl:98-111."""
        return {"schema_version": 1, "nX": self.nX, "nY": self.nY, "nZ": self.nZ,
                "delta_x": self.dx, "delta_y": self.dy, "delta_z": self.dz,
                "x": np.asarray(self.x), "y": np.asarray(self.y), "z": np.asarray(self.z),
                "matrix_size": [self.nX, self.nY, self.nZ],
                "resolution": [self.dx, self.dy, self.dz]}

    @classmethod
    def from_dict(cls, d):
        """Restore from ``struct_to_dict`` output (Grid.jl:126-152)."""
        s = lambda v: np.asarray(v).reshape(-1)[0].item() if np.ndim(v) else v
        return cls(int(s(d["nX"])), int(s(d["nY"])), int(s(d["nZ"])), float(s(d["delta_x"])),
                   float(s(d["delta_y"])), float(s(d["delta_z"])),
                   x=np.asarray(d["x"], dtype=np.float64).ravel(),
                   y=np.asarray(d["y"], dtype=np.float64).ravel(),
                   z=np.asarray(d["z"], dtype=np.float64).ravel())


def _term(t: int, x, y, z):
    r2 = x * x + y * y + z * z
    if t == 1:
        return np.ones_like(x)
    if t == 2:
        return x.copy()
    if t == 3:
        return y.copy()
    if t == 4:
        return z.copy()
    if t == 5:
        return x * y
    if t == 6:
        return z * y
    if t == 7:
        return 3 * z ** 2 - r2
    if t == 8:
        return x * z
    if t == 9:
        return x ** 2 - y ** 2
    if t == 10:
        return 3 * y * x ** 2 - y ** 3
    if t == 11:
        return x * z * y
    if t == 12:
        return (5 * z ** 2 - r2) * y
    if t == 13:
        return 5 * z ** 3 - 3 * z * r2
    if t == 14:
        return (5 * z ** 2 - r2) * x
    if t == 15:
        return x ** 2 * z - y ** 2 * z
    if t == 16:
        return x ** 3 - 3 * x * y ** 2
    if 17 <= t <= 36:
        return _HIGHER[t](x, y, z, r2)
    raise ArgumentError("Basis function undefined.")


# Fourth- (terms 17-25) and fifth-order (26-36) solid harmonics of
# basisfunction.jl:79-118 (the explicit operator itself uses terms 1-16).
_HIGHER = {
    17: lambda x, y, z, r2: x * y * (x ** 2 - y ** 2),
    18: lambda x, y, z, r2: y * z * (3 * x ** 2 - y ** 2),
    19: lambda x, y, z, r2: x * y * (7 * z ** 2 - r2),
    20: lambda x, y, z, r2: y * (7 * z ** 3 - 3 * z * r2),
    21: lambda x, y, z, r2: 35 * z ** 4 - 30 * z ** 2 * r2 + 3 * r2 ** 2,
    22: lambda x, y, z, r2: x * (7 * z ** 3 - 3 * z * r2),
    23: lambda x, y, z, r2: (x ** 2 - y ** 2) * (7 * z ** 2 - r2),
    24: lambda x, y, z, r2: x * (x ** 2 - 3 * y ** 2) * z,
    25: lambda x, y, z, r2: x ** 2 * (x ** 2 - 3 * y ** 2) - y ** 2 * (3 * x ** 2 - y ** 2),
    26: lambda x, y, z, r2: y * (5 * x ** 4 - 10 * x ** 2 * y ** 2 + y ** 4),
    27: lambda x, y, z, r2: x * y * z * (x ** 2 - y ** 2),
    28: lambda x, y, z, r2: y * (r2 - 9 * z ** 2) * (y ** 2 - 3 * x ** 2),
    29: lambda x, y, z, r2: x * y * z * (3 * z ** 2 - r2),
    30: lambda x, y, z, r2: y * (r2 ** 2 - 14 * r2 * z ** 2 + 21 * z ** 4),
    31: lambda x, y, z, r2: 63 * z ** 5 - 70 * z ** 3 * r2 + 15 * z * r2 ** 2,
    32: lambda x, y, z, r2: x * (r2 ** 2 - 14 * r2 * z ** 2 + 21 * z ** 4),
    33: lambda x, y, z, r2: z * (3 * z ** 2 - r2) * (x ** 2 - y ** 2),
    34: lambda x, y, z, r2: x * (r2 - 9 * z ** 2) * (3 * y ** 2 - x ** 2),
    35: lambda x, y, z, r2: z * (x ** 4 - 6 * x ** 2 * y ** 2 + y ** 4),
    36: lambda x, y, z, r2: x ** 5 - 10 * x ** 3 * y ** 2 + 5 * x * y ** 4,
}


def basisfunc_spha(x, y, z, terms):
    """Unnormalised real solid harmonics (basisfunction.jl:27-126), terms 1-36
    (orders 0-5; the explicit operator uses 1-9 or 1-16).

    Returns ``(len(x), len(terms))``, columns in the requested order.
    """
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    z = np.asarray(z, dtype=np.float64)
    if np.isscalar(terms):
        return _term(int(terms), x, y, z)
    out = np.empty((x.size, len(terms)), dtype=np.float64, order="F")
    for i, t in enumerate(terms):
        out[:, i] = _term(int(t), x, y, z)
    return out


def prep_kspha(kspha, k_nominal, nTerm: int, recon_terms=None):
    """Order selection of prep_kspha.jl:1-56; returns a modified copy.

    A '0' digit zeroes its order, except first order, whose rows 2:4 are
    replaced by ``k_nominal``.  Three-dimensional coefficients
    ``(nTerm, nSam, nDyn)`` with ``k_nominal`` ``(3, nSam, nDyn)`` are
    prepared as one ``(nTerm, nSam*nDyn)`` matrix in column-major order and
    reshaped back (prep_kspha.jl:59-73).
    """
    kspha = np.asarray(kspha)
    if kspha.ndim == 3:
        nT, nSam, nDyn = kspha.shape
        kn = np.asarray(k_nominal, dtype=np.float64)
        if kn.size != 3 * nSam * nDyn:
            raise DimensionMismatch(f"k_nominal must have size (3, {nSam}, {nDyn}), got {kn.shape}")
        flat = prep_kspha(kspha.reshape(nT, nSam * nDyn, order="F"),
                          kn.reshape(3, nSam * nDyn, order="F"), nTerm, recon_terms)
        return flat.reshape(nT, nSam, nDyn, order="F")
    if recon_terms is None:
        recon_terms = "111" if nTerm == 9 else "1111"
    expected = 3 if nTerm == 9 else (4 if nTerm == 16 else 0)
    if expected == 0:
        raise ArgumentError(f"nTerm must be 9 or 16, got {nTerm}")
    if len(recon_terms) != expected:
        raise ArgumentError(f"recon_terms must contain {expected} binary digits for nTerm={nTerm}")
    if any(c not in "01" for c in recon_terms):
        raise ArgumentError(f"recon_terms must contain only '0' and '1', got {recon_terms!r}")
    flags = [c == "1" for c in recon_terms] + ([False] if nTerm == 9 else [])
    out = np.array(kspha, dtype=np.float64, copy=True)
    if not flags[0]:
        out[0, :] = 0.0
    if not flags[1]:
        out[1:4, :] = np.asarray(k_nominal, dtype=np.float64)
    if not flags[2]:
        out[4:9, :] = 0.0
    if nTerm == 16 and not flags[3]:
        out[9:16, :] = 0.0
    return out


def prep_concomitant(bf, kspha, x, y, z, concomitant=None):
    """Append the concomitant basis [z^2, x^2+y^2, xz, yz] and its 4
    coefficient rows (prep_kspha.jl:78-98).  x, y, z are masked coordinates."""
    if concomitant is None:
        return bf, kspha
    c = np.asarray(concomitant)
    if np.iscomplexobj(c) or not np.issubdtype(c.dtype, np.number):
        raise ArgumentError("concomitant must be a real array or nothing")
    kspha = np.asarray(kspha)
    dims = (4,) + kspha.shape[1:]
    # a (4, nSam) matrix also serves coefficients (nTerm, nSam, 1) (prep_kspha.jl:89-92)
    single = kspha.ndim == 3 and kspha.shape[2] == 1 and c.shape == dims[:2]
    if c.shape != dims and not single:
        raise DimensionMismatch(f"concomitant must have size {dims}, got {c.shape}")
    bf_c = np.stack([z ** 2, x ** 2 + y ** 2, x * z, y * z], axis=1)
    return (np.asfortranarray(np.hstack([bf, bf_c])),
            np.concatenate([kspha, c.astype(np.float64).reshape(dims, order="F")], axis=0))
