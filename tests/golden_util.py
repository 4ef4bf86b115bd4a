"""Loading helpers for the committed golden fixtures (tests/golden/*.npz)."""
from pathlib import Path

import numpy as np

from oracle import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name):
    with np.load(GOLDEN / f"{name}.npz") as d:
        return {k: d[k] for k in d.files}


def model_from_golden(g):
    """Oracle model from a fixture: basis of the masked coordinates (plus
    concomitant columns when present)."""
    mask = g["mask"].astype(bool)
    idx = np.flatnonzero(mask)
    nt = g["kspha"].shape[0]
    bf = oracle.basis(g["x"][idx], g["y"][idx], g["z"][idx], list(range(1, nt + 1)))
    k = g["kspha"]
    if "concomitant" in g:
        x, y, z = g["x"][idx], g["y"][idx], g["z"][idx]
        bf = np.hstack([bf, np.stack([z ** 2, x ** 2 + y ** 2, x * z, y * z], axis=1)])
        k = np.vstack([k, g["concomitant"]])
    m = oracle.Model(bf, k, g["times"], g["fieldmap"][idx], g["csm"][idx], nTerm=nt)
    return m, mask
