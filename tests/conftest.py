"""Test configuration: import paths and the ``gpu`` marker.

``-m "not gpu"`` runs on a machine without a GPU (oracle vs golden vectors,
host-side logic, C-ABI exports); ``-m gpu`` runs the parity tests through the
C ABI on a GB300.
"""
import os
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "highordermri.jl_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
