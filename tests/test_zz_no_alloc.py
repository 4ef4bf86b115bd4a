"""The allocation-free forward (hoe_forward_noalloc) against hoe_forward.

hoe_forward_noalloc serves callers that cannot allocate device memory: it
takes the model as device arrays the caller already owns and keeps its
scratch in a fixed static device array.  This test calls it through the C ABI
twice in a row on the same inputs and checks both results against the
handle-based hoe_forward within the plain FP32 tolerance (1e-5 relative L2).
It lives in its own file, collected last, and passes alone or after the
other tests.
"""
import ctypes

import numpy as np
import pytest

from hoexplicit import _lib

TOL = 1e-5


def _raw_model(op, torch):
    k = op._keep
    dev = op.torch_device
    arrays = {
        "mask_idx": torch.from_numpy(k["mask_idx"]).to(dev),
        "bf": torch.from_numpy(np.ascontiguousarray(k["bf"].T)).to(dev),        # (nTermEff, nVox): v fastest
        "kspha": torch.from_numpy(np.ascontiguousarray(k["kspha"].T)).to(dev),  # (nSam, nTermEff): l fastest
        "times": torch.from_numpy(k["times"]).to(dev),
        "fieldmap": torch.from_numpy(k["fieldmap"]).to(dev),
        "csm": torch.from_numpy(np.ascontiguousarray(k["csm"].T.astype(np.complex64))).to(dev),
    }
    m = _lib.HoeRawModel()
    m.nVox, m.nSam, m.nCha, m.nTermEff = op.nVox, op.nSam, op.nCha, op.nTermEff
    for name, t in arrays.items():
        setattr(m, name, t.data_ptr())
    return m, arrays


@pytest.mark.gpu
@pytest.mark.parametrize("params", [
    dict(shape=(33, 29, 1), nSam=700, nCha=8, nTerm=16, conc=True),
    dict(shape=(20, 18, 3), nSam=517, nCha=20, nTerm=9),
], ids=["2d-8c-conc", "3d-20c"])
def test_noalloc_forward_matches_handle_forward(params):
    torch = pytest.importorskip("torch")
    from hoexplicit import HighOrderExplicitOp, workloads
    w = workloads.small(seed=17, **params)
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="fp32", **w.op_kwargs())
    x = torch.from_numpy(w.x.astype(np.complex64)).to(op.torch_device)
    y_ref = (op * x).cpu().numpy()
    m, keep = _raw_model(op, torch)
    lib = _lib.load()
    stream = torch.cuda.current_stream(op.device).cuda_stream
    for call in range(2):
        y = torch.full((op.nrow,), complex(np.nan, np.nan), dtype=torch.complex64, device=op.torch_device)
        rc = lib.hoe_forward_noalloc(ctypes.byref(m), x.data_ptr(), y.data_ptr(), stream)
        assert rc == _lib.HOE_OK, lib.hoe_last_error(None)
        torch.cuda.synchronize()
        yn = y.cpu().numpy()
        err = np.linalg.norm(yn - y_ref) / np.linalg.norm(y_ref)
        assert err < TOL, (call, err)
    op.close()


def test_noalloc_rejects_sizes_beyond_the_static_scratch():
    lib = _lib.load()
    m = _lib.HoeRawModel()
    m.nVox, m.nSam, m.nCha, m.nTermEff = 10, 200_000, 16, 16
    for name in ("mask_idx", "bf", "kspha", "times", "csm"):
        setattr(m, name, 1)  # never dereferenced: the size check comes first
    rc = lib.hoe_forward_noalloc(ctypes.byref(m), 1, 1, None)
    assert rc == _lib.HOE_ERR_DIM
    assert b"static scratch" in lib.hoe_last_error(None)
