"""The allocation-free forward (hoe_forward_noalloc) against hoe_forward.

hoe_forward_noalloc serves callers that cannot allocate device memory: it
takes the model as device arrays the caller already owns and keeps its
scratch in a fixed static device array.  This test calls it through the C ABI
twice in a row on the same inputs and checks both results against the
handle-based hoe_forward and against the FP64 oracle, within the plain FP32
tolerance (1e-5 relative L2).
It lives in its own file, collected last, and passes alone or after the
other tests.
"""
import ctypes

import numpy as np
import pytest

from hoexplicit import _lib

TOL = 1e-5


def _raw_model(op, torch, with_fieldmap=True):
    k = op._keep
    dev = op.torch_device
    arrays = {
        "mask_idx": torch.from_numpy(k["mask_idx"]).to(dev),
        "bf": torch.from_numpy(np.ascontiguousarray(k["bf"].T)).to(dev),        # (nTermEff, nVox): v fastest
        "kspha": torch.from_numpy(np.ascontiguousarray(k["kspha"].T)).to(dev),  # (nSam, nTermEff): l fastest
        "times": torch.from_numpy(k["times"]).to(dev),
        "csm": torch.from_numpy(np.ascontiguousarray(k["csm"].T.astype(np.complex64))).to(dev),
    }
    if with_fieldmap:
        arrays["fieldmap"] = torch.from_numpy(k["fieldmap"]).to(dev)
    m = _lib.HoeRawModel()
    m.nVox, m.nSam, m.nCha, m.nTermEff = op.nVox, op.nSam, op.nCha, op.nTermEff
    for name, t in arrays.items():
        setattr(m, name, t.data_ptr())
    return m, arrays


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


# 8 and 20 coils run the 8- and 16-coil kernels; 3 coils without a fieldmap
# (NULL) the 4-coil kernel; 131,072 samples x 16 coils fill the static scratch
# exactly (one split of 2^21 partial sums)
NOALLOC_CASES = [
    dict(shape=(33, 29, 1), nSam=700, nCha=8, nTerm=16, conc=True),
    dict(shape=(20, 18, 3), nSam=517, nCha=20, nTerm=9),
    dict(shape=(17, 15, 1), nSam=389, nCha=3, nTerm=16, fieldmap=False),
    dict(shape=(8, 7, 1), nSam=131072, nCha=16, nTerm=9),
]


@pytest.mark.gpu
@pytest.mark.parametrize("params", NOALLOC_CASES, ids=["2d-8c-conc", "3d-20c", "2d-3c-nofieldmap", "full-scratch-16c"])
def test_noalloc_forward_matches_handle_forward(params):
    torch = pytest.importorskip("torch")
    from hoexplicit import HighOrderExplicitOp, workloads
    from oracle import oracle
    params = dict(params)
    with_fm = params.pop("fieldmap", True)
    w = workloads.small(seed=17, **params)
    kw = w.op_kwargs()
    if not with_fm:
        kw.pop("fieldmap")
    op = HighOrderExplicitOp(w.grid, w.kspha, w.times, engine="fp32", **kw)
    x = torch.from_numpy(w.x.astype(np.complex64)).to(op.torch_device)
    y_ref = (op * x).cpu().numpy()
    # the FP64 oracle on the same model arrays
    k = op._keep
    fm = k["fieldmap"] if with_fm else None
    y64 = oracle.forward(oracle.Model(k["bf"], k["kspha"], k["times"], fm, k["csm"]),
                         w.x[k["mask_idx"]])
    assert _rel(y_ref, y64) < TOL
    m, keep = _raw_model(op, torch, with_fieldmap=with_fm)
    lib = _lib.load()
    stream = torch.cuda.current_stream(op.device).cuda_stream
    for call in range(2):
        y = torch.full((op.nrow,), complex(np.nan, np.nan), dtype=torch.complex64, device=op.torch_device)
        rc = lib.hoe_forward_noalloc(ctypes.byref(m), x.data_ptr(), y.data_ptr(), stream)
        assert rc == _lib.HOE_OK, lib.hoe_last_error(None)
        torch.cuda.synchronize()
        yn = y.cpu().numpy()
        assert _rel(yn, y_ref) < TOL, (call, _rel(yn, y_ref))
        assert _rel(yn, y64) < TOL, (call, _rel(yn, y64))
    op.close()


@pytest.mark.parametrize("nSam,nCha", [(200_000, 16), (131_073, 16), (2_097_153 // 4 + 1, 4)])
def test_noalloc_rejects_sizes_beyond_the_static_scratch(nSam, nCha):
    # one sample tile beyond the 2^21 partial sums is rejected before any
    # device access
    lib = _lib.load()
    m = _lib.HoeRawModel()
    m.nVox, m.nSam, m.nCha, m.nTermEff = 10, nSam, nCha, 16
    for name in ("mask_idx", "bf", "kspha", "times", "csm"):
        setattr(m, name, 1)  # never dereferenced: the size check comes first
    rc = lib.hoe_forward_noalloc(ctypes.byref(m), 1, 1, None)
    assert rc == _lib.HOE_ERR_DIM
    assert b"static scratch" in lib.hoe_last_error(None)
