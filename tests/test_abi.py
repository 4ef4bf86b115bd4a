"""The C-ABI library loads and exports every symbol include/hoexplicit.h
declares; argument validation that happens before any CUDA call."""
import ctypes
import os
import re
from pathlib import Path

import pytest

from hoexplicit import _lib

HEADER = Path(__file__).resolve().parent.parent / "include" / "hoexplicit.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"HOE_API[^;(]*?\b(hoe_\w+)\s*\(", text)))


def test_header_declares_expected_entry_points():
    syms = declared_symbols()
    assert set(_lib.EXPORTED) == set(syms), syms


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_version_and_abi():
    lib = _lib.load()
    assert lib.hoe_abi_version() == _lib.HOE_ABI_VERSION
    assert b"sm_103a" in lib.hoe_version()


def test_struct_layouts_match_header():
    # two int32 blocks followed by pointers / doubles, natural alignment
    assert ctypes.sizeof(_lib.HoeDesc) == 14 * 4 + 7 * 8
    assert ctypes.sizeof(_lib.HoeInfo) == 14 * 4 + 8 + 8 + 2 * 4
    assert ctypes.sizeof(_lib.HoeCgParams) == 2 * 4 + 2 * 8
    assert ctypes.sizeof(_lib.HoeCgStats) == 2 * 4 + 2 * 8


STRUCTS = {
    "hoe_desc": "HoeDesc", "hoe_info": "HoeInfo", "hoe_timings": "HoeTimings",
    "hoe_cg_params": "HoeCgParams", "hoe_cg_stats": "HoeCgStats", "hoe_delay_params": "HoeDelayParams",
    "hoe_delay_result": "HoeDelayResult", "hoe_tune_result": "HoeTuneResult",
    "hoe_batch_info": "HoeBatchInfo", "hoe_raw_model": "HoeRawModel",
}


def test_struct_offsets_match_the_c_header(tmp_path):
    # every ctypes field at the offset and every struct at the size that a C
    # compiler gives the declarations in include/hoexplicit.h
    import shutil
    import subprocess
    from pathlib import Path
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    inc = Path(__file__).resolve().parent.parent / "include"
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "hoexplicit.h"', "int main(void) {"]
    expect = {}
    for cname, pyname in STRUCTS.items():
        st = getattr(_lib, pyname)
        lines.append(f'  printf("{cname} %zu\\n", sizeof({cname}));')
        expect[cname] = ctypes.sizeof(st)
        for f in st._fields_:
            cfield = f[0].rstrip("_")   # ctypes spells the C field `lambda` as `lambda_`
            lines.append(f'  printf("{cname}.{f[0]} %zu\\n", offsetof({cname}, {cfield}));')
            expect[f"{cname}.{f[0]}"] = getattr(st, f[0]).offset
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", str(inc), str(src), "-o", str(exe)], check=True)
    got = dict(ln.split() for ln in subprocess.run([str(exe)], check=True, capture_output=True,
                                                    text=True).stdout.splitlines())
    assert {k: int(v) for k, v in got.items()} == expect


def _desc(**over):
    d = _lib.HoeDesc()
    d.abi_version = _lib.HOE_ABI_VERSION
    d.nX, d.nY, d.nZ, d.nSam, d.nCha, d.nTerm, d.nVox = 2, 2, 1, 3, 1, 9, 4
    for k, v in over.items():
        setattr(d, k, v)
    return d


@pytest.mark.parametrize("over,code", [
    (dict(abi_version=99), _lib.HOE_ERR_ARG),
    (dict(nTerm=10), _lib.HOE_ERR_ARG),
    (dict(nVox=0), _lib.HOE_ERR_ARG),
    (dict(nSam=0), _lib.HOE_ERR_ARG),
    (dict(nX=0), _lib.HOE_ERR_DIM),
    (dict(nVox=5), _lib.HOE_ERR_DIM),
    (dict(engine=7), _lib.HOE_ERR_ARG),
])
def test_create_rejects_bad_descriptors_before_any_device_call(over, code):
    lib = _lib.load()
    h = ctypes.c_void_p()
    d = _desc(**over)
    assert lib.hoe_create(ctypes.byref(h), ctypes.byref(d)) == code
    assert not h.value
    assert lib.hoe_last_error(None)


def test_null_arguments():
    lib = _lib.load()
    assert lib.hoe_create(None, None) == _lib.HOE_ERR_ARG
    h = ctypes.c_void_p()
    assert lib.hoe_create(ctypes.byref(h), None) == _lib.HOE_ERR_ARG
    assert lib.hoe_forward(None, None, None, None) == _lib.HOE_ERR_ARG
    p = _lib.HoeCgParams(10, 1, 0.0, 0.0)
    assert lib.hoe_recon(None, None, None, None, ctypes.byref(p), None, None) == _lib.HOE_ERR_ARG
    assert lib.hoe_is_closed(None) == 1
    lib.hoe_free(None)  # no-op


def test_error_mapping():
    with pytest.raises(_lib.ArgumentError):
        _lib.check(_lib.HOE_ERR_CLOSED)
    with pytest.raises(_lib.DimensionMismatch):
        _lib.check(_lib.HOE_ERR_DIM)
    with pytest.raises(_lib.OutOfMemoryError):
        _lib.check(_lib.HOE_ERR_OOM)
    with pytest.raises(_lib.ArgumentError):
        _lib.check(_lib.HOE_ERR_UNSUPPORTED)   # engine unavailable for this operator
    with pytest.raises(_lib.HoeError):
        _lib.check(_lib.HOE_ERR_TIMEOUT)


def test_missing_library_fails_loudly(tmp_path):
    """Without the built library the package raises ImportError on first use;
    there is no CPU or PyTorch fallback of any product."""
    import subprocess
    import sys
    code = ("import sys; sys.path[:0] = ['.', 'highordermri.jl_gb300']\n"
            "from hoexplicit import _lib\n"
            "try:\n"
            "    _lib.load()\n"
            "except ImportError as e:\n"
            "    print('ImportError', 'not found' in str(e))\n")
    env = dict(os.environ, HOE_LIBRARY=str(tmp_path / "absent" / "libhoexplicit.so"))
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                         cwd=str(Path(__file__).resolve().parent.parent), timeout=120)
    assert out.stdout.strip() == "ImportError True", (out.stdout, out.stderr)
