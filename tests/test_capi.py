"""The C-ABI library loads and exports every entry point its headers
declare (no GPU needed; nothing here launches a kernel)."""
import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import pytest

import cuspfft_gb300 as gb
from cuspfft_gb300 import _capi

ROOT = Path(__file__).resolve().parent.parent


def declared_c_functions():
    text = (ROOT / "include" / "gbspfft.h").read_text()
    return sorted(set(re.findall(r"\b(gbsp_\w+)\s*\(", text)))


def test_c_symbols_exported():
    lib = _capi.load()
    names = declared_c_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    assert set(_capi.EXPORTED) == set(names)


@pytest.mark.skipif(shutil.which("nm") is None, reason="nm not available")
def test_cpp_dropin_symbols_exported():
    out = subprocess.run(["nm", "-DC", "--defined-only", str(_capi.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    text = (ROOT / "include" / "sparse_fft.h").read_text() + (ROOT / "include" / "mtx_reader.h").read_text() \
        + (ROOT / "include" / "sparse_fft_csc.h").read_text()
    funcs = set(re.findall(r"^\w[\w:<>]*\s+(\w+)\(", text, re.M))
    assert {"sparse_fft_csc_bluestein_mixed_radix", "sparse_fft_csc_bluestein_cufft_smooth", "read_mtx",
            "make_compact_csc", "coo_to_csr"} <= funcs
    for f in funcs:
        assert re.search(rf"\b{f}\(", out), f"{f} not exported"


def test_status_and_errors_without_gpu():
    lib = _capi.load()
    assert lib.gbsp_version() > 0
    assert _capi.status_string(_capi.GBSP_ERR_INVALID) == "invalid argument"
    # invalid CSC is rejected before any device work
    cp = (C.c_int * 2)(0, 5)
    ri = (C.c_int * 1)(0)
    sc = (C.c_int * 1)(0)
    h = C.c_void_p()
    st = lib.gbsp_plan_create(3, 3, 1, 1, cp, ri, sc, None, None, C.byref(h))
    assert st == _capi.GBSP_ERR_INVALID
    assert "col_ptr" in _capi.last_error()
    assert lib.gbsp_next_smooth(16437, 9) == -1


def test_plan_create_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    coo = gb.COOMatrix(4, 4, [0, 1], [1, 2])
    with pytest.raises(gb.GbspError):
        gb.Plan(coo)


def test_missing_library_raises(monkeypatch, tmp_path):
    # no fallback implementation: without the native library the package refuses to run
    monkeypatch.setattr(_capi, "_lib", None)
    monkeypatch.setattr(_capi, "LIB_PATH", tmp_path / "libgbspfft.so")
    with pytest.raises(RuntimeError, match="native library missing"):
        _capi.load(build_if_missing=False)


@pytest.mark.parametrize("flags,words", [(1, ["bounded device wait"]), (2, ["not compiled for"]),
                                         (3, ["bounded device wait", "not compiled for"]), (8, ["unknown bits"])])
def test_device_error_word_status(flags, words):
    # the status every synchronous entry point and the C++ API derive from a
    # plan's device error word (here injected on the host): an error word
    # other than 0 is a CUDA failure whose message names the bits
    lib = _capi.load()
    assert lib.gbsp_device_flags_status(0) == _capi.GBSP_OK
    assert lib.gbsp_device_flags_status(flags) == _capi.GBSP_ERR_CUDA
    msg = _capi.last_error()
    assert f"device error flags {flags}" in msg and "not valid" in msg
    for w in words:
        assert w in msg
    with pytest.raises(gb.GbspError, match="not valid"):
        _capi.check(lib.gbsp_device_flags_status(flags), "gbsp_execute")
