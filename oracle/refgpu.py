"""The reference's own GPU methods run on this GPU -- TEST INFRASTRUCTURE ONLY.

oracle/_ref/ref_kernels.fatbin holds the reference's kernels, compiled for
sm_103a from its src/sparse_fft_bluestein.cu by oracle/build_ref.sh;
oracle/_build/libref_gpu_driver.so (ref_gpu_driver.cpp) launches them in the
order the reference's host code does for

  method 3  sparse_fft_csc_bluestein_mixed_radix   src/sparse_fft_bluestein.cu:2256-2392
  method 7  sparse_fft_csc_bluestein_cufft_smooth  src/sparse_fft_bluestein.cu:2557-2719

The host inputs (compact CSC, chirp, b, radix list) come from ref_port.py,
whose functions are pinned bit for bit to the reference's compiled host code.
Used by tests/ (parity against the reference's GPU output) and by bench.py
(the reference's GPU time on the same device); never by the library.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import ref_port

HERE = Path(__file__).resolve().parent
FATBIN = HERE / "_ref" / "ref_kernels.fatbin"
DRIVER = HERE / "_build" / "libref_gpu_driver.so"
_lib = None


def available() -> bool:
    """True when the reference's kernels were compiled into oracle/_ref."""
    return FATBIN.exists()


def _load():
    global _lib
    if _lib is None:
        if not DRIVER.exists():
            from . import build as _b
            _b.build()
        lib = C.CDLL(str(DRIVER))
        ip, fp = C.POINTER(C.c_int), C.POINTER(C.c_float)
        lib.refgpu_last_error.restype = C.c_char_p
        lib.refgpu_init.argtypes = [C.c_char_p]
        lib.refgpu_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, ip, ip, ip, fp, fp, C.c_int, ip, C.c_int,
                                   C.c_int, fp, C.c_int, C.c_int, fp]
        if lib.refgpu_init(str(FATBIN).encode()) != 0:
            raise RuntimeError("refgpu_init: " + lib.refgpu_last_error().decode())
        _lib = lib
    return _lib


def fft_len(cols: int, method: int) -> int:
    """The method's Bluestein length (next_3_smooth / next_7_smooth of 2*cols-1)."""
    return ref_port.next_smooth(2 * cols - 1, seven=(method == 7))


def run(rows: int, cols: int, row_idx, col_idx, method: int, u_tile: int = 128, n_times: int = 1):
    """(spectrum rows x (cols/2+1) complex64, [ms of each timed tile loop]).

    One call of the reference method on the binary COO matrix: setup, one
    warm-up tile loop, then n_times timed loops (CUDA events around the loop,
    as the reference times it)."""
    lib = _load()
    sc, cp, ri = ref_port.make_compact_csc(rows, cols, row_idx, col_idx)
    L = fft_len(cols, method)
    chirp = np.ascontiguousarray(ref_port.bluestein_chirp(cols), np.float32)
    b = np.ascontiguousarray(ref_port.bluestein_b(cols, L), np.float32)
    factors = np.asarray(ref_port.factor_3_smooth(L) if method == 3 else [0], np.int32)
    stride = (cols // 2 + 1 + 3) // 4 * 4
    out = np.zeros((rows, stride, 2), np.float32)
    times = np.zeros(max(n_times, 1), np.float32)
    ip, fp = C.POINTER(C.c_int), C.POINTER(C.c_float)
    sc = np.ascontiguousarray(sc, np.int32)
    cp = np.ascontiguousarray(cp, np.int32)
    ri = np.ascontiguousarray(ri if ri.size else np.zeros(1, np.int32), np.int32)
    rc = lib.refgpu_run(method, rows, cols, int(sc.size), cp.ctypes.data_as(ip), ri.ctypes.data_as(ip),
                        sc.ctypes.data_as(ip), chirp.ctypes.data_as(fp), b.ctypes.data_as(fp), L,
                        factors.ctypes.data_as(ip), int(factors.size), u_tile, out.ctypes.data_as(fp), stride,
                        n_times, times.ctypes.data_as(fp))
    if rc != 0:
        raise RuntimeError("refgpu_run: " + lib.refgpu_last_error().decode())
    spec = out[:, : cols // 2 + 1, 0] + 1j * out[:, : cols // 2 + 1, 1]
    return spec.astype(np.complex64), times[:n_times].tolist()
