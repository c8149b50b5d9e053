"""Restatement of the reference's CPU path -- test / baseline infrastructure only.

The reference's CPU implementation of this transform is cpu_fft_r2c_2d
(src/cpu_reference.cpp:8-63): scatter the binary COO into a dense float32
rows x cols array, plan fftwf_plan_dft_r2c_2d(rows, cols, FFTW_ESTIMATE),
and time only fftwf_execute; the result is rows x (cols/2+1) complex64.
FFTW (a third-party library the reference links, version unpinned; README
suggests 3.3.10) is not installed here or on the GPU host, so the execute
step is restated with scipy.fft.rfft2 on float32 input (pocketfft:
single-precision mixed-radix / Bluestein, an FFTW-class CPU FFT).  The same
two steps are timed the same way: the dense scatter is untimed, the 2-D R2C
transform is timed on the host clock.
"""
from __future__ import annotations

import os
import time

import numpy as np


def dense_scatter(rows: int, cols: int, row_idx, col_idx) -> np.ndarray:
    """Step 1 of cpu_fft_r2c_2d: zeroed float32 array, 1.0 at every nonzero."""
    a = np.zeros((rows, cols), dtype=np.float32)
    a[np.asarray(row_idx), np.asarray(col_idx)] = 1.0
    return a


def cpu_fft_r2c_2d(rows: int, cols: int, row_idx, col_idx, workers: int = 1):
    """Returns (spectrum rows x (cols/2+1) complex64, ms of the execute step)."""
    import scipy.fft
    a = dense_scatter(rows, cols, row_idx, col_idx)
    t0 = time.perf_counter()
    out = scipy.fft.rfft2(a, workers=workers)
    ms = (time.perf_counter() - t0) * 1e3
    return out.astype(np.complex64, copy=False), ms


def time_cpu_baseline(rows: int, cols: int, row_idx, col_idx, budget_s: float = 15.0,
                      workers: int | None = None, max_reps: int = 50) -> dict:
    """Times the execute step repeatedly within ~budget_s; median ms."""
    import scipy.fft
    workers = workers or (os.cpu_count() or 1)
    a = dense_scatter(rows, cols, row_idx, col_idx)
    times = []
    t_start = time.perf_counter()
    while len(times) < max_reps:
        t0 = time.perf_counter()
        scipy.fft.rfft2(a, workers=workers)
        times.append((time.perf_counter() - t0) * 1e3)
        if time.perf_counter() - t_start > budget_s and len(times) >= 3:
            break
    times.sort()
    return {"ms_median": times[len(times) // 2], "ms_min": times[0], "reps": len(times),
            "workers": workers}


# ---------------------------------------------------------------------------
# Host-side restatements of the reference's integer / table code for this path
# ---------------------------------------------------------------------------
import ctypes as _C
import math as _math
from pathlib import Path as _Path

_HERE = _Path(__file__).resolve().parent


def read_mtx(path: str):
    """src/mtx_reader.cu:7-77: returns (rows, cols, row_idx, col_idx) as int32
    arrays, binarized, mirrored when the header says symmetric, sorted and
    de-duplicated.  Raises RuntimeError with the reference's messages."""
    with open(path, "r") as f:
        lines = f.read().split("\n")
    if lines and lines[-1] == "":
        lines = lines[:-1]
    if not lines:
        raise RuntimeError(f"Empty file: {path}")
    if not lines[0].startswith("%%MatrixMarket"):
        raise RuntimeError(f"Not a Matrix Market file: {path}")
    symmetric = ("symmetric" in lines[0]) or ("Symmetric" in lines[0])
    i = 1
    dims = None
    while i < len(lines):
        ln = lines[i]
        i += 1
        if ln and ln[0] != "%":
            dims = ln
            break
    toks = (dims or "").split()
    try:
        rows, cols, stored = int(toks[0]), int(toks[1]), int(toks[2])
    except (IndexError, ValueError):
        raise RuntimeError(f"Bad dimension line in: {path}") from None
    pairs = []
    for _ in range(stored):
        if i >= len(lines):
            raise RuntimeError(f"Unexpected EOF in: {path}")
        t = lines[i].split()
        i += 1
        try:
            r, c = int(t[0]) - 1, int(t[1]) - 1
        except (IndexError, ValueError):
            raise RuntimeError(f"Bad entry line in: {path}") from None
        pairs.append((r, c))
        if symmetric and r != c:
            pairs.append((c, r))
    pairs = sorted(set(pairs))
    r = np.array([p[0] for p in pairs], dtype=np.int32)
    c = np.array([p[1] for p in pairs], dtype=np.int32)
    return rows, cols, r, c


def make_compact_csc(rows: int, cols: int, row_idx, col_idx):
    """include/sparse_fft_internal.cuh:102-120, 193-222: active columns sorted
    and unique, col_ptr over active columns, row_idx by a stable pass over the
    COO order."""
    col_idx = np.asarray(col_idx, dtype=np.int64)
    row_idx = np.asarray(row_idx, dtype=np.int32)
    sparse_cols = np.unique(col_idx).astype(np.int32)
    slot = np.full(cols, -1, dtype=np.int64)
    slot[sparse_cols] = np.arange(sparse_cols.size)
    ids = slot[col_idx]
    counts = np.bincount(ids, minlength=sparse_cols.size) if ids.size else np.zeros(sparse_cols.size, np.int64)
    col_ptr = np.zeros(sparse_cols.size + 1, dtype=np.int32)
    col_ptr[1:] = np.cumsum(counts)
    order = np.argsort(ids, kind="stable")
    return sparse_cols, col_ptr, row_idx[order].astype(np.int32)


def can_pack_u16(rows: int, cols: int) -> bool:
    """include/sparse_fft_internal.cuh:122-124"""
    return rows <= 65536 and cols <= 65536


def next_power_of_two(n: int) -> int:
    """include/sparse_fft_internal.cuh:153-157"""
    p = 1
    while p < n:
        p <<= 1
    return p


def next_smooth(n: int, seven: bool) -> int:
    """src/sparse_fft_bluestein.cu:1975-1994"""
    m = n
    while True:
        x = m
        for p in ((2, 3, 5, 7) if seven else (2, 3)):
            while x % p == 0:
                x //= p
        if x == 1:
            return m
        m += 1


def factor_3_smooth(n: int) -> list:
    """src/sparse_fft_bluestein.cu:2000-2011: 9s, then one 3 if left, then 2s."""
    c3 = 0
    while n % 3 == 0:
        c3 += 1
        n //= 3
    out = [9] * (c3 // 2) + ([3] if c3 % 2 else [])
    while n % 2 == 0:
        out.append(2)
        n //= 2
    if n != 1:
        raise RuntimeError("factor_3_smooth: not 3-smooth")
    return out


def bluestein_chirp(n: int) -> np.ndarray:
    """include/sparse_fft_internal.cuh:168-177: FP64 cos/sin of -pi*k^2/n (k^2
    as a double product, no reduction), rounded to float32; (n, 2) array."""
    out = np.zeros((n, 2), dtype=np.float32)
    for k in range(n):
        a = -_math.pi * (float(k) * float(k)) / float(n)
        out[k] = (_math.cos(a), _math.sin(a))
    return out


def bluestein_b(n: int, fft_len: int) -> np.ndarray:
    """include/sparse_fft_internal.cuh:179-191: b[0] = 1, b[k] = b[L-k] =
    exp(+i*pi*k^2/n) for 0 < k < n, zero elsewhere; (fft_len, 2) float32."""
    out = np.zeros((fft_len, 2), dtype=np.float32)
    out[0] = (1.0, 0.0)
    for k in range(1, n):
        a = _math.pi * (float(k) * float(k)) / float(n)
        z = (_math.cos(a), _math.sin(a))
        out[k] = z
        out[fft_len - k] = z
    return out


# ---------------------------------------------------------------------------
# FP32 CPU restatement of the reference's GPU methods (oracle/ref_gpu_port.c)
# ---------------------------------------------------------------------------
_port = None


def _port_lib():
    global _port
    if _port is None:
        path = _HERE / "_build" / "libref_port.so"
        if not path.exists():
            from . import build as _b
            _b.build()
        lib = _C.CDLL(str(path))
        ip = _C.POINTER(_C.c_int)
        lib.port_sparse_fft.argtypes = [_C.c_int, _C.c_int, _C.c_int, ip, ip, ip, _C.c_int,
                                        _C.POINTER(_C.c_float)]
        lib.port_sparse_fft.restype = _C.c_int
        _port = lib
    return _port


def reference_gpu_method(rows: int, cols: int, row_idx, col_idx, method: int) -> np.ndarray:
    """rows x (cols/2+1) complex64 spectrum from the FP32 CPU restatement of
    sparse_fft_csc_bluestein_mixed_radix (method 3),
    sparse_fft_csc_bluestein_cufft_smooth (method 7) or the power-of-two
    methods (method 2: sparse_fft_csc_bluestein and its wrappers)."""
    sc, cp, ri = make_compact_csc(rows, cols, row_idx, col_idx)
    sc, cp = np.ascontiguousarray(sc, np.int32), np.ascontiguousarray(cp, np.int32)
    ri = np.ascontiguousarray(ri if ri.size else np.zeros(1, np.int32), np.int32)
    sc1 = sc if sc.size else np.zeros(1, np.int32)
    out = np.zeros((rows, cols // 2 + 1, 2), dtype=np.float32)
    ip = _C.POINTER(_C.c_int)
    rc = _port_lib().port_sparse_fft(rows, cols, int(sc.size), sc1.ctypes.data_as(ip), cp.ctypes.data_as(ip),
                                     ri.ctypes.data_as(ip), method,
                                     out.ctypes.data_as(_C.POINTER(_C.c_float)))
    if rc != 0:
        raise RuntimeError(f"port_sparse_fft failed ({rc})")
    return out[..., 0] + 1j * out[..., 1]
