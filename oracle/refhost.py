"""ctypes access to the reference's own host code -- TEST INFRASTRUCTURE ONLY.

oracle/_ref/libref_host.so is compiled from the reference sources by
oracle/build_ref.sh (see ref_shim.cu for the wrapped symbols).  It exists only
where the reference tree does; callers skip when available() is False.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB = Path(__file__).resolve().parent / "_ref" / "libref_host.so"
_lib = None


def available() -> bool:
    return LIB.exists()


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(LIB))
        ip = C.POINTER(C.c_int)
        _lib.ref_last_error.restype = C.c_char_p
        _lib.ref_read_mtx.argtypes = [C.c_char_p, ip, ip, ip, C.POINTER(ip), C.POINTER(ip)]
        _lib.ref_free.argtypes = [C.c_void_p]
        _lib.ref_make_compact_csc.argtypes = [C.c_int, C.c_int, C.c_int, ip, ip, ip, ip, ip, ip]
        _lib.ref_can_pack_u16.argtypes = [C.c_int, C.c_int]
        _lib.ref_pack_cols_u16.argtypes = [ip, C.c_int, C.POINTER(C.c_uint16)]
        _lib.ref_bluestein_chirp.argtypes = [C.c_int, C.POINTER(C.c_float)]
        _lib.ref_bluestein_b.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_float)]
        _lib.ref_next_3_smooth.argtypes = [C.c_int]
        _lib.ref_next_7_smooth.argtypes = [C.c_int]
        _lib.ref_next_power_of_two.argtypes = [C.c_int]
        _lib.ref_factor_3_smooth.argtypes = [C.c_int, ip, C.c_int]
    return _lib


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def read_mtx(path: str):
    L = lib()
    rows, cols, nnz = C.c_int(), C.c_int(), C.c_int()
    r, c = C.POINTER(C.c_int)(), C.POINTER(C.c_int)()
    if L.ref_read_mtx(str(path).encode(), C.byref(rows), C.byref(cols), C.byref(nnz), C.byref(r), C.byref(c)):
        raise RuntimeError(L.ref_last_error().decode())
    n = nnz.value
    ri = np.ctypeslib.as_array(r, shape=(max(n, 1),))[:n].copy()
    ci = np.ctypeslib.as_array(c, shape=(max(n, 1),))[:n].copy()
    L.ref_free(C.cast(r, C.c_void_p))
    L.ref_free(C.cast(c, C.c_void_p))
    return rows.value, cols.value, ri, ci


def make_compact_csc(rows, cols, row_idx, col_idx):
    row_idx = np.ascontiguousarray(row_idx, np.int32)
    col_idx = np.ascontiguousarray(col_idx, np.int32)
    nnz = row_idx.size
    na = C.c_int()
    sc = np.zeros(max(cols, 1), np.int32)
    cp = np.zeros(cols + 1, np.int32)
    ri = np.zeros(max(nnz, 1), np.int32)
    lib().ref_make_compact_csc(rows, cols, nnz, _ip(row_idx if nnz else ri), _ip(col_idx if nnz else ri),
                               C.byref(na), _ip(sc), _ip(cp), _ip(ri))
    n = na.value
    return sc[:n].copy(), cp[:n + 1].copy(), ri[:nnz].copy()


def bluestein_chirp(n: int) -> np.ndarray:
    out = np.zeros((n, 2), np.float32)
    lib().ref_bluestein_chirp(n, out.ctypes.data_as(C.POINTER(C.c_float)))
    return out


def bluestein_b(n: int, fft_len: int) -> np.ndarray:
    out = np.zeros((fft_len, 2), np.float32)
    lib().ref_bluestein_b(n, fft_len, out.ctypes.data_as(C.POINTER(C.c_float)))
    return out


def next_3_smooth(n: int) -> int:
    return lib().ref_next_3_smooth(n)


def next_7_smooth(n: int) -> int:
    return lib().ref_next_7_smooth(n)


def next_power_of_two(n: int) -> int:
    return lib().ref_next_power_of_two(n)


def factor_3_smooth(n: int) -> list:
    out = np.zeros(64, np.int32)
    k = lib().ref_factor_3_smooth(n, _ip(out), 64)
    if k < 0:
        raise RuntimeError(lib().ref_last_error().decode())
    return out[:k].tolist()


def can_pack_u16(rows: int, cols: int) -> bool:
    return bool(lib().ref_can_pack_u16(rows, cols))
