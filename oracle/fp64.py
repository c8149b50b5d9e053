"""FP64 oracle for the binary-sparse 2-D R2C FFT -- test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / accuracy
legs may import this module; the library never does.

What it computes is the definition of the reference's output
(src/sparse_fft_bluestein.cu:2256-2392; README "2-pass" description):

    F[u][v] = sum over nonzeros (r, c) of exp(-2*pi*i*(u*r/rows + v*c/cols))

for v in [0, cols/2], in float64:
  * pass 1 (rows axis) with EXACT integer phases (u*r) mod rows -- the same
    reduction the reference performs in 32-bit (phase_idx,
    include/sparse_fft_internal.cuh:51-53), here in int64 so it is exact for
    every size;
  * pass 2 (columns axis) with numpy's float64 FFT (pocketfft, exact-length
    mixed radix / Bluestein internally), an independent FFT implementation.

For large matrices the spectrum is evaluated on a subset of rows u (every
row of the output is an independent function of the input), which is how the
bench states rel-L2 for the full-size configurations.
"""
from __future__ import annotations

import numpy as np


def column_sums_fp64(rows: int, cols: int, row_idx: np.ndarray, col_idx: np.ndarray,
                     us: np.ndarray) -> np.ndarray:
    """S[i][c] = sum_{r: A[r,c]=1} exp(-2*pi*i*(us[i]*r mod rows)/rows), dense over c."""
    us = np.asarray(us, dtype=np.int64)
    r = np.asarray(row_idx, dtype=np.int64)
    c = np.asarray(col_idx, dtype=np.int64)
    out = np.zeros((us.size, cols), dtype=np.complex128)
    if r.size == 0:
        return out
    # chunk the (u, nnz) product to bound memory
    chunk = max(1, int(4_000_000 // max(r.size, 1)))
    for i0 in range(0, us.size, chunk):
        u = us[i0:i0 + chunk]
        ph = (u[:, None] * r[None, :]) % rows
        w = np.exp(-2j * np.pi * ph.astype(np.float64) / rows)
        for k in range(u.size):
            out[i0 + k] = np.bincount(c, weights=w[k].real, minlength=cols) + \
                1j * np.bincount(c, weights=w[k].imag, minlength=cols)
    return out


def spectrum_rows_fp64(rows: int, cols: int, row_idx: np.ndarray, col_idx: np.ndarray,
                       us=None) -> np.ndarray:
    """F[us][0..cols/2] in complex128.  us=None means every row."""
    if us is None:
        us = np.arange(rows)
    s = column_sums_fp64(rows, cols, row_idx, col_idx, us)
    return np.fft.fft(s, axis=1)[:, : cols // 2 + 1]


def spectrum_dense_fp64(rows: int, cols: int, row_idx: np.ndarray, col_idx: np.ndarray) -> np.ndarray:
    """Same spectrum via a dense float64 rfft2 (independent cross-check, small sizes)."""
    a = np.zeros((rows, cols), dtype=np.float64)
    a[np.asarray(row_idx), np.asarray(col_idx)] = 1.0
    return np.fft.rfft2(a)


def direct_dft_fp64(rows: int, cols: int, row_idx, col_idx) -> np.ndarray:
    """Brute-force O(rows*cols*nnz) definition, for tiny matrices only."""
    u = np.arange(rows)[:, None, None]
    v = np.arange(cols // 2 + 1)[None, :, None]
    r = np.asarray(row_idx, dtype=np.int64)[None, None, :]
    c = np.asarray(col_idx, dtype=np.int64)[None, None, :]
    ph = ((u * r) % rows) / rows + ((v * c) % cols) / cols
    return np.exp(-2j * np.pi * ph).sum(axis=2)


def rel_l2(x: np.ndarray, ref: np.ndarray) -> float:
    """||x - ref||_2 / ||ref||_2 over all elements (complex)."""
    x = np.asarray(x, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    den = np.linalg.norm(ref.ravel())
    num = np.linalg.norm((x - ref).ravel())
    return float(num / den) if den > 0 else float(num)


def check_stats(x: np.ndarray, ref: np.ndarray) -> dict:
    """The reference CLI's check line: max_abs, max_rel (|d|/max(1,|ref|)),
    rms_abs (src/main.cu:168-206), plus rel_l2."""
    d = np.abs(np.asarray(x, np.complex128) - np.asarray(ref, np.complex128))
    m = np.abs(ref)
    return {"max_abs": float(d.max(initial=0.0)),
            "max_rel": float((d / np.maximum(1.0, m)).max(initial=0.0)),
            "rms_abs": float(np.sqrt(np.mean(d ** 2))) if d.size else 0.0,
            "rel_l2": rel_l2(x, ref)}
