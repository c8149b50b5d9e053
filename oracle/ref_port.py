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
