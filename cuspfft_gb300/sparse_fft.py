"""Python mirror of the reference's sparse FFT interface over the C ABI.

Names, argument meanings and error behaviour follow the reference's C++ API
(include/sparse_fft.h:7-83, include/mtx_reader.h:7-30,
include/sparse_fft_internal.cuh:193-222); every call goes through
libgbspfft.so (include/gbspfft.h).  torch supplies device memory and streams.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _capi
from ._capi import (GBSP_LEN_3SMOOTH, GBSP_LEN_7SMOOTH, GBSP_LEN_POW2, GBSP_PLANNER_LEARNED, GBSP_PLANNER_MODEL,
                    GbspMatrix, GbspOptions, GbspPlanInfo, check, load)


@dataclass
class COOMatrix:
    """Binary sparse matrix: (row, col) pairs, values implicitly 1."""
    rows: int
    cols: int
    row_idx: np.ndarray
    col_idx: np.ndarray

    def __post_init__(self):
        self.row_idx = np.ascontiguousarray(self.row_idx, dtype=np.int32)
        self.col_idx = np.ascontiguousarray(self.col_idx, dtype=np.int32)
        if self.row_idx.shape != self.col_idx.shape or self.row_idx.ndim != 1:
            raise ValueError("row_idx and col_idx must be 1-D arrays of equal length")

    @property
    def nnz(self) -> int:
        return int(self.row_idx.size)


@dataclass
class CompactCSC:
    n_sparse_cols: int
    sparse_cols: np.ndarray
    col_ptr: np.ndarray
    row_idx: np.ndarray


@dataclass
class SparseFFTResult:
    """d_output: torch complex64 tensor (rows, output_cols) on the GPU;
    output_cols is the padded row pitch (cols/2+1 rounded up to 4)."""
    d_output: object
    output_cols: int
    ms: float
    mem_bytes: int
    h_output: list = field(default_factory=list)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def read_mtx(path: str) -> COOMatrix:
    """Binarizing Matrix Market reader; raises RuntimeError on failure
    (the reference throws std::runtime_error, src/mtx_reader.cu:7-77)."""
    lib = load()
    rows, cols, nnz = C.c_int(), C.c_int(), C.c_int()
    ri, ci = C.POINTER(C.c_int)(), C.POINTER(C.c_int)()
    st = lib.gbsp_read_mtx(str(path).encode(), C.byref(rows), C.byref(cols), C.byref(nnz),
                           C.byref(ri), C.byref(ci))
    if st != 0:
        raise RuntimeError(_capi.last_error())
    try:
        n = nnz.value
        r = np.ctypeslib.as_array(ri, shape=(max(n, 1),))[:n].copy()
        c = np.ctypeslib.as_array(ci, shape=(max(n, 1),))[:n].copy()
    finally:
        lib.gbsp_free(C.cast(ri, C.c_void_p))
        lib.gbsp_free(C.cast(ci, C.c_void_p))
    return COOMatrix(rows.value, cols.value, r, c)


def make_compact_csc(coo: COOMatrix) -> CompactCSC:
    lib = load()
    sc = np.zeros(max(coo.cols, 1), np.int32)
    cp = np.zeros(coo.cols + 1, np.int32)
    ri = np.zeros(max(coo.nnz, 1), np.int32)
    na = C.c_int()
    check(lib.gbsp_build_compact_csc(coo.rows, coo.cols, coo.nnz, _ip(coo.row_idx), _ip(coo.col_idx),
                                     C.byref(na), _ip(sc), _ip(cp), _ip(ri)), "make_compact_csc")
    n = na.value
    return CompactCSC(n, sc[:n].copy(), cp[:n + 1].copy(), ri[:coo.nnz].copy())


def next_smooth(n: int, policy: int = GBSP_LEN_3SMOOTH) -> int:
    return int(load().gbsp_next_smooth(int(n), int(policy)))


def set_memory_cache(nbytes: int) -> None:
    """Freed plan memory the library's pool keeps for later plans, per device
    (default 1 GiB); 0 keeps nothing."""
    check(load().gbsp_set_memory_cache(int(nbytes)), "gbsp_set_memory_cache")


def _stream_handle(stream) -> Optional[int]:
    """cudaStream_t of a torch stream; torch's current stream when None (the
    legacy default stream if CUDA is unavailable -- the library then reports
    the missing device itself)."""
    import torch
    if stream is None:
        if not torch.cuda.is_available():
            return None
        stream = torch.cuda.current_stream()
    return stream.cuda_stream


def planner_code(planner) -> int:
    """"model" (analytic, default) or "learned" (the installed MLP cost model;
    the packaged model is installed on first use)."""
    if planner in (None, "model", GBSP_PLANNER_MODEL):
        return GBSP_PLANNER_MODEL
    if planner in ("learned", GBSP_PLANNER_LEARNED):
        from . import costmodel
        costmodel.ensure_installed()
        return GBSP_PLANNER_LEARNED
    raise ValueError(f"unknown planner {planner!r}")


def make_options(options: Optional[GbspOptions] = None, radix=None, planner=None, **fields) -> GbspOptions:
    """GbspOptions from an existing one (e.g. an autotuner result) with the
    given fields overriding; zero fields mean automatic."""
    o = GbspOptions()
    if options is not None:
        C.memmove(C.byref(o), C.byref(options), C.sizeof(GbspOptions))
    for k, v in fields.items():
        if v:
            setattr(o, k, int(v))
    if radix:
        for i in range(8):
            o.radix[i] = int(radix[i]) if i < len(radix) else 0
    if planner is not None or options is None:
        o.planner = planner_code(planner)
    return o


class Plan:
    """One matrix's transform: tables and uploaded CSC live on the GPU until
    close().  execute() is the reference's timed tile loop."""

    def __init__(self, coo: COOMatrix, *, length_policy: int = 0, u_tile: int = 0,
                 kahan_min_degree: int = 0, index_bytes: int = 0, max_channel_len: int = 0,
                 rows_threads: int = 0, row_table_mode: int = 0, radix=None, pass1_shape: int = 0,
                 channel_mode: int = 0, stream_tile_rows: int = 0, exact_phases: int = 0,
                 force_bluestein: int = 0, planner=None,
                 options: Optional[GbspOptions] = None, stream=None,
                 csc: Optional[CompactCSC] = None):
        lib = load()
        self._lib = lib
        self._h = C.c_void_p()
        csc = csc if csc is not None else make_compact_csc(coo)
        self.rows, self.cols = coo.rows, coo.cols
        o = make_options(options, radix=radix, planner=planner, length_policy=length_policy, u_tile=u_tile,
                         kahan_min_degree=kahan_min_degree, index_bytes=index_bytes,
                         max_channel_len=max_channel_len, rows_threads=rows_threads,
                         row_table_mode=row_table_mode, pass1_shape=pass1_shape, channel_mode=channel_mode,
                         stream_tile_rows=stream_tile_rows, exact_phases=exact_phases,
                         force_bluestein=force_bluestein)
        cp = np.ascontiguousarray(csc.col_ptr, np.int32)
        ri = np.ascontiguousarray(csc.row_idx if coo.nnz else np.zeros(1, np.int32), np.int32)
        sc = np.ascontiguousarray(csc.sparse_cols if csc.n_sparse_cols else np.zeros(1, np.int32),
                                  np.int32)
        check(lib.gbsp_plan_create(coo.rows, coo.cols, csc.n_sparse_cols, coo.nnz, _ip(cp), _ip(ri),
                                   _ip(sc), C.byref(o), _stream_handle(stream), C.byref(self._h)),
              "gbsp_plan_create")
        info = GbspPlanInfo()
        check(lib.gbsp_plan_get_info(self._h, C.byref(info)), "gbsp_plan_get_info")
        self.info = info.as_dict()

    @property
    def output_pitch(self) -> int:
        return self.info["output_pitch"]

    def empty_output(self):
        import torch
        return torch.empty((self.rows, self.output_pitch), dtype=torch.complex64, device="cuda")

    def execute(self, out, stream=None) -> None:
        if out.dtype.__str__() != "torch.complex64" or not out.is_cuda or not out.is_contiguous():
            raise ValueError("out must be a contiguous complex64 CUDA tensor")
        if out.dim() != 2 or out.shape[0] < self.rows:
            raise ValueError("out must have shape (rows, pitch)")
        check(self._lib.gbsp_execute(self._h, C.c_void_p(out.data_ptr()), out.shape[1],
                                     _stream_handle(stream)), "gbsp_execute")

    def execute_to_host(self, host_out, tile_rows: int = 0, stream=None) -> None:
        """Streams the spectrum into host_out (rows x pitch complex64, CPU,
        contiguous; pinned memory lets the copies overlap the compute) one
        tile of Bluestein rows at a time.  Blocks until done."""
        if str(host_out.dtype) != "torch.complex64" or host_out.is_cuda or not host_out.is_contiguous():
            raise ValueError("host_out must be a contiguous complex64 CPU tensor")
        if host_out.dim() != 2 or host_out.shape[0] < self.rows:
            raise ValueError("host_out must have shape (rows, pitch)")
        check(self._lib.gbsp_execute_to_host(self._h, C.c_void_p(host_out.data_ptr()), host_out.shape[1],
                                             tile_rows, _stream_handle(stream)), "gbsp_execute_to_host")

    def execute_profiled(self, out, stream=None) -> tuple[float, float]:
        """Runs execute() with events around each phase; returns (ms pass 1, ms rows)."""
        a, b = C.c_float(), C.c_float()
        check(self._lib.gbsp_execute_profiled(self._h, C.c_void_p(out.data_ptr()), out.shape[1],
                                              _stream_handle(stream), C.byref(a), C.byref(b)),
              "gbsp_execute_profiled")
        return a.value, b.value

    def error_flags(self) -> int:
        """Reads and clears the device error word (0 = no bounded wait timed out)."""
        f = C.c_int()
        check(self._lib.gbsp_plan_error_flags(self._h, C.byref(f)), "gbsp_plan_error_flags")
        return f.value

    def check_device_flags(self, who: str = "transform") -> None:
        """Reads and clears the device error word; raises GbspError if a
        kernel of this plan reported an error since the last read."""
        check(self._lib.gbsp_device_flags_status(self.error_flags()), who)

    @property
    def device_bytes(self) -> int:
        """Device memory the plan holds now (its allocation and any streaming slabs)."""
        info = GbspPlanInfo()
        check(self._lib.gbsp_plan_get_info(self._h, C.byref(info)), "gbsp_plan_get_info")
        return int(info.device_bytes)

    def column_sums(self, u0: int, n_rows: int, out, stream=None) -> None:
        """S[u-u0][c] for u in [u0, u0+n_rows) and every column c (pitch >= cols rounded up to even)."""
        check(self._lib.gbsp_column_sums(self._h, u0, n_rows, C.c_void_p(out.data_ptr()), out.shape[1],
                                         _stream_handle(stream)), "gbsp_column_sums")

    def close(self) -> None:
        if self._h:
            self._lib.gbsp_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Batch:
    """Many matrices transformed together: one persistent launch per pass fed
    by device work queues (gbsp_batch_* in include/gbspfft.h).

    outputs are bound with set_outputs(); execute() enqueues the whole batch,
    graph_launch() replays it as a CUDA graph.  Each output equals what
    Plan(coo).execute() writes for the same matrix and options."""

    def __init__(self, coos, *, length_policy: int = 0, kahan_min_degree: int = 0,
                 index_bytes: int = 0, max_channel_len: int = 0, row_table_mode: int = 0, pass1_shape: int = 0,
                 exact_phases: int = 0, planner=None, stream=None):
        lib = load()
        self._lib = lib
        self._h = C.c_void_p()
        self.shapes = [(c.rows, c.cols) for c in coos]
        n = len(coos)
        if n < 1:
            raise ValueError("Batch needs at least one matrix")
        keep = []
        mats = (GbspMatrix * n)()
        for i, coo in enumerate(coos):
            csc = make_compact_csc(coo)
            cp = np.ascontiguousarray(csc.col_ptr, np.int32)
            ri = np.ascontiguousarray(csc.row_idx if coo.nnz else np.zeros(1, np.int32), np.int32)
            sc = np.ascontiguousarray(csc.sparse_cols if csc.n_sparse_cols else np.zeros(1, np.int32), np.int32)
            keep += [cp, ri, sc]
            mats[i] = GbspMatrix(coo.rows, coo.cols, csc.n_sparse_cols, coo.nnz, _ip(cp), _ip(ri), _ip(sc))
        o = make_options(None, planner=planner, length_policy=length_policy, kahan_min_degree=kahan_min_degree,
                         index_bytes=index_bytes, max_channel_len=max_channel_len, row_table_mode=row_table_mode,
                         pass1_shape=pass1_shape, exact_phases=exact_phases)
        check(lib.gbsp_batch_create(n, mats, C.byref(o), _stream_handle(stream), C.byref(self._h)),
              "gbsp_batch_create")
        self.infos = []
        for i in range(n):
            info = GbspPlanInfo()
            check(lib.gbsp_batch_plan_info(self._h, i, C.byref(info)), "gbsp_batch_plan_info")
            self.infos.append(info.as_dict())
        self._outs = None

    def __len__(self) -> int:
        return len(self.shapes)

    def empty_outputs(self):
        import torch
        return [torch.empty((r, info["output_pitch"]), dtype=torch.complex64, device="cuda")
                for (r, _), info in zip(self.shapes, self.infos)]

    def set_outputs(self, outs) -> None:
        n = len(self.shapes)
        if len(outs) != n:
            raise ValueError(f"set_outputs needs {n} tensors")
        for (r, _), out in zip(self.shapes, outs):
            if str(out.dtype) != "torch.complex64" or not out.is_cuda or not out.is_contiguous():
                raise ValueError("outputs must be contiguous complex64 CUDA tensors")
            if out.dim() != 2 or out.shape[0] < r:
                raise ValueError("each output must have shape (rows, pitch)")
        ptrs = (C.c_void_p * n)(*[o.data_ptr() for o in outs])
        pitches = (C.c_size_t * n)(*[o.shape[1] for o in outs])
        check(self._lib.gbsp_batch_set_outputs(self._h, ptrs, pitches), "gbsp_batch_set_outputs")
        self._outs = list(outs)  # keeps the memory alive while bound

    def execute(self, stream=None) -> None:
        check(self._lib.gbsp_batch_execute(self._h, _stream_handle(stream)), "gbsp_batch_execute")

    def graph_launch(self, stream=None) -> None:
        check(self._lib.gbsp_batch_graph_launch(self._h, _stream_handle(stream)), "gbsp_batch_graph_launch")

    def error_flags(self) -> int:
        f = C.c_int()
        check(self._lib.gbsp_batch_error_flags(self._h, C.byref(f)), "gbsp_batch_error_flags")
        return f.value

    def close(self) -> None:
        if self._h:
            self._lib.gbsp_batch_destroy(self._h)
            self._h = C.c_void_p()
        self._outs = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _run_method(coo: COOMatrix, u_tile: int, policy: int) -> SparseFFTResult:
    import torch
    if u_tile <= 0:
        raise RuntimeError("CSC tile size must be positive")
    with Plan(coo, length_policy=policy, u_tile=u_tile) as plan:
        out = plan.empty_output()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        plan.execute(out)
        e1.record()
        e1.synchronize()
        plan.check_device_flags("gbsp_execute")
        # the reference's metric is the device memory the call holds at its
        # end (src/sparse_fft_bluestein.cu:7-20): plan buffers and output
        mem = plan.device_bytes + out.numel() * out.element_size()
        return SparseFFTResult(out, plan.output_pitch, e0.elapsed_time(e1), mem)


def sparse_fft_csc_bluestein_mixed_radix(coo: COOMatrix, u_tile: int = 128) -> SparseFFTResult:
    """Reference include/sparse_fft.h:57 -- fft_len = next 3-smooth >= 2*cols-1."""
    return _run_method(coo, u_tile, GBSP_LEN_3SMOOTH)


def sparse_fft_csc_bluestein_cufft_smooth(coo: COOMatrix, u_tile: int = 128) -> SparseFFTResult:
    """Reference include/sparse_fft.h:70 -- fft_len = next 7-smooth >= 2*cols-1,
    computed by this library's own FFT (no cuFFT)."""
    return _run_method(coo, u_tile, GBSP_LEN_7SMOOTH)


def sparse_fft_csc_bluestein(coo: COOMatrix, u_tile: int = 256, use_stockham: bool = False,
                             fft_backend: int = 0) -> SparseFFTResult:
    """Reference include/sparse_fft.h:23 -- fft_len = next power of two >=
    2*cols-1.  use_stockham and fft_backend pick the reference's FFT
    implementation; here every backend runs this library's kernels."""
    return _run_method(coo, u_tile, GBSP_LEN_POW2)


def sparse_fft_csc_bluestein_smem(coo: COOMatrix, u_tile: int = 256) -> SparseFFTResult:
    """Reference include/sparse_fft.h:26 (fft_backend 1 of the above)."""
    return _run_method(coo, u_tile, GBSP_LEN_POW2)


def sparse_fft_csc_bluestein_cufft(coo: COOMatrix, u_tile: int = 256) -> SparseFFTResult:
    """Reference include/sparse_fft.h:27 (fft_backend 3; no cuFFT here)."""
    return _run_method(coo, u_tile, GBSP_LEN_POW2)


def sparse_fft_csc_stockham_binary_smem(coo: COOMatrix, u_tile: int = 128) -> SparseFFTResult:
    """Reference include/sparse_fft.h:83 -- power-of-two length, non-streaming;
    the byte-mask LUT pass 1 is replaced by this library's pass 1 (same sums)."""
    return _run_method(coo, u_tile, GBSP_LEN_POW2)
