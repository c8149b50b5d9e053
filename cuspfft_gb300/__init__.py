"""cuspfft_gb300 -- GB300-native (sm_103a) 2-D R2C FFT of binary sparse matrices.

Drop-in for the reference's hot path (include/sparse_fft.h): the binarizing
Matrix Market reader, the compact-CSC builder, and the
sparse_fft_csc_bluestein_mixed_radix / _cufft_smooth methods, computed by
hand-written CUDA kernels behind a C ABI (include/gbspfft.h).
"""
from ._capi import (GBSP_LEN_3SMOOTH, GBSP_LEN_7SMOOTH, GBSP_LEN_POW2, GBSP_STREAM_TILE_AUTO, GbspError, LIB_PATH,
                    load)
from .sparse_fft import (Batch, COOMatrix, CompactCSC, Plan, SparseFFTResult, make_compact_csc, next_smooth,
                         read_mtx, set_memory_cache, sparse_fft_csc_bluestein, sparse_fft_csc_bluestein_cufft,
                         sparse_fft_csc_bluestein_cufft_smooth, sparse_fft_csc_bluestein_mixed_radix,
                         sparse_fft_csc_bluestein_smem, sparse_fft_csc_stockham_binary_smem)

__all__ = [
    "GBSP_LEN_3SMOOTH", "GBSP_LEN_7SMOOTH", "GBSP_LEN_POW2", "GBSP_STREAM_TILE_AUTO", "GbspError", "LIB_PATH", "load",
    "Batch", "COOMatrix", "CompactCSC", "Plan", "SparseFFTResult", "make_compact_csc", "next_smooth", "read_mtx",
    "set_memory_cache", "sparse_fft_csc_bluestein", "sparse_fft_csc_bluestein_cufft",
    "sparse_fft_csc_bluestein_cufft_smooth", "sparse_fft_csc_bluestein_mixed_radix", "sparse_fft_csc_bluestein_smem",
    "sparse_fft_csc_stockham_binary_smem",
]
