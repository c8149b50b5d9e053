// sparse_fft.h -- the drop-in C++ API of the reference's sparse FFT
// (reference include/sparse_fft.h:7-83): same result struct, same entry
// points, same default arguments, same ownership rules.
//
// Implemented in cuspfft_gb300/csrc/sparse_fft_api.cu on top of the C ABI in
// gbspfft.h.  The two hot methods run this library's sm_103a kernels:
//   sparse_fft_csc_bluestein_mixed_radix   fft_len = next 3-smooth >= 2*cols-1
//   sparse_fft_csc_bluestein_cufft_smooth  fft_len = next 7-smooth >= 2*cols-1
// (no cuFFT is called by either).  sparse_fft_csc_bluestein_mixed_radix_graph
// replays the same work as one CUDA graph.  The reference's other methods
// (power-of-two lengths, streaming to host memory, the byte-mask LUT pass 1)
// compute the same spectrum; here they run the same kernels at the
// power-of-two length, the streamed ones through gbsp_execute_to_host.
// Every entry point throws std::runtime_error on a bad u_tile, a CUDA
// failure or a device error word a kernel set.
#pragma once
#include <cuComplex.h>
#include <vector>
#include "mtx_reader.h"

struct SparseFFTResult {
    cuFloatComplex* d_output;  // device array of rows * output_cols; the caller cudaFree()s it
    int output_cols;           // row pitch of d_output: (cols/2+1) rounded up to a multiple of 4
    float ms;                  // device time of the transform loop (setup excluded)
    size_t mem_bytes;          // device memory the call holds at its end: plan buffers + output
    std::vector<cuFloatComplex> h_output;  // host copy for streamed methods (empty otherwise)
};

// --- hot path (reference include/sparse_fft.h:57, :63, :70) ---------------
// u_tile: Bluestein rows per tile; each Bluestein row u <= rows/2 produces
// output rows u and rows-u.  Must be positive (std::runtime_error otherwise).
SparseFFTResult sparse_fft_csc_bluestein_mixed_radix(const COOMatrix& coo, int u_tile = 128);
SparseFFTResult sparse_fft_csc_bluestein_mixed_radix_graph(const COOMatrix& coo, int u_tile = 128);
SparseFFTResult sparse_fft_csc_bluestein_cufft_smooth(const COOMatrix& coo, int u_tile = 128);

// --- the reference's other methods (reference include/sparse_fft.h:23-50, :83) ---
SparseFFTResult sparse_fft_csc_bluestein(const COOMatrix& coo, int u_tile = 256,
                                         bool use_stockham = false, int fft_backend = 0);
SparseFFTResult sparse_fft_csc_bluestein_smem(const COOMatrix& coo, int u_tile = 256);
SparseFFTResult sparse_fft_csc_bluestein_cufft(const COOMatrix& coo, int u_tile = 256);
SparseFFTResult sparse_fft_csc_stockham_streaming(const COOMatrix& coo, int u_tile = 128,
                                                   int fft_backend = 0);
SparseFFTResult sparse_fft_csc_bluestein_cufft_streaming(const COOMatrix& coo, int u_tile = 128);
SparseFFTResult sparse_fft_csc_stockham_graph(const COOMatrix& coo, int u_tile = 128);
SparseFFTResult sparse_fft_csc_bluestein_binary_lut(const COOMatrix& coo, int u_tile = 128);
SparseFFTResult sparse_fft_csc_stockham_binary_smem(const COOMatrix& coo, int u_tile = 128);
