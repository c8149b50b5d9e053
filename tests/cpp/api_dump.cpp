// api_dump.cpp -- test helper: calls one method of the C++ drop-in API
// (include/sparse_fft.h) on a Matrix Market file `repeat` times in one
// process, prints each call's SparseFFTResult fields, and writes the last
// call's spectrum for the Python tests to compare with the FP64 oracle.
//
//   api_dump <method> <matrix.mtx> <u_tile> <repeat> <out.bin>
//   method: mixed_radix | cufft_smooth | mixed_radix_graph | stockham_streaming
//   out.bin: int32 rows, cols, output_cols, then rows x output_cols complex64
//
// Compiled by tests/test_gpu_api.py against libgbspfft.so.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "mtx_reader.h"
#include "sparse_fft.h"

int main(int argc, char** argv) {
    if (argc != 6) {
        std::fprintf(stderr, "usage: %s <method> <matrix.mtx> <u_tile> <repeat> <out.bin>\n", argv[0]);
        return 2;
    }
    const std::string method = argv[1];
    const int u_tile = std::atoi(argv[3]), repeat = std::atoi(argv[4]);
    try {
        COOMatrix coo = read_mtx(argv[2]);
        SparseFFTResult r{};
        for (int i = 0; i < repeat; i++) {
            if (r.d_output) cudaFree(r.d_output);
            if (method == "mixed_radix") r = sparse_fft_csc_bluestein_mixed_radix(coo, u_tile);
            else if (method == "cufft_smooth") r = sparse_fft_csc_bluestein_cufft_smooth(coo, u_tile);
            else if (method == "mixed_radix_graph") r = sparse_fft_csc_bluestein_mixed_radix_graph(coo, u_tile);
            else if (method == "stockham_streaming") r = sparse_fft_csc_stockham_streaming(coo, u_tile);
            else {
                std::fprintf(stderr, "unknown method %s\n", method.c_str());
                return 2;
            }
            std::printf("call %d ms %.4f mem_bytes %zu output_cols %d\n", i, r.ms, r.mem_bytes, r.output_cols);
        }
        const size_t n = (size_t)coo.rows * r.output_cols;
        std::vector<float> h(2 * std::max<size_t>(n, 1));
        if (r.d_output) {
            if (cudaMemcpy(h.data(), r.d_output, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
            cudaFree(r.d_output);
        } else {
            std::memcpy(h.data(), r.h_output.data(), n * 8);
        }
        std::FILE* f = std::fopen(argv[5], "wb");
        if (!f) return 4;
        const int hdr[3] = {coo.rows, coo.cols, r.output_cols};
        std::fwrite(hdr, sizeof(int), 3, f);
        std::fwrite(h.data(), 8, n, f);
        std::fclose(f);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
