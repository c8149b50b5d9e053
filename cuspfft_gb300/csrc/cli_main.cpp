// cli_main.cpp -- command-line driver with the reference's flags and output
// lines (reference src/main.cu:217-311 for the flags, :74-83 for the timing
// line, :208-215 for the check line), so its sweep scripts parse our output.
//
//   cuspfft_gb300 <matrix.mtx> [--csc-mixed-radix] [--csc-cufft-smooth]
//                 [--csc-mixed-radix-graph] [--csc-tile N] [--repeat N]
//                 [--sparse-only] [--dense-only] [--cpu-reference] ...
//
// Methods the reference offers but this library does not implement print the
// reference's failure row ("<label>  OOM  OOM  [reason]").
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbspfft.h"
#include "host_reference.h"
#include "sparse_fft.h"

namespace {

// 1 untimed warm-up then n timed runs when n > 1; median (times[n/2]), min
// and max of the timed runs (reference src/main.cu:45-70).
SparseFFTResult run_repeated(int n, const std::function<SparseFFTResult()>& fn, float* mn,
                             float* mx) {
    SparseFFTResult res{};
    std::vector<float> times;
    if (n > 1) {
        res = fn();
        if (res.d_output) { cudaFree(res.d_output); res.d_output = nullptr; }
    }
    for (int i = 0; i < n; i++) {
        if (res.d_output) cudaFree(res.d_output);
        res = fn();
        times.push_back(res.ms);
    }
    if (n > 1) {
        std::sort(times.begin(), times.end());
        res.ms = times[n / 2];
        *mn = times.front();
        *mx = times.back();
    }
    return res;
}

void print_bench(const char* label, float ms, size_t mem, int n, float mn, float mx) {
    if (n > 1)
        printf("%-26s  %10.3f  %12.2f  [min %.3f, max %.3f]  n=%d\n", label, ms, mem / 1e6, mn, mx, n);
    else
        printf("%-26s  %10.3f  %12.2f\n", label, ms, mem / 1e6);
}

void print_fail(const char* label, const std::string& why) {
    printf("%-26s  %10s  %12s  [%s]\n", label, "OOM", "OOM", why.c_str());
}

// max_abs, max_rel (|d| / max(1,|ref|)) and rms_abs over rows x (cols/2+1)
// (reference src/main.cu:168-206).
void print_check(const char* method, const gbsp_cli::HostSpectrum& ref, const SparseFFTResult& r) {
    if (ref.rows == 0) return;
    const int fc = ref.freq_cols;
    std::vector<float> h((size_t)ref.rows * fc * 2);
    if (!r.h_output.empty()) {  // streamed methods return the spectrum on the host
        for (int row = 0; row < ref.rows; row++)
            std::memcpy(h.data() + (size_t)row * fc * 2, r.h_output.data() + (size_t)row * r.output_cols,
                        (size_t)fc * 8);
    } else {
        cudaError_t e = cudaMemcpy2D(h.data(), (size_t)fc * 8, r.d_output, (size_t)r.output_cols * 8,
                                     (size_t)fc * 8, ref.rows, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e));
    }
    double max_abs = 0, max_rel = 0, sum_sq = 0;
    const size_t n = (size_t)ref.rows * fc;
    for (size_t i = 0; i < n; i++) {
        double dx = (double)h[2 * i] - ref.data[i].real();
        double dy = (double)h[2 * i + 1] - ref.data[i].imag();
        double a = std::sqrt(dx * dx + dy * dy);
        double m = std::abs(ref.data[i]);
        max_abs = std::max(max_abs, a);
        max_rel = std::max(max_rel, a / std::max(1.0, m));
        sum_sq += a * a;
    }
    printf("  check %-19s  max_abs %.3e  max_rel %.3e  rms_abs %.3e\n", method, max_abs, max_rel,
           std::sqrt(sum_sq / (double)n));
}

void usage(const char* prog) {
    fprintf(stderr,
            "Usage: %s <matrix.mtx> [options]\n"
            "Options:\n"
            "  --sparse-only    Skip the dense baseline row\n"
            "  --dense-only     Skip sparse FFT methods\n"
            "  --csc-mixed-radix  Binary CSC + Bluestein, fft_len next 3-smooth (sm_103a kernels)\n"
            "  --csc-mixed-radix-graph  Same, replayed as one CUDA graph\n"
            "  --csc-cufft-smooth  Binary CSC + Bluestein, fft_len next 7-smooth (own kernels, no cuFFT)\n"
            "  --csc-stockham-smem  Binary CSC + Bluestein, fft_len next power of two\n"
            "  --csc-stockham-cufft  Same length (own kernels, no cuFFT)\n"
            "  --csc-stockham-stream  Streaming variant: tiles copied to pinned host memory (power of two)\n"
            "  --csc-stockham-cufft-stream  Streaming variant, power-of-two length (own kernels, no cuFFT)\n"
            "  --csc-binary-lut  Streaming, power-of-two length (pass 1: exact twiddle table)\n"
            "  --csc-binary-stockham-smem  Non-streaming, power-of-two length (same pass 1)\n"
            "  --csc-tile N     Bluestein rows per tile (default: 1024)\n"
            "  --cpu-reference  Host FP64 reference spectrum; every method is checked against it\n"
            "  --repeat N       1 warm-up + N timed runs; report median, min, max (default 1)\n"
            "  (--csc-bluestein --csc-stockham --csc-stockham-graph, which select nothing in the\n"
            "   reference CLI, and --spfft are accepted and report 'not in this library')\n",
            prog);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) { usage(argv[0]); return 1; }
    const std::string first(argv[1]);
    if (first == "--help" || first == "-h") { usage(argv[0]); return 0; }

    bool run_dense = true, run_sparse = true;
    bool mixed = false, mixed_graph = false, smooth = false, cpu_ref = false, stream3 = false, stream7 = false;
    bool stk_smem = false, stk_cufft = false, bin_lut = false, bin_smem = false;
    std::vector<std::string> unbuilt;
    int tile = 1024, repeat = 1;
    try {
        for (int i = 2; i < argc; i++) {
            std::string f(argv[i]);
            if (f == "--sparse-only") run_dense = false;
            else if (f == "--dense-only") run_sparse = false;
            else if (f == "--csc-mixed-radix") mixed = true;
            else if (f == "--csc-mixed-radix-graph") mixed_graph = true;
            else if (f == "--csc-cufft-smooth") smooth = true;
            else if (f == "--cpu-reference") cpu_ref = true;
            else if (f == "--csc-stockham-stream") stream3 = true;
            else if (f == "--csc-stockham-cufft-stream") stream7 = true;
            else if (f == "--csc-stockham-smem") stk_smem = true;
            else if (f == "--csc-stockham-cufft") stk_cufft = true;
            else if (f == "--csc-binary-lut") bin_lut = true;
            else if (f == "--csc-binary-stockham-smem") bin_smem = true;
            else if (f == "--csc-tile" || f == "--repeat") {
                if (++i >= argc) throw std::runtime_error(f + " requires an integer value");
                int v = std::stoi(argv[i]);
                if (v <= 0) throw std::runtime_error(f + " must be positive");
                (f == "--csc-tile" ? tile : repeat) = v;
            } else if (f == "--csc-bluestein" || f == "--csc-stockham" || f == "--csc-stockham-graph" ||
                       f == "--spfft") {
                unbuilt.push_back(f);
            } else {
                throw std::runtime_error("Unknown option: " + f);
            }
        }
    } catch (const std::exception& e) {
        fprintf(stderr, "Fatal error: %s\n", e.what());
        return 1;
    }

    try {
        printf("Matrix: %s\n", argv[1]);
        COOMatrix coo = read_mtx(argv[1]);
        printf("Size:   %d x %d\n", coo.rows, coo.cols);
        printf("nnz:    %d  (density %.4f%%)\n\n", coo.nnz,
               100.0 * coo.nnz / ((double)coo.rows * coo.cols));
        printf("%-26s  %10s  %12s\n", "Method", "Time (ms)", "Mem (MB)");
        printf("%-26s  %10s  %12s\n", "--------------------------", "----------", "------------");

        gbsp_cli::HostSpectrum ref;
        if (cpu_ref) {
            try {
                auto t0 = std::chrono::steady_clock::now();
                ref = gbsp_cli::host_reference_fp64(coo);
                double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
                printf("%-26s  %10.3f  %12.2f  [CPU, FP64 host, single-thread]\n", "CPU reference (FP64)",
                       (float)ms, ref.data.size() * 16 / 1e6);
            } catch (const std::exception& e) {
                printf("%-26s  %10s  %12s  [%s]\n", "CPU reference (FP64)", "FAIL", "FAIL", e.what());
            }
        }
        if (run_dense) print_fail("Dense cuFFT (baseline)", "not in this library");

        struct M { bool on; const char* label; const char* check; std::function<SparseFFTResult()> fn; };
        // rows in the reference CLI's order (src/main.cu:480-700)
        std::vector<M> methods = {
            {mixed, "Sparse CSC (mixed-radix)", "Sparse CSC mixed-radix",
             [&] { return sparse_fft_csc_bluestein_mixed_radix(coo, tile); }},
            {smooth, "Sparse CSC (cufft smooth)", "Sparse CSC cufft smooth",
             [&] { return sparse_fft_csc_bluestein_cufft_smooth(coo, tile); }},
            {stk_smem, "Sparse CSC (Stk smem)", "Sparse CSC Stk smem",
             [&] { return sparse_fft_csc_bluestein_smem(coo, tile); }},
            {stk_cufft, "Sparse CSC (Bluestein+cufft)", "Sparse CSC Bluestein+cufft",
             [&] { return sparse_fft_csc_bluestein_cufft(coo, tile); }},
            {stream3, "Sparse CSC (Stockham strm)", "Sparse CSC Stockham strm",
             [&] { return sparse_fft_csc_stockham_streaming(coo, tile, 0); }},
            {stream7, "Sparse CSC (cufft stream)", "Sparse CSC cufft stream",
             [&] { return sparse_fft_csc_bluestein_cufft_streaming(coo, tile); }},
            {bin_lut, "Sparse CSC (binary LUT)", "Sparse CSC binary LUT",
             [&] { return sparse_fft_csc_bluestein_binary_lut(coo, tile); }},
            {mixed_graph, "Sparse CSC (mr-graph)", "Sparse CSC mr-graph",
             [&] { return sparse_fft_csc_bluestein_mixed_radix_graph(coo, tile); }},
            {bin_smem, "Sparse CSC (binary Stk smem)", "Sparse CSC binary Stk smem",
             [&] { return sparse_fft_csc_stockham_binary_smem(coo, tile); }},
        };
        for (auto& m : methods) {
            if (!run_sparse || !m.on) continue;
            try {
                float mn = 0, mx = 0;
                SparseFFTResult r = run_repeated(repeat, m.fn, &mn, &mx);
                print_bench(m.label, r.ms, r.mem_bytes, repeat, mn, mx);
                print_check(m.check, ref, r);
                cudaFree(r.d_output);
            } catch (const std::exception& e) {
                print_fail(m.label, e.what());
                cudaGetLastError();
            }
        }
        if (run_sparse)
            for (auto& f : unbuilt) print_fail(f.c_str(), "not in this library");
        printf("\n");
    } catch (const std::exception& e) {
        fprintf(stderr, "Fatal error: %s\n", e.what());
        return 1;
    }
    return 0;
}
