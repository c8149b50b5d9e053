// host_reference.h -- the CLI's --cpu-reference spectrum: an FP64 host
// evaluation of the same 2-D R2C DFT, used only to print check lines.
//
// The reference fills this role with a single-threaded FFTW3f
// fftwf_plan_dft_r2c_2d (src/cpu_reference.cpp:8-63); FFTW is a third-party
// library this project does not link, so the CLI evaluates the transform
// directly in double precision: exact integer phases (u*r mod rows) along the
// rows, then a Bluestein FP64 FFT (radix-2 core) along the columns.
#pragma once
#include <cmath>
#include <complex>
#include <cstdint>
#include <vector>

#include "mtx_reader.h"
#include "sparse_fft_csc.h"

namespace gbsp_cli {

struct HostSpectrum {
    int rows = 0, freq_cols = 0;
    std::vector<std::complex<double>> data;  // rows x freq_cols, row-major
};

namespace detail {
using cd = std::complex<double>;

inline void fft_pow2(std::vector<cd>& a, bool inverse) {
    const size_t n = a.size();
    for (size_t i = 1, j = 0; i < n; i++) {
        size_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    for (size_t len = 2; len <= n; len <<= 1) {
        const double ang = 2.0 * M_PI / (double)len * (inverse ? 1 : -1);
        for (size_t i = 0; i < n; i += len)
            for (size_t k = 0; k < len / 2; k++) {
                cd w = std::polar(1.0, ang * (double)k);
                cd x = a[i + k], y = a[i + k + len / 2] * w;
                a[i + k] = x + y;
                a[i + k + len / 2] = x - y;
            }
    }
}

// DFT of length n of x via Bluestein with a power-of-two convolution.
struct Bluestein64 {
    size_t n = 0, m = 0;
    std::vector<cd> chirp, bfft;
    explicit Bluestein64(size_t n_) : n(n_) {
        m = 1;
        while (m < 2 * n - 1) m <<= 1;
        chirp.resize(n);
        for (size_t k = 0; k < n; k++) {
            uint64_t k2 = (uint64_t)k * k % (2 * n);
            chirp[k] = std::polar(1.0, -M_PI * (double)k2 / (double)n);
        }
        bfft.assign(m, cd(0, 0));
        bfft[0] = 1.0;
        for (size_t k = 1; k < n; k++) bfft[k] = bfft[m - k] = std::conj(chirp[k]);
        fft_pow2(bfft, false);
    }
    void run(const std::vector<cd>& x, std::vector<cd>& out, size_t n_out) const {
        std::vector<cd> a(m, cd(0, 0));
        for (size_t k = 0; k < n; k++) a[k] = x[k] * chirp[k];
        fft_pow2(a, false);
        for (size_t k = 0; k < m; k++) a[k] *= bfft[k];
        fft_pow2(a, true);
        for (size_t v = 0; v < n_out; v++) out[v] = a[v] * chirp[v] / (double)m;
    }
};
}  // namespace detail

inline HostSpectrum host_reference_fp64(const COOMatrix& coo) {
    using detail::cd;
    HostSpectrum hs;
    hs.rows = coo.rows;
    hs.freq_cols = coo.cols / 2 + 1;
    hs.data.assign((size_t)hs.rows * hs.freq_cols, cd(0, 0));
    CompactCSC csc = make_compact_csc(coo);
    std::vector<cd> tw(coo.rows);
    for (int p = 0; p < coo.rows; p++) tw[p] = std::polar(1.0, -2.0 * M_PI * (double)p / coo.rows);
    detail::Bluestein64 bl((size_t)coo.cols);
    std::vector<cd> s(coo.cols), f(hs.freq_cols);
    for (int u = 0; u < coo.rows; u++) {
        std::fill(s.begin(), s.end(), cd(0, 0));
        for (int j = 0; j < csc.n_sparse_cols; j++) {
            cd acc(0, 0);
            for (int p = csc.col_ptr[j]; p < csc.col_ptr[j + 1]; p++)
                acc += tw[(uint64_t)u * (uint64_t)csc.row_idx[p] % (uint64_t)coo.rows];
            s[csc.sparse_cols[j]] = acc;
        }
        bl.run(s, f, (size_t)hs.freq_cols);
        std::copy(f.begin(), f.end(), hs.data.begin() + (size_t)u * hs.freq_cols);
    }
    return hs;
}

}  // namespace gbsp_cli
