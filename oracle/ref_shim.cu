// ref_shim.cu -- TEST INFRASTRUCTURE ONLY.  Exposes the reference's own host
// functions for the hot path through a C ABI so the oracle and the library
// can be checked against them bit for bit.  It is compiled (by
// oracle/build_ref.sh) straight from the reference's sources where they lie;
// nothing here is a copy of them.  Only tests/ and the golden-fixture script
// load the resulting oracle/_ref/libref_host.so.
//
// The same file compiled with -fatbin gives oracle/_ref/ref_kernels.fatbin:
// the device code of the included reference translation unit, i.e. the
// reference's own GPU kernels, which oracle/ref_gpu_driver.cpp launches.
//
// Wrapped reference symbols:
//   read_mtx                    src/mtx_reader.cu:7-77
//   make_compact_csc            include/sparse_fft_internal.cuh:200-222
//   can_pack_u16 / pack_cols_u16 include/sparse_fft_internal.cuh:122-124, 146-151
//   make_bluestein_chirp / _b   include/sparse_fft_internal.cuh:168-191
//   next_3_smooth / next_7_smooth / factor_3_smooth
//                               src/sparse_fft_bluestein.cu:1975-2011
//   next_power_of_two           include/sparse_fft_internal.cuh:153-157
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>

// The reference translation unit itself (its static helpers become visible).
#include "sparse_fft_bluestein.cu"
#include "mtx_reader.cu"

static thread_local std::string g_err;

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

int ref_read_mtx(const char* path, int* rows, int* cols, int* nnz, int** r, int** c) {
    try {
        COOMatrix coo = read_mtx(path);
        *rows = coo.rows;
        *cols = coo.cols;
        *nnz = coo.nnz;
        *r = (int*)std::malloc(sizeof(int) * (coo.nnz ? coo.nnz : 1));
        *c = (int*)std::malloc(sizeof(int) * (coo.nnz ? coo.nnz : 1));
        std::memcpy(*r, coo.row_idx.data(), sizeof(int) * coo.nnz);
        std::memcpy(*c, coo.col_idx.data(), sizeof(int) * coo.nnz);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 1;
    }
}

void ref_free(void* p) { std::free(p); }

int ref_make_compact_csc(int rows, int cols, int nnz, const int* r, const int* c, int* n_active,
                         int* sparse_cols, int* col_ptr, int* row_idx) {
    COOMatrix coo;
    coo.rows = rows;
    coo.cols = cols;
    coo.nnz = nnz;
    coo.row_idx.assign(r, r + nnz);
    coo.col_idx.assign(c, c + nnz);
    CompactCSC csc = make_compact_csc(coo);
    *n_active = csc.n_sparse_cols;
    std::memcpy(sparse_cols, csc.sparse_cols.data(), sizeof(int) * csc.n_sparse_cols);
    std::memcpy(col_ptr, csc.col_ptr.data(), sizeof(int) * (csc.n_sparse_cols + 1));
    std::memcpy(row_idx, csc.row_idx.data(), sizeof(int) * nnz);
    return 0;
}

int ref_can_pack_u16(int rows, int cols) { return can_pack_u16(rows, cols) ? 1 : 0; }

void ref_pack_cols_u16(const int* in, int n, uint16_t* out) {
    std::vector<uint16_t> v = pack_cols_u16(in, n);
    std::memcpy(out, v.data(), sizeof(uint16_t) * n);
}

// interleaved (re, im) float pairs
void ref_bluestein_chirp(int n, float* out) {
    std::vector<cuFloatComplex> v = make_bluestein_chirp(n);
    std::memcpy(out, v.data(), sizeof(float) * 2 * n);
}

void ref_bluestein_b(int n, int fft_len, float* out) {
    std::vector<cuFloatComplex> v = make_bluestein_b(n, fft_len);
    std::memcpy(out, v.data(), sizeof(float) * 2 * fft_len);
}

int ref_next_3_smooth(int n) { return next_3_smooth(n); }
int ref_next_7_smooth(int n) { return next_7_smooth(n); }
int ref_next_power_of_two(int n) { return next_power_of_two(n); }

int ref_factor_3_smooth(int n, int* out, int cap) {
    try {
        std::vector<int> f = factor_3_smooth(n);
        if ((int)f.size() > cap) return -1;
        for (size_t i = 0; i < f.size(); i++) out[i] = f[i];
        return (int)f.size();
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

}  // extern "C"
