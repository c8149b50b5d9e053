// gbsp_host.cpp -- host-side input path of the C ABI: the binarizing Matrix
// Market reader, the compact-CSC builder, the smooth-length policy and the
// thread-local error channel.  Pure C++17, no CUDA.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "gbspfft.h"
#include "gbsp_internal.h"

namespace gbsp {

static thread_local std::string g_last_error;

int set_error(int status, const std::string& msg) {
    g_last_error = msg;
    return status;
}

long next_smooth(long n, int policy) {
    if (n < 1) n = 1;
    if (policy == GBSP_LEN_POW2) {
        long p = 1;
        while (p < n) p <<= 1;
        return p;
    }
    static const int p3[] = {2, 3};
    static const int p7[] = {2, 3, 5, 7};
    const int* ps = (policy == GBSP_LEN_7SMOOTH) ? p7 : p3;
    const int np = (policy == GBSP_LEN_7SMOOTH) ? 4 : 2;
    for (long m = n;; ++m) {
        long x = m;
        for (int i = 0; i < np; i++)
            while (x % ps[i] == 0) x /= ps[i];
        if (x == 1) return m;
    }
}

}  // namespace gbsp

using gbsp::set_error;

extern "C" {

int gbsp_version(void) { return 10000; }

const char* gbsp_status_string(int status) {
    switch (status) {
        case GBSP_OK: return "ok";
        case GBSP_ERR_INVALID: return "invalid argument";
        case GBSP_ERR_CUDA: return "CUDA error";
        case GBSP_ERR_ALLOC: return "allocation failed";
        case GBSP_ERR_UNSUPPORTED: return "unsupported shape";
        case GBSP_ERR_IO: return "I/O or parse error";
        case GBSP_ERR_NOT_BUILT: return "not in this library";
        default: return "unknown status";
    }
}

int gbsp_last_error(char* buf, size_t buflen) {
    if (!buf || buflen == 0) return GBSP_ERR_INVALID;
    size_t n = std::min(buflen - 1, gbsp::g_last_error.size());
    std::memcpy(buf, gbsp::g_last_error.data(), n);
    buf[n] = '\0';
    return GBSP_OK;
}

int gbsp_device_flags_status(int flags) {
    if (flags == 0) return GBSP_OK;
    std::string why;
    if (flags & 1) why += "a bounded device wait gave up";
    if (flags & 2) why += std::string(why.empty() ? "" : "; ") + "a stage radix the row kernel was not compiled for";
    if (flags & ~3) why += std::string(why.empty() ? "" : "; ") + "unknown bits";
    return set_error(GBSP_ERR_CUDA, "device error flags " + std::to_string(flags) + " (" + why +
                                        "): the transform's result is not valid");
}

int gbsp_next_smooth(int n, int policy) {
    if (policy != GBSP_LEN_3SMOOTH && policy != GBSP_LEN_7SMOOTH && policy != GBSP_LEN_POW2) return -1;
    long m = gbsp::next_smooth(n, policy);
    return m > 0x7fffffffL ? -1 : (int)m;
}

void gbsp_free(void* p) { std::free(p); }

// Matrix Market reader with the reference's semantics (src/mtx_reader.cu:7-77):
//  * line 1 must start with "%%MatrixMarket"; the file is symmetric when that
//    line contains "symmetric" or "Symmetric" (so skew-symmetric mirrors too);
//  * every following line that starts with '%' (or is empty) before the size
//    line is skipped;
//  * the size line gives rows, cols and the number of stored entries;
//  * each entry line contributes (r-1, c-1); its value, if any, is ignored,
//    and off-diagonal entries of symmetric files are mirrored;
//  * pairs are sorted (row, then column) and duplicates dropped.
int gbsp_read_mtx(const char* path, int* rows_out, int* cols_out, int* nnz_out,
                  int** row_idx, int** col_idx) {
    if (!path || !rows_out || !cols_out || !nnz_out || !row_idx || !col_idx)
        return set_error(GBSP_ERR_INVALID, "gbsp_read_mtx: null argument");
    *row_idx = nullptr;
    *col_idx = nullptr;
    std::ifstream f(path);
    if (!f.is_open()) return set_error(GBSP_ERR_IO, std::string("Cannot open file: ") + path);
    std::string line;
    if (!std::getline(f, line)) return set_error(GBSP_ERR_IO, std::string("Empty file: ") + path);
    if (line.compare(0, 14, "%%MatrixMarket") != 0)
        return set_error(GBSP_ERR_IO, std::string("Not a Matrix Market file: ") + path);
    const bool symmetric = line.find("symmetric") != std::string::npos ||
                           line.find("Symmetric") != std::string::npos;
    bool have_dims = false;
    while (std::getline(f, line)) {
        if (!line.empty() && line[0] != '%') { have_dims = true; break; }
    }
    long rows = 0, cols = 0, stored = 0;
    {
        std::istringstream ss(have_dims ? line : std::string());
        if (!(ss >> rows >> cols >> stored))
            return set_error(GBSP_ERR_IO, std::string("Bad dimension line in: ") + path);
    }
    if (rows < 0 || cols < 0 || stored < 0 || rows > 0x7fffffffL || cols > 0x7fffffffL)
        return set_error(GBSP_ERR_IO, std::string("Bad dimension line in: ") + path);
    std::vector<std::pair<int, int>> pairs;
    pairs.reserve((size_t)stored * (symmetric ? 2 : 1));
    for (long i = 0; i < stored; i++) {
        if (!std::getline(f, line))
            return set_error(GBSP_ERR_IO, std::string("Unexpected EOF in: ") + path);
        std::istringstream ss(line);
        long r, c;
        if (!(ss >> r >> c))
            return set_error(GBSP_ERR_IO, std::string("Bad entry line in: ") + path);
        // the reference does no bounds check; an out-of-range entry would be
        // undefined behaviour downstream, so it is rejected here
        if (r < 1 || c < 1 || r > rows || c > cols)
            return set_error(GBSP_ERR_IO, std::string("Entry out of range in: ") + path);
        pairs.emplace_back((int)(r - 1), (int)(c - 1));
        if (symmetric && r != c) pairs.emplace_back((int)(c - 1), (int)(r - 1));
    }
    std::sort(pairs.begin(), pairs.end());
    pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
    const size_t n = pairs.size();
    int* ri = (int*)std::malloc(std::max<size_t>(1, n) * sizeof(int));
    int* ci = (int*)std::malloc(std::max<size_t>(1, n) * sizeof(int));
    if (!ri || !ci) {
        std::free(ri);
        std::free(ci);
        return set_error(GBSP_ERR_ALLOC, "gbsp_read_mtx: out of host memory");
    }
    for (size_t i = 0; i < n; i++) { ri[i] = pairs[i].first; ci[i] = pairs[i].second; }
    *rows_out = (int)rows;
    *cols_out = (int)cols;
    *nnz_out = (int)n;
    *row_idx = ri;
    *col_idx = ci;
    return GBSP_OK;
}

// Compact CSC with the reference's layout (include/sparse_fft_internal.cuh:
// 102-120 and 193-222): the active columns are the sorted distinct column ids,
// col_ptr counts nonzeros per active column, and row_idx is filled by a
// stable pass over the COO order (so rows ascend inside a column whenever the
// COO is row-sorted, as gbsp_read_mtx returns it).
int gbsp_build_compact_csc(int rows, int cols, int nnz, const int* coo_row, const int* coo_col,
                           int* n_active_out, int* sparse_cols, int* col_ptr, int* row_idx_out) {
    if (rows < 0 || cols < 0 || nnz < 0 || !n_active_out || !sparse_cols || !col_ptr ||
        (nnz > 0 && (!coo_row || !coo_col || !row_idx_out)))
        return set_error(GBSP_ERR_INVALID, "gbsp_build_compact_csc: bad argument");
    for (int i = 0; i < nnz; i++) {
        if (coo_col[i] < 0 || coo_col[i] >= cols || coo_row[i] < 0 || coo_row[i] >= rows)
            return set_error(GBSP_ERR_INVALID, "gbsp_build_compact_csc: index out of range");
    }
    std::vector<int> slot(cols, -1);
    for (int i = 0; i < nnz; i++) slot[coo_col[i]] = 0;
    int na = 0;
    for (int c = 0; c < cols; c++)
        if (slot[c] == 0) { slot[c] = na; sparse_cols[na++] = c; }
    std::fill(col_ptr, col_ptr + na + 1, 0);
    for (int i = 0; i < nnz; i++) col_ptr[slot[coo_col[i]] + 1]++;
    for (int j = 0; j < na; j++) col_ptr[j + 1] += col_ptr[j];
    std::vector<int> next(col_ptr, col_ptr + na);
    for (int i = 0; i < nnz; i++) row_idx_out[next[slot[coo_col[i]]]++] = coo_row[i];
    *n_active_out = na;
    return GBSP_OK;
}

}  // extern "C"
