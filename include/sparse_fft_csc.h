// sparse_fft_csc.h -- the compact-CSC builder of the hot path as a C++ API.
//
// Mirrors the reference's CompactCSC / make_compact_csc / can_pack_u16
// (include/sparse_fft_internal.cuh:122-124, :193-222), which the reference
// keeps in an internal header; here they are public so callers can inspect
// the exact index arrays the kernels consume.
#pragma once
#include <vector>
#include "mtx_reader.h"

struct CompactCSC {
    int n_sparse_cols = 0;         // number of active (non-empty) columns
    std::vector<int> sparse_cols;  // active column ids, ascending
    std::vector<int> col_ptr;      // n_sparse_cols + 1 offsets into row_idx
    std::vector<int> row_idx;      // row of each nonzero, grouped by active column
};

CompactCSC make_compact_csc(const COOMatrix& coo);

// 16-bit device indices are used when both dimensions fit.
inline bool can_pack_u16(int rows, int cols) { return rows <= 65536 && cols <= 65536; }
