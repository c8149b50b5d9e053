// mtx_reader.h -- binary sparse matrices and the Matrix Market reader.
//
// Same declarations as the reference's include/mtx_reader.h (the types are
// part of the drop-in boundary): COOMatrix (:7-13), read_mtx (:18),
// CSRMatrix / coo_to_csr (:22-30).  Implemented in
// cuspfft_gb300/csrc/sparse_fft_api.cu on top of gbsp_read_mtx (gbspfft.h).
#pragma once
#include <string>
#include <vector>

// A binary sparse matrix as (row, col) pairs; every stored value is 1.
struct COOMatrix {
    int rows;
    int cols;
    int nnz;
    std::vector<int> row_idx;
    std::vector<int> col_idx;
};

// Reads a coordinate Matrix Market file, drops the values (binarizes),
// mirrors off-diagonal entries of symmetric files, and returns the pairs
// sorted by (row, col) without duplicates.  Throws std::runtime_error on any
// open or parse failure.
COOMatrix read_mtx(const std::string& path);

// Row-compressed form; row_ptr has rows+1 entries.
struct CSRMatrix {
    int rows, cols, nnz;
    std::vector<int> row_ptr;
    std::vector<int> col_idx;
};

// Expects a row-sorted COO (read_mtx returns one).
CSRMatrix coo_to_csr(const COOMatrix& coo);
