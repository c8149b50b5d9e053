// gbsp_rows.cu -- the single-channel row kernels, Bluestein and direct (both
// block-size bounds), the batched row kernel, and the host launch functions; the
// multi-channel modes compile in gbsp_rows_multi.cu.
#include "gbsp_launch.h"

namespace gbsp {
namespace {

template <int NTMAX, int MODE>
int single_capacity(const RowsKernel& k, int sms, int* cap) {
    auto kern = k_bluestein_rows<NTMAX, MODE>;
    if (int rc = allow_full_smem((const void*)kern)) return rc;
    int nb = 0;
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, k.nt, k.smem));
    *cap = nb * sms;
    return GBSP_OK;
}

template <int NTMAX, int MODE>
int single_launch(const RowsKernel& k, int grid, cudaStream_t st, const RowsArgs& a, const FFTDesc& fd, int* err) {
    k_bluestein_rows<NTMAX, MODE><<<grid, k.nt, k.smem, st>>>(a, fd, err);
    GB_CUDA(cudaGetLastError());
    return GBSP_OK;
}

}  // namespace

int rows_capacity(const RowsKernel& k, int sms, int* cap) {
    *cap = 0;
    if (k.mode == ROW_DIRECT)
        return k.ntmax == 512 ? single_capacity<512, ROW_DIRECT>(k, sms, cap)
                              : single_capacity<1024, ROW_DIRECT>(k, sms, cap);
    if (k.mode != ROW_SINGLE) return rows_capacity_multi(k, sms, cap);
    return k.ntmax == 512 ? single_capacity<512, ROW_SINGLE>(k, sms, cap)
                          : single_capacity<1024, ROW_SINGLE>(k, sms, cap);
}

int rows_launch(const RowsKernel& k, int grid, cudaStream_t st, const RowsArgs& a, const FFTDesc& fd, int* err) {
    if (k.mode == ROW_DIRECT)
        return k.ntmax == 512 ? single_launch<512, ROW_DIRECT>(k, grid, st, a, fd, err)
                              : single_launch<1024, ROW_DIRECT>(k, grid, st, a, fd, err);
    if (k.mode != ROW_SINGLE) return rows_launch_multi(k, grid, st, a, fd, err);
    return k.ntmax == 512 ? single_launch<512, ROW_SINGLE>(k, grid, st, a, fd, err)
                          : single_launch<1024, ROW_SINGLE>(k, grid, st, a, fd, err);
}

int rows_batch_blocks_per_sm(int nt, size_t smem, int* nb) {
    auto kern = k_bluestein_rows_batch<512>;
    if (int rc = allow_full_smem((const void*)kern)) return rc;
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(nb, kern, nt, smem));
    return GBSP_OK;
}

int rows_batch_launch(int grid, int nt, size_t smem, cudaStream_t st, const RowsBatch* descs, const long* row_begin,
                      int nmat, unsigned long long* queue, int* err) {
    k_bluestein_rows_batch<512><<<grid, nt, smem, st>>>(descs, row_begin, nmat, queue, err);
    GB_CUDA(cudaGetLastError());
    return GBSP_OK;
}

}  // namespace gbsp
