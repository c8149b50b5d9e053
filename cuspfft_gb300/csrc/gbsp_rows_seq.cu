// gbsp_rows_seq.cu -- the Bluestein row kernel for convolutions split into
// K channels that one CTA runs in turn (512-thread bound; a separate instance
// above MAX_CHANNELS channels).
#include "gbsp_rows_impl.cuh"

namespace gbsp {

int rows_capacity_seq(const RowsKernel& k, int sms, int* cap) {
    return k.mode == ROW_SEQW ? rows_impl::capacity<512, ROW_SEQW>(k, sms, cap)
                              : rows_impl::capacity<512, ROW_SEQ>(k, sms, cap);
}

int rows_launch_seq(const RowsKernel& k, int grid, cudaStream_t st, const RowsArgs& a, const FFTDesc& fd, int* err) {
    return k.mode == ROW_SEQW ? rows_impl::launch<512, ROW_SEQW>(k, grid, st, a, fd, err)
                              : rows_impl::launch<512, ROW_SEQ>(k, grid, st, a, fd, err);
}

}  // namespace gbsp
