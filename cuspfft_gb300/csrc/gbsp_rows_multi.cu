// gbsp_rows_multi.cu -- the Bluestein row kernel for convolutions split into
// K channels run as one thread-block cluster (both block-size bounds), and
// the dispatch of the multi-channel modes; sequential channels compile in
// gbsp_rows_seq.cu.
#include "gbsp_rows_impl.cuh"

namespace gbsp {

int rows_capacity_multi(const RowsKernel& k, int sms, int* cap) {
    using namespace rows_impl;
    switch (k.mode) {
        case ROW_CLUSTER:
            return k.ntmax == 512 ? capacity<512, ROW_CLUSTER>(k, sms, cap) : capacity<1024, ROW_CLUSTER>(k, sms, cap);
        case ROW_SEQ:
        case ROW_SEQW:
            return rows_capacity_seq(k, sms, cap);
        default:
            return set_error(GBSP_ERR_INVALID, "row kernel: unknown channel mode");
    }
}

int rows_launch_multi(const RowsKernel& k, int grid, cudaStream_t st, const RowsArgs& a, const FFTDesc& fd,
                      int* err) {
    using namespace rows_impl;
    switch (k.mode) {
        case ROW_CLUSTER:
            return k.ntmax == 512 ? launch<512, ROW_CLUSTER>(k, grid, st, a, fd, err)
                                  : launch<1024, ROW_CLUSTER>(k, grid, st, a, fd, err);
        case ROW_SEQ:
        case ROW_SEQW:
            return rows_launch_seq(k, grid, st, a, fd, err);
        default:
            return set_error(GBSP_ERR_INVALID, "row kernel: unknown channel mode");
    }
}

}  // namespace gbsp
