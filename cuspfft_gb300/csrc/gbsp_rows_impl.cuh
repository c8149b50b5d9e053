// gbsp_rows_impl.cuh -- launch helpers shared by the translation units that
// compile the multi-channel row kernels (gbsp_rows_multi.cu: clusters,
// gbsp_rows_seq.cu: sequential channels).
#pragma once
#include "gbsp_launch.h"

namespace gbsp {
namespace rows_impl {

// Launch configuration: clusters of K CTAs for ROW_CLUSTER.
inline cudaLaunchConfig_t config(const RowsKernel& k, unsigned grid, cudaStream_t st, cudaLaunchAttribute* attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(k.nt);
    cfg.dynamicSmemBytes = k.smem;
    cfg.stream = st;
    if (k.mode == ROW_CLUSTER) {
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = k.K;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    return cfg;
}

template <int NTMAX, int MODE>
int capacity(const RowsKernel& k, int sms, int* cap) {
    auto kern = k_bluestein_rows<NTMAX, MODE>;
    if (int rc = allow_full_smem((const void*)kern)) return rc;
    if (MODE == ROW_CLUSTER) {
        cudaLaunchAttribute attr[1];
        cudaLaunchConfig_t cfg = config(k, (unsigned)(k.K * sms), nullptr, attr);
        GB_CUDA(cudaOccupancyMaxActiveClusters(cap, kern, &cfg));
    } else {
        int nb = 0;
        GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, k.nt, k.smem));
        *cap = nb * sms;
    }
    return GBSP_OK;
}

template <int NTMAX, int MODE>
int launch(const RowsKernel& k, int grid, cudaStream_t st, const RowsArgs& a, const FFTDesc& fd, int* err) {
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = config(k, (unsigned)grid, st, attr);
    GB_CUDA(cudaLaunchKernelEx(&cfg, k_bluestein_rows<NTMAX, MODE>, a, fd, err));
    return GBSP_OK;
}

}  // namespace rows_impl
}  // namespace gbsp
