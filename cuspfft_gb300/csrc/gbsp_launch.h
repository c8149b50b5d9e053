// gbsp_launch.h -- host entry points of the kernel translation units.
//
// The kernels compile in separate translation units so the build runs them
// in parallel: pass 1 (gbsp_pass1.cu), single-channel rows and batches
// (gbsp_rows.cu), multi-channel rows (gbsp_rows_multi.cu).  The plan code
// (gbsp_plan.cu) reaches them through these functions.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "gbspfft.h"
#include "gbsp_internal.h"
#include "gbsp_kernels.cuh"

// Returns a GBSP_ERR_* status (with the message recorded) from the calling
// function when a CUDA runtime call fails.
#define GB_CUDA(call)                                                                         \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return gbsp::set_error(e_ == cudaErrorMemoryAllocation ? GBSP_ERR_ALLOC : GBSP_ERR_CUDA, \
                                   std::string(#call) + ": " + cudaGetErrorString(e_));      \
    } while (0)

namespace gbsp {

// Per-device limits, queried once per device.
struct DeviceLimits {
    size_t smem_optin = 0;
    int sms = 0;
};
int device_limits(int dev, DeviceLimits* out);

// Lets `kern` take all the opt-in shared memory of a CTA on the current
// device.  The limit is a property of the kernel, shared by every plan in the
// process; one fixed value keeps a later, smaller plan from invalidating an
// earlier one.  Done once per (kernel, device).
int allow_full_smem(const void* kern);

// ---- pass 1 (gbsp_pass1.cu, gbsp_pass1_exact.cu): one compiled kernel per
// (index bytes, table layout, 64-bit phases, rows per lane, phase mode)
struct P1Kernel {
    int idx_bytes, tab;
    bool big;
    int ku;
    bool exact;  // every twiddle an exact table lookup (no recurrence)
};
// CTAs of k_twiddle_sum resident per SM with `smem` bytes (raises the limit)
int p1_blocks_per_sm(const P1Kernel& k, size_t smem, int* nb);
int p1_launch(const P1Kernel& k, int grid, size_t smem, cudaStream_t st, const P1Args& a);
int p1_batch_blocks_per_sm(const P1Kernel& k, size_t smem, int* nb);
int p1_batch_launch(const P1Kernel& k, int grid, size_t smem, cudaStream_t st, const P1Args* args,
                    const long* item_begin, int nmat, unsigned long long* queue);

// ---- Bluestein rows: mode ROW_*, compiled block bound ntmax (512 or 1024)
struct RowsKernel {
    int mode, ntmax, K, nt;
    size_t smem;
};
// CTAs (single channel, sequential channels) or clusters resident at once
int rows_capacity(const RowsKernel& k, int sms, int* cap);
int rows_launch(const RowsKernel& k, int grid, cudaStream_t st, const RowsArgs& a, const FFTDesc& fd, int* err);
int rows_batch_blocks_per_sm(int nt, size_t smem, int* nb);
int rows_batch_launch(int grid, int nt, size_t smem, cudaStream_t st, const RowsBatch* descs, const long* row_begin,
                      int nmat, unsigned long long* queue, int* err);
// the multi-channel modes (clusters: gbsp_rows_multi.cu, sequential
// channels: gbsp_rows_seq.cu); rows_capacity / rows_launch forward to these
int rows_capacity_multi(const RowsKernel& k, int sms, int* cap);
int rows_launch_multi(const RowsKernel& k, int grid, cudaStream_t st, const RowsArgs& a, const FFTDesc& fd,
                      int* err);
int rows_capacity_seq(const RowsKernel& k, int sms, int* cap);
int rows_launch_seq(const RowsKernel& k, int grid, cudaStream_t st, const RowsArgs& a, const FFTDesc& fd, int* err);

}  // namespace gbsp
