// gbsp_plan.cu -- plans and execution behind the C ABI (include/gbspfft.h).
//
// A plan owns everything the timed loop reads: the uploaded CSC (columns
// re-ordered into degree-sorted slots), the FP64-built tables rounded to
// FP32, and the pass-1 scratch tile.  Execution is two launches per tile of
// Bluestein rows: k_twiddle_sum (pass 1) and k_bluestein_rows (convolution +
// R2C writer).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gbspfft.h"
#include "gbsp_internal.h"
#include "gbsp_kernels.cuh"

using gbsp::set_error;

struct gbsp_plan_s {
    int device = 0;
    int rows = 0, cols = 0, nnz = 0, n_active = 0;
    int L = 0, K = 1, Lp = 0;
    gbsp::FFTDesc fd{};
    int half_rows = 0, u_tile = 0, out_cols = 0, out_pitch = 0;
    int idx_bytes = 2, tab_half = 0, big = 0, kahan_min = 64, ntab = 0;
    uint32_t rows_magic = 0;
    std::vector<int> slot_col_host;  // column of each slot
    int* d_slot_ptr = nullptr;       // n_active + 1
    void* d_row_idx = nullptr;       // nnz, u16 or u32, grouped by slot
    int* d_slot_col = nullptr;       // n_active
    float2* d_rowtab = nullptr;
    float2* d_pre = nullptr;         // K x n_active (slot order)
    float2* d_post = nullptr;        // K x cols
    float2* d_filt = nullptr;        // K x Lp (fused-stage thread order)
    float2* d_fftw = nullptr;        // stage twiddles, q-major blocks
    float2* d_S = nullptr;
    size_t s_pitch = 0;
    int p1_grid = 0;
    size_t p1_smem = 0;
    int rows_grid = 0;
    size_t rows_smem = 0;
    size_t device_bytes = 0;
    std::vector<void*> allocs;
};

namespace {

#define GB_CUDA(call)                                                                     \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return set_error(e_ == cudaErrorMemoryAllocation ? GBSP_ERR_ALLOC : GBSP_ERR_CUDA, \
                             std::string(#call) + ": " + cudaGetErrorString(e_));        \
    } while (0)

int dev_alloc(gbsp_plan_s* p, void** ptr, size_t bytes) {
    bytes = std::max<size_t>(bytes, 16);
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(GBSP_ERR_ALLOC, std::string("cudaMalloc(") + std::to_string(bytes) +
                                             "): " + cudaGetErrorString(e));
    }
    p->allocs.push_back(*ptr);
    p->device_bytes += bytes;
    return GBSP_OK;
}

void free_plan(gbsp_plan_s* p) {
    if (!p) return;
    for (void* a : p->allocs) cudaFree(a);
    delete p;
}

inline unsigned blocks_for(long n, int t) { return (unsigned)((n + t - 1) / t); }

// Radix plan for a 7-smooth channel length: radix-8 stages while three or
// more factors of 2 remain, then 4 or 2, then 3s, 5s and 7s (an odd radix
// last keeps the span-1 stage free of shared-memory bank conflicts).
int build_fft_desc(int Lp, gbsp::FFTDesc* fd) {
    int e2 = 0, e3 = 0, e5 = 0, e7 = 0, x = Lp;
    while (x % 2 == 0) { x /= 2; e2++; }
    while (x % 3 == 0) { x /= 3; e3++; }
    while (x % 5 == 0) { x /= 5; e5++; }
    while (x % 7 == 0) { x /= 7; e7++; }
    if (x != 1) return GBSP_ERR_UNSUPPORTED;
    std::vector<int> rs;
    while (e2 >= 3) { rs.push_back(8); e2 -= 3; }
    if (e2 == 2) rs.push_back(4);
    if (e2 == 1) rs.push_back(2);
    for (int i = 0; i < e3; i++) rs.push_back(3);
    for (int i = 0; i < e5; i++) rs.push_back(5);
    for (int i = 0; i < e7; i++) rs.push_back(7);
    if ((int)rs.size() > gbsp::MAX_STAGES || rs.empty()) return GBSP_ERR_UNSUPPORTED;
    fd->Lp = Lp;
    fd->nst = (int)rs.size();
    int l = 1, off = 0;
    for (int s = 0; s < fd->nst; s++) {
        const int R = rs[s];
        const int m = Lp / (l * R);
        fd->R[s] = R;
        fd->m[s] = m;
        fd->magic[s] = (m <= 1) ? 0u : (uint32_t)(((1ull << 32) + (uint64_t)m - 1) / (uint64_t)m);
        fd->twoff[s] = off;
        off += (R - 1) * m;
        l *= R;
    }
    fd->rest_base = (fd->R[0] - 1) * fd->m[0];
    fd->rest_len = off - fd->rest_base;
    return GBSP_OK;
}

int fft_tw_count(const gbsp::FFTDesc& fd) { return fd.rest_base + fd.rest_len; }

size_t rows_smem_bytes(const gbsp::FFTDesc& fd) {
    return ((size_t)gbsp::padded_len(fd.Lp) + (size_t)fd.rest_len) * sizeof(float2);
}

template <typename IDX, bool HALF, bool BIG>
int p1_prepare(gbsp_plan_s* p, int sms) {
    auto kern = gbsp::k_twiddle_sum<IDX, HALF, BIG>;
    GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->p1_smem));
    int nb = 0;
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, gbsp::P1_THREADS, p->p1_smem));
    if (nb < 1) return set_error(GBSP_ERR_UNSUPPORTED, "pass-1 kernel does not fit on an SM");
    p->p1_grid = nb * sms;
    return GBSP_OK;
}

template <typename IDX, bool HALF, bool BIG>
void p1_launch(const gbsp_plan_s* p, int u0, int n, float2* S, size_t s_pitch, cudaStream_t st) {
    gbsp::k_twiddle_sum<IDX, HALF, BIG><<<p->p1_grid, gbsp::P1_THREADS, p->p1_smem, st>>>(
        p->d_slot_ptr, (const IDX*)p->d_row_idx, p->n_active, p->d_rowtab, p->ntab, p->rows,
        p->rows_magic, u0, n, S, s_pitch, p->kahan_min);
}

// prepare == true: set attributes and grid; false: launch
template <bool HALF, bool BIG>
int p1_dispatch_idx(gbsp_plan_s* p, bool prepare, int sms, int u0, int n, float2* S, size_t sp,
                    cudaStream_t st) {
    if (p->idx_bytes == 2) {
        if (prepare) return p1_prepare<uint16_t, HALF, BIG>(p, sms);
        p1_launch<uint16_t, HALF, BIG>(p, u0, n, S, sp, st);
    } else {
        if (prepare) return p1_prepare<uint32_t, HALF, BIG>(p, sms);
        p1_launch<uint32_t, HALF, BIG>(p, u0, n, S, sp, st);
    }
    return GBSP_OK;
}

int p1_dispatch(gbsp_plan_s* p, bool prepare, int sms, int u0, int n, float2* S, size_t sp,
                cudaStream_t st) {
    if (p->tab_half) {
        if (p->big) return p1_dispatch_idx<true, true>(p, prepare, sms, u0, n, S, sp, st);
        return p1_dispatch_idx<true, false>(p, prepare, sms, u0, n, S, sp, st);
    }
    if (p->big) return p1_dispatch_idx<false, true>(p, prepare, sms, u0, n, S, sp, st);
    return p1_dispatch_idx<false, false>(p, prepare, sms, u0, n, S, sp, st);
}

int launch_pass1(const gbsp_plan_s* p, int u0, int n, float2* S, size_t sp, cudaStream_t st) {
    p1_dispatch(const_cast<gbsp_plan_s*>(p), false, 0, u0, n, S, sp, st);
    GB_CUDA(cudaGetLastError());
    return GBSP_OK;
}

int launch_rows(const gbsp_plan_s* p, int u0, int n, void* d_out, size_t out_pitch,
                cudaStream_t st) {
    if (p->K == 1) {
        gbsp::k_bluestein_rows<false><<<p->rows_grid, gbsp::ROWS_THREADS, p->rows_smem, st>>>(
            p->d_S, p->s_pitch, p->n_active, p->d_slot_col, p->d_pre, p->d_post, p->d_filt,
            p->d_fftw, p->fd, 1, p->rows, p->cols, u0, n, (float2*)d_out, out_pitch);
        GB_CUDA(cudaGetLastError());
        return GBSP_OK;
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    cfg.gridDim = dim3(p->rows_grid);
    cfg.blockDim = dim3(gbsp::ROWS_THREADS);
    cfg.dynamicSmemBytes = p->rows_smem;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = p->K;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    GB_CUDA(cudaLaunchKernelEx(&cfg, gbsp::k_bluestein_rows<true>, (const float2*)p->d_S,
                               p->s_pitch, p->n_active, (const int*)p->d_slot_col,
                               (const float2*)p->d_pre, (const float2*)p->d_post,
                               (const float2*)p->d_filt, (const float2*)p->d_fftw, p->fd, p->K,
                               p->rows, p->cols, u0, n, (float2*)d_out, out_pitch));
    return GBSP_OK;
}

int validate_csc(int rows, int cols, int n_active, int nnz, const int* col_ptr,
                 const int* row_idx, const int* sparse_cols) {
    if (rows < 1 || cols < 1 || nnz < 0 || n_active < 0 || n_active > cols)
        return set_error(GBSP_ERR_INVALID, "gbsp_plan_create: bad sizes");
    if (!col_ptr || (n_active > 0 && !sparse_cols) || (nnz > 0 && !row_idx))
        return set_error(GBSP_ERR_INVALID, "gbsp_plan_create: null CSC array");
    if (col_ptr[0] != 0 || col_ptr[n_active] != nnz)
        return set_error(GBSP_ERR_INVALID, "gbsp_plan_create: col_ptr must run from 0 to nnz");
    for (int j = 0; j < n_active; j++) {
        if (col_ptr[j + 1] < col_ptr[j])
            return set_error(GBSP_ERR_INVALID, "gbsp_plan_create: col_ptr not monotone");
        if (sparse_cols[j] < 0 || sparse_cols[j] >= cols || (j > 0 && sparse_cols[j] <= sparse_cols[j - 1]))
            return set_error(GBSP_ERR_INVALID, "gbsp_plan_create: sparse_cols not strictly increasing in [0,cols)");
    }
    for (int i = 0; i < nnz; i++)
        if (row_idx[i] < 0 || row_idx[i] >= rows)
            return set_error(GBSP_ERR_INVALID, "gbsp_plan_create: row index out of range");
    return GBSP_OK;
}

int plan_build(gbsp_plan_s* p, const int* col_ptr, const int* row_idx, const int* sparse_cols,
               const gbsp_options* o, cudaStream_t st) {
    const int policy = (o && o->length_policy) ? o->length_policy : GBSP_LEN_3SMOOTH;
    if (policy != GBSP_LEN_3SMOOTH && policy != GBSP_LEN_7SMOOTH)
        return set_error(GBSP_ERR_INVALID, "gbsp_plan_create: length_policy must be 3 or 7");
    GB_CUDA(cudaGetDevice(&p->device));
    cudaDeviceProp prop;
    GB_CUDA(cudaGetDeviceProperties(&prop, p->device));
    const size_t smem_cap = prop.sharedMemPerBlockOptin;
    const int sms = prop.multiProcessorCount;

    // ---- lengths and channel split
    long L = gbsp::next_smooth(2L * p->cols - 1, policy);
    if (L < 2) L = 2;
    if (L > (1L << 28)) return set_error(GBSP_ERR_UNSUPPORTED, "fft_len too large");
    p->L = (int)L;
    const int maxLp = (o && o->max_channel_len > 0) ? o->max_channel_len : 20736;
    p->K = 0;
    for (int k = 1; k <= gbsp::MAX_CHANNELS && !p->K; k++) {
        if (L % k || L / k > maxLp || L / k < 2) continue;
        gbsp::FFTDesc fd{};
        if (build_fft_desc((int)(L / k), &fd) != GBSP_OK) continue;
        if (rows_smem_bytes(fd) > smem_cap) continue;
        p->K = k;
        p->fd = fd;
    }
    if (p->K == 0)
        return set_error(GBSP_ERR_UNSUPPORTED,
                         "fft_len " + std::to_string(L) + " does not split into <= 8 channels of <= " +
                             std::to_string(maxLp) + " that fit in shared memory");
    p->Lp = (int)(L / p->K);

    p->half_rows = p->rows / 2 + 1;
    p->out_cols = p->cols / 2 + 1;
    p->out_pitch = (p->out_cols + 3) / 4 * 4;
    p->u_tile = (o && o->u_tile > 0) ? std::min(o->u_tile, p->half_rows) : p->half_rows;
    p->kahan_min = (o && o->kahan_min_degree != 0) ? o->kahan_min_degree : 64;
    if (p->kahan_min < 0) p->kahan_min = 0;  // 0 disables compensation in the kernel
    int ib = (o && o->index_bytes) ? o->index_bytes : ((p->rows <= 65536 && p->cols <= 65536) ? 2 : 4);
    if (ib != 2 && ib != 4) return set_error(GBSP_ERR_INVALID, "index_bytes must be 2 or 4");
    if (ib == 2 && p->rows > 65536) return set_error(GBSP_ERR_INVALID, "rows > 65536 need 4-byte indices");
    p->idx_bytes = ib;
    p->big = p->rows > 65535;
    p->rows_magic = (p->rows >= 2) ? (uint32_t)(((1ull << 32) + (uint64_t)p->rows - 1) / (uint64_t)p->rows) : 0u;

    // ---- pass-1 configuration: staging tile + twiddle table in shared memory
    const size_t tab_budget = smem_cap - gbsp::P1_STAGE_BYTES - 256;
    if ((size_t)p->rows * sizeof(float2) <= std::min<size_t>(tab_budget, 160 * 1024)) {
        p->tab_half = 0;
        p->ntab = p->rows;
    } else if ((size_t)(p->rows / 2 + 1) * sizeof(float2) <= tab_budget) {
        p->tab_half = 1;
        p->ntab = p->rows / 2 + 1;
    } else {
        return set_error(GBSP_ERR_UNSUPPORTED, "rows too large for a shared-memory twiddle table");
    }
    p->p1_smem = gbsp::P1_STAGE_BYTES + (size_t)p->ntab * sizeof(float2);
    int rc = p1_dispatch(p, true, sms, 0, 0, nullptr, 0, st);
    if (rc) return rc;

    // ---- row-kernel configuration
    p->rows_smem = rows_smem_bytes(p->fd);
    if (p->K == 1) {
        GB_CUDA(cudaFuncSetAttribute(gbsp::k_bluestein_rows<false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->rows_smem));
        int nb = 0;
        GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, gbsp::k_bluestein_rows<false>,
                                                              gbsp::ROWS_THREADS, p->rows_smem));
        if (nb < 1) return set_error(GBSP_ERR_UNSUPPORTED, "row kernel does not fit on an SM");
        p->rows_grid = nb * sms;
    } else {
        GB_CUDA(cudaFuncSetAttribute(gbsp::k_bluestein_rows<true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->rows_smem));
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute attr[1];
        cfg.gridDim = dim3(p->K * sms);
        cfg.blockDim = dim3(gbsp::ROWS_THREADS);
        cfg.dynamicSmemBytes = p->rows_smem;
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = p->K;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int ncl = 0;
        GB_CUDA(cudaOccupancyMaxActiveClusters(&ncl, gbsp::k_bluestein_rows<true>, &cfg));
        if (ncl < 1) return set_error(GBSP_ERR_UNSUPPORTED, "row-kernel cluster does not fit");
        p->rows_grid = ncl * p->K;
    }

    // ---- slots: active columns sorted by degree (descending, stable)
    const int na = p->n_active;
    std::vector<int> order(na);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (col_ptr[a + 1] - col_ptr[a]) > (col_ptr[b + 1] - col_ptr[b]);
    });
    std::vector<int> slot_ptr(na + 1, 0);
    p->slot_col_host.resize(na);
    std::vector<uint32_t> rows32(std::max(p->nnz, 1));
    for (int s = 0; s < na; s++) {
        const int j = order[s];
        p->slot_col_host[s] = sparse_cols[j];
        int w = slot_ptr[s];
        for (int e = col_ptr[j]; e < col_ptr[j + 1]; e++) rows32[w++] = (uint32_t)row_idx[e];
        slot_ptr[s + 1] = w;
    }
    if ((rc = dev_alloc(p, (void**)&p->d_slot_ptr, (size_t)(na + 1) * sizeof(int)))) return rc;
    if ((rc = dev_alloc(p, (void**)&p->d_slot_col, (size_t)std::max(na, 1) * sizeof(int)))) return rc;
    if ((rc = dev_alloc(p, &p->d_row_idx, (size_t)std::max(p->nnz, 1) * p->idx_bytes))) return rc;
    GB_CUDA(cudaMemcpyAsync(p->d_slot_ptr, slot_ptr.data(), (size_t)(na + 1) * sizeof(int),
                            cudaMemcpyHostToDevice, st));
    if (na > 0)
        GB_CUDA(cudaMemcpyAsync(p->d_slot_col, p->slot_col_host.data(), (size_t)na * sizeof(int),
                                cudaMemcpyHostToDevice, st));
    std::vector<uint16_t> r16;
    if (p->nnz > 0) {
        if (p->idx_bytes == 2) {
            r16.resize(p->nnz);
            for (int i = 0; i < p->nnz; i++) r16[i] = (uint16_t)rows32[i];
            GB_CUDA(cudaMemcpyAsync(p->d_row_idx, r16.data(), (size_t)p->nnz * 2,
                                    cudaMemcpyHostToDevice, st));
        } else {
            GB_CUDA(cudaMemcpyAsync(p->d_row_idx, rows32.data(), (size_t)p->nnz * 4,
                                    cudaMemcpyHostToDevice, st));
        }
    }

    // ---- tables (FP64 on the device, rounded to FP32)
    const int K = p->K, Lp = p->Lp, cols = p->cols;
    if ((rc = dev_alloc(p, (void**)&p->d_rowtab, (size_t)p->ntab * sizeof(float2)))) return rc;
    if ((rc = dev_alloc(p, (void**)&p->d_pre, (size_t)K * std::max(na, 1) * sizeof(float2)))) return rc;
    if ((rc = dev_alloc(p, (void**)&p->d_post, (size_t)K * cols * sizeof(float2)))) return rc;
    if ((rc = dev_alloc(p, (void**)&p->d_filt, (size_t)K * Lp * sizeof(float2)))) return rc;
    const int ntw = std::max(fft_tw_count(p->fd), 1);
    if ((rc = dev_alloc(p, (void**)&p->d_fftw, (size_t)ntw * sizeof(float2)))) return rc;

    gbsp::k_table_rows<<<blocks_for(p->ntab, 256), 256, 0, st>>>(p->d_rowtab, p->ntab, p->rows);
    GB_CUDA(cudaGetLastError());
    if (na > 0) {
        gbsp::k_table_pre<<<blocks_for((long)K * na, 256), 256, 0, st>>>(p->d_pre, p->d_slot_col, na,
                                                                          cols, p->L, K);
        GB_CUDA(cudaGetLastError());
    }
    gbsp::k_table_post<<<blocks_for((long)K * cols, 256), 256, 0, st>>>(p->d_post, cols, p->L, K);
    GB_CUDA(cudaGetLastError());
    for (int s = 0; s < p->fd.nst; s++) {
        const int n = (p->fd.R[s] - 1) * p->fd.m[s];
        if (n == 0) continue;
        gbsp::k_table_fft<<<blocks_for(n, 256), 256, 0, st>>>(p->d_fftw, Lp, p->fd.R[s], p->fd.m[s],
                                                               p->fd.twoff[s]);
        GB_CUDA(cudaGetLastError());
    }
    double2* d_spec = nullptr;
    GB_CUDA(cudaMalloc((void**)&d_spec, (size_t)K * Lp * sizeof(double2)));
    gbsp::k_table_filter_input<<<blocks_for((long)K * Lp, 256), 256, 0, st>>>(d_spec, cols, p->L, K, Lp);
    cudaError_t e = cudaGetLastError();
    for (int s = 0; s < p->fd.nst && e == cudaSuccess; s++) {
        const long nbf = (long)K * (Lp / p->fd.R[s]);
        gbsp::k_dif_stage_f64<<<blocks_for(nbf, 128), 128, 0, st>>>(d_spec, K, Lp, p->fd.R[s], p->fd.m[s]);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        gbsp::k_table_filter_final<<<blocks_for((long)K * Lp, 256), 256, 0, st>>>(
            p->d_filt, d_spec, K, Lp, p->fd.R[p->fd.nst - 1], 1.0 / (double)p->L);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_spec);
    if (e != cudaSuccess)
        return set_error(GBSP_ERR_CUDA, std::string("plan tables: ") + cudaGetErrorString(e));

    // ---- pass-1 scratch tile
    p->s_pitch = (size_t)std::max(na, 1);
    p->s_pitch = (p->s_pitch + 1) & ~(size_t)1;
    if ((rc = dev_alloc(p, (void**)&p->d_S, (size_t)p->u_tile * p->s_pitch * sizeof(float2)))) return rc;
    return GBSP_OK;
}

int check_out(const gbsp_plan_s* p, const void* d_out, size_t out_pitch, const char* who) {
    if (!p || !d_out) return set_error(GBSP_ERR_INVALID, std::string(who) + ": null argument");
    if (out_pitch < (size_t)p->out_cols || (out_pitch & 1))
        return set_error(GBSP_ERR_INVALID, std::string(who) + ": out_pitch must be even and >= cols/2+1");
    if (((uintptr_t)d_out & 15) != 0)
        return set_error(GBSP_ERR_INVALID, std::string(who) + ": d_out must be 16-byte aligned");
    return GBSP_OK;
}

}  // namespace

extern "C" {

int gbsp_plan_create(int rows, int cols, int n_active, int nnz, const int* col_ptr,
                     const int* row_idx, const int* sparse_cols, const gbsp_options* opts,
                     void* stream, gbsp_plan_t* plan) {
    if (!plan) return set_error(GBSP_ERR_INVALID, "gbsp_plan_create: plan is null");
    *plan = nullptr;
    int rc = validate_csc(rows, cols, n_active, nnz, col_ptr, row_idx, sparse_cols);
    if (rc) return rc;
    gbsp_plan_s* p = new (std::nothrow) gbsp_plan_s();
    if (!p) return set_error(GBSP_ERR_ALLOC, "gbsp_plan_create: out of host memory");
    p->rows = rows;
    p->cols = cols;
    p->nnz = nnz;
    p->n_active = n_active;
    rc = plan_build(p, col_ptr, row_idx, sparse_cols, opts, (cudaStream_t)stream);
    if (rc) {
        free_plan(p);
        return rc;
    }
    *plan = p;
    return GBSP_OK;
}

int gbsp_plan_get_info(gbsp_plan_t p, gbsp_plan_info* info) {
    if (!p || !info) return set_error(GBSP_ERR_INVALID, "gbsp_plan_get_info: null argument");
    std::memset(info, 0, sizeof(*info));
    info->rows = p->rows;
    info->cols = p->cols;
    info->nnz = p->nnz;
    info->n_active = p->n_active;
    info->fft_len = p->L;
    info->channels = p->K;
    info->channel_len = p->Lp;
    info->n_stages = p->fd.nst;
    for (int s = 0; s < p->fd.nst; s++) info->radix[s] = p->fd.R[s];
    info->output_cols = p->out_cols;
    info->output_pitch = p->out_pitch;
    info->half_rows = p->half_rows;
    info->u_tile = p->u_tile;
    info->index_bytes = p->idx_bytes;
    info->row_table_mode = p->tab_half;
    info->device_bytes = p->device_bytes;
    return GBSP_OK;
}

int gbsp_plan_slot_columns(gbsp_plan_t p, int* cols_out) {
    if (!p || (!cols_out && p->n_active > 0))
        return set_error(GBSP_ERR_INVALID, "gbsp_plan_slot_columns: null argument");
    std::copy(p->slot_col_host.begin(), p->slot_col_host.end(), cols_out);
    return GBSP_OK;
}

int gbsp_plan_destroy(gbsp_plan_t p) {
    free_plan(p);
    return GBSP_OK;
}

int gbsp_execute(gbsp_plan_t p, void* d_out, size_t out_pitch, void* stream) {
    int rc = check_out(p, d_out, out_pitch, "gbsp_execute");
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    for (int u0 = 0; u0 < p->half_rows; u0 += p->u_tile) {
        const int n = std::min(p->u_tile, p->half_rows - u0);
        if ((rc = launch_pass1(p, u0, n, p->d_S, p->s_pitch, st))) return rc;
        if ((rc = launch_rows(p, u0, n, d_out, out_pitch, st))) return rc;
    }
    return GBSP_OK;
}

int gbsp_execute_profiled(gbsp_plan_t p, void* d_out, size_t out_pitch, void* stream,
                          float* ms_pass1, float* ms_rows) {
    int rc = check_out(p, d_out, out_pitch, "gbsp_execute_profiled");
    if (rc) return rc;
    if (!ms_pass1 || !ms_rows) return set_error(GBSP_ERR_INVALID, "gbsp_execute_profiled: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    const int ntiles = (p->half_rows + p->u_tile - 1) / p->u_tile;
    std::vector<cudaEvent_t> ev(2 * ntiles + 1, nullptr);
    for (auto& e : ev) {
        if (cudaEventCreate(&e) != cudaSuccess) { e = nullptr; rc = GBSP_ERR_CUDA; }
    }
    if (rc == GBSP_OK && cudaEventRecord(ev[0], st) != cudaSuccess) rc = GBSP_ERR_CUDA;
    for (int t = 0; t < ntiles && rc == GBSP_OK; t++) {
        const int u0 = t * p->u_tile;
        const int n = std::min(p->u_tile, p->half_rows - u0);
        rc = launch_pass1(p, u0, n, p->d_S, p->s_pitch, st);
        if (rc == GBSP_OK && cudaEventRecord(ev[2 * t + 1], st) != cudaSuccess) rc = GBSP_ERR_CUDA;
        if (rc == GBSP_OK) rc = launch_rows(p, u0, n, d_out, out_pitch, st);
        if (rc == GBSP_OK && cudaEventRecord(ev[2 * t + 2], st) != cudaSuccess) rc = GBSP_ERR_CUDA;
    }
    if (rc == GBSP_OK && cudaEventSynchronize(ev[2 * ntiles]) != cudaSuccess) rc = GBSP_ERR_CUDA;
    float a = 0.f, b = 0.f;
    for (int t = 0; t < ntiles && rc == GBSP_OK; t++) {
        float x = 0.f, y = 0.f;
        cudaEventElapsedTime(&x, ev[2 * t], ev[2 * t + 1]);
        cudaEventElapsedTime(&y, ev[2 * t + 1], ev[2 * t + 2]);
        a += x;
        b += y;
    }
    for (auto e : ev)
        if (e) cudaEventDestroy(e);
    if (rc != GBSP_OK) return set_error(rc, "gbsp_execute_profiled: CUDA failure");
    *ms_pass1 = a;
    *ms_rows = b;
    return GBSP_OK;
}

int gbsp_column_sums(gbsp_plan_t p, int u0, int n_rows, void* d_s, size_t s_pitch, void* stream) {
    if (!p || !d_s) return set_error(GBSP_ERR_INVALID, "gbsp_column_sums: null argument");
    if (u0 < 0 || n_rows < 1 || u0 + n_rows > p->rows || s_pitch < (size_t)std::max(p->n_active, 1))
        return set_error(GBSP_ERR_INVALID, "gbsp_column_sums: bad range or pitch");
    return launch_pass1(p, u0, n_rows, (float2*)d_s, s_pitch, (cudaStream_t)stream);
}

}  // extern "C"
