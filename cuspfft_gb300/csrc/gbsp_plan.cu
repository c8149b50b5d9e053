// gbsp_plan.cu -- plans and execution behind the C ABI (include/gbspfft.h).
//
// A plan owns everything the timed loop reads: the uploaded CSC, the
// per-window column order of pass 1, the FP64-built tables rounded to FP32,
// and the pass-1 scratch tile.  Execution is two launches per tile of
// Bluestein rows: k_twiddle_sum (pass 1) and k_bluestein_rows (convolution +
// R2C writer).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gbspfft.h"
#include "gbsp_internal.h"
#include "gbsp_launch.h"
#include "gbsp_planner.h"
#include "gbsp_tables.cuh"

using gbsp::DeviceLimits;
using gbsp::device_limits;
using gbsp::set_error;
using gbsp::rows_smem_bytes;
using gbsp::fft_tw_count;
using gbsp::max_radix_for;

struct gbsp_plan_s {
    int device = 0;
    int rows = 0, cols = 0, nnz = 0, n_active = 0;
    int L = 0, K = 1, Lp = 0;
    gbsp::FFTDesc fd{};
    int half_rows = 0, u_tile = 0, out_cols = 0, out_pitch = 0;
    int idx_bytes = 2, tab_mode = 0, big = 0, kahan_min = 64, ntab = 0;  // tab_mode: gbsp::TAB_*
    int exact = 0;                   // pass-1 twiddles all exact table lookups (no recurrence)
    int direct = 0;                  // one forward FFT of length cols per row (cols smooth), no Bluestein
    int* d_drev = nullptr;           // direct: where the forward network leaves each frequency
    int p1_ku = 8, p1_cw = 32;       // pass-1 rows per lane (x32 per item) and window width
    int p1_shape = 1;                // 1-based index of (p1_ku, p1_cw, tab_mode) in the shape table
    int planner = GBSP_PLANNER_MODEL;
    uint32_t rows_magic = 0;
    unsigned long long rows_magic64 = 0;  // ceil(2^64 / rows)
    void* d_row_idx = nullptr;       // nnz, u16 or u32, column order
    uint8_t* d_win_slot0 = nullptr;  // pass-1 windows: first tile column of each column
    int2* d_win_task = nullptr;      // pass-1 windows: nonzero range of each task
    uint8_t* d_win_task_col = nullptr;  // pass-1 windows: tile column of each task
    int s_cols = 0;                  // columns pass 1 writes per S row (cols rounded up to even)
    int* d_err = nullptr;            // kernel error flags (bounded waits that timed out)
    float2* d_rowtab = nullptr;
    float2* d_pre = nullptr;         // K x cols channel pre-twiddles W_L^{c*q}
    float2* d_post = nullptr;        // K x cols
    float2* d_filt = nullptr;        // K x Lp (fused-stage thread order)
    float2* d_fftw = nullptr;        // stage twiddles, q-major blocks
    float2* d_S = nullptr;
    size_t s_pitch = 0;
    int p1_grid = 0;
    size_t p1_smem = 0;
    int rows_grid = 0, rows_threads = 1024, rows_ntmax = 1024;
    int row_mode = 0;                // gbsp::ROW_SINGLE / ROW_DIRECT / ROW_CLUSTER / ROW_SEQ / ROW_SEQW
    float2* d_zscratch = nullptr;    // ROW_SEQ: rows_grid x (K-1) x Lp channel results
    size_t rows_smem = 0;
    size_t device_bytes = 0;
    std::vector<void*> allocs;
    char* arena = nullptr;           // one allocation carved into the plan's buffers
    size_t arena_size = 0, arena_off = 0;
    // streaming to the host (gbsp_execute_to_host), created on first use and
    // kept: copy stream, per-slab events, two device slabs
    cudaStream_t stream_cs = nullptr;
    cudaEvent_t stream_done[2] = {nullptr, nullptr}, stream_copied[2] = {nullptr, nullptr};
    void* stream_slab[2] = {nullptr, nullptr};
    size_t stream_slab_bytes = 0;
    int stream_tile_auto = 1;        // tile_rows 0 of gbsp_execute_to_host
    int sms = 1;                     // the device's SM count
    bool stream_slab_owned = false;  // allocated on first use (else carved from the arena)
    bool arena_pooled = false;       // arena from the library's memory pool (else cudaMalloc)
};

namespace {

// Carves `bytes` (256-byte aligned) from the plan's arena when it has room,
// else allocates on its own.
int dev_alloc(gbsp_plan_s* p, void** ptr, size_t bytes) {
    bytes = std::max<size_t>(bytes, 16);
    const size_t need = (bytes + 255) & ~(size_t)255;
    if (p->arena && p->arena_off + need <= p->arena_size) {
        *ptr = p->arena + p->arena_off;
        p->arena_off += need;
        return GBSP_OK;
    }
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

// ---- plan memory: one stream-ordered pool per device, private to the
// library, that keeps up to g_cache_limit bytes of freed plan memory for the
// next plan (a cudaMalloc and a cudaFree of a plan's arena cost ~0.1 ms each).
// The pool's release threshold counts the memory in use too, so it is kept
// at the live plans' bytes plus the cache limit: with a large plan alive, a
// smaller one created and destroyed beside it still reuses its memory (a
// fixed 1 GiB threshold released and re-reserved it every time: 16706^2
// plan build 0.25 -> 0.61 ms and release 0.02 -> 0.56 ms beside a resident
// plan).
constexpr int MAX_POOL_DEVICES = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pool[MAX_POOL_DEVICES] = {};
unsigned long long g_pool_live[MAX_POOL_DEVICES] = {};
unsigned long long g_cache_limit = 1ull << 30;

// adds delta bytes of live plan memory on device dev and moves its pool's
// release threshold to live + cache limit (g_pool_mu held)
void pool_account_locked(int dev, long long delta) {
    if (dev < 0 || dev >= MAX_POOL_DEVICES || !g_pool[dev]) return;
    g_pool_live[dev] = (unsigned long long)((long long)g_pool_live[dev] + delta);
    unsigned long long thr = g_pool_live[dev] + g_cache_limit;
    cudaMemPoolSetAttribute(g_pool[dev], cudaMemPoolAttrReleaseThreshold, &thr);
}
void pool_account(int dev, long long delta) {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    pool_account_locked(dev, delta);
}

// *pool = the device's plan pool (created on first use), or nullptr for a
// device number the table does not cover (plain cudaMalloc then)
int plan_pool(int dev, cudaMemPool_t* pool) {
    *pool = nullptr;
    if (dev < 0 || dev >= MAX_POOL_DEVICES) return GBSP_OK;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pool[dev]) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t mp = nullptr;
        GB_CUDA(cudaMemPoolCreate(&mp, &props));
        unsigned long long thr = g_cache_limit;
        GB_CUDA(cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &thr));
        g_pool[dev] = mp;
    }
    *pool = g_pool[dev];
    return GBSP_OK;
}

// *hs = the device's helper stream for plan-build work that runs beside the
// caller's stream (created on first use), or nullptr (run on the caller's)
cudaStream_t g_helper[MAX_POOL_DEVICES] = {};
int helper_stream(int dev, cudaStream_t* hs) {
    *hs = nullptr;
    if (dev < 0 || dev >= MAX_POOL_DEVICES) return GBSP_OK;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_helper[dev]) GB_CUDA(cudaStreamCreateWithFlags(&g_helper[dev], cudaStreamNonBlocking));
    *hs = g_helper[dev];
    return GBSP_OK;
}

// the streaming path's copy stream and events, created once per plan
int stream_objects(gbsp_plan_s* p) {
    if (p->stream_cs) return GBSP_OK;
    GB_CUDA(cudaStreamCreateWithFlags(&p->stream_cs, cudaStreamNonBlocking));
    for (int b = 0; b < 2; b++) {
        GB_CUDA(cudaEventCreateWithFlags(&p->stream_done[b], cudaEventDisableTiming));
        GB_CUDA(cudaEventCreateWithFlags(&p->stream_copied[b], cudaEventDisableTiming));
    }
    return GBSP_OK;
}

void free_plan(gbsp_plan_s* p) {
    if (!p) return;
    if (p->arena && p->arena_pooled) {
        // the plan's kernels may run on any stream: wait for the plan's
        // device, as cudaFree would, before the arena goes back to its pool
        int cur = -1;
        cudaGetDevice(&cur);
        if (cur != p->device) cudaSetDevice(p->device);
        cudaDeviceSynchronize();
        pool_account(p->device, -(long long)p->arena_size);
        cudaFreeAsync(p->arena, 0);
        cudaStreamSynchronize(0);
        if (cur >= 0 && cur != p->device) cudaSetDevice(cur);
    }
    for (void* a : p->allocs) cudaFree(a);
    for (int b = 0; b < 2; b++) {
        if (p->stream_slab[b] && p->stream_slab_owned) cudaFree(p->stream_slab[b]);
        if (p->stream_done[b]) cudaEventDestroy(p->stream_done[b]);
        if (p->stream_copied[b]) cudaEventDestroy(p->stream_copied[b]);
    }
    if (p->stream_cs) cudaStreamDestroy(p->stream_cs);
    delete p;
}

inline unsigned blocks_for(long n, int t) { return (unsigned)((n + t - 1) / t); }

gbsp::P1Kernel p1_kernel(const gbsp_plan_s* p) {
    return gbsp::P1Kernel{p->idx_bytes, p->tab_mode, p->big != 0, p->p1_ku, p->exact != 0};
}

// sizes pass 1's persistent grid (and raises the kernel's shared-memory limit)
int p1_prepare(gbsp_plan_s* p, int sms) {
    int nb = 0;
    if (int rc = gbsp::p1_blocks_per_sm(p1_kernel(p), p->p1_smem, &nb)) return rc;
    if (nb < 1) return set_error(GBSP_ERR_UNSUPPORTED, "pass-1 kernel does not fit on an SM");
    p->p1_grid = nb * sms;
    return GBSP_OK;
}

gbsp::P1Args p1_args(const gbsp_plan_s* p, int u0, int n, float2* S, size_t s_pitch, const float2* chirp) {
    gbsp::P1Args a;
    a.row_idx = p->d_row_idx;
    a.win_slot0 = p->d_win_slot0;
    a.win_task = p->d_win_task;
    a.win_task_col = p->d_win_task_col;
    a.row_tab = p->d_rowtab;
    a.chirp = chirp;
    a.S = S;
    a.s_pitch = s_pitch;
    a.cw = p->p1_cw;
    a.cols = p->cols;
    a.s_cols = p->s_cols;
    a.ntab = p->ntab;
    a.rows = p->rows;
    a.u0 = u0;
    a.tile_rows = n;
    a.kahan_min = p->kahan_min;
    a.magic = p->rows_magic;
    a.magic64 = p->rows_magic64;
    a.queue = reinterpret_cast<unsigned int*>(p->d_err + 2);
    return a;
}

// The chirp pass 1 multiplies S by: the Bluestein pre-chirp (the channel-0
// post table, chirp[c] * W^0), or none for direct plans.
const float2* p1_chirp(const gbsp_plan_s* p) { return p->direct ? nullptr : p->d_post; }

// chirp == nullptr gives the raw column sums (gbsp_column_sums)
int launch_pass1(const gbsp_plan_s* p, int u0, int n, float2* S, size_t sp, const float2* chirp,
                 cudaStream_t st) {
    return gbsp::p1_launch(p1_kernel(p), p->p1_grid, p->p1_smem, st, p1_args(p, u0, n, S, sp, chirp));
}

gbsp::RowsKernel rows_kernel(const gbsp_plan_s* p) {
    return gbsp::RowsKernel{p->row_mode, p->rows_ntmax, p->K, p->rows_threads, p->rows_smem};
}

gbsp::RowsArgs rows_args(const gbsp_plan_s* p, const float2* S, size_t s_pitch, int u0, int n, void* d_out,
                         size_t out_pitch, int map_split = INT_MAX, int map_lo = 0, int map_hi = 0) {
    gbsp::RowsArgs a;
    a.S = S;
    a.s_pitch = s_pitch;
    a.pre = p->d_pre;
    a.post = p->d_post;
    a.filt = p->d_filt;
    a.fft_tw = p->d_fftw;
    a.out = (float2*)d_out;
    a.out_pitch = out_pitch;
    a.K = p->K;
    a.rows = p->rows;
    a.cols = p->cols;
    a.u0 = u0;
    a.tile_rows = n;
    a.map_split = map_split;
    a.map_lo = map_lo;
    a.map_hi = map_hi;
    a.zscratch = p->d_zscratch;
    a.drev = p->direct ? p->d_drev : nullptr;
    return a;
}

// the row kernel with fully specified arguments (input tile, output slab
// and row map)
int launch_rows_args(const gbsp_plan_s* p, const gbsp::RowsArgs& a, cudaStream_t st) {
    return gbsp::rows_launch(rows_kernel(p), p->rows_grid, st, a, p->fd, p->d_err);
}

int launch_rows(const gbsp_plan_s* p, int u0, int n, void* d_out, size_t out_pitch, cudaStream_t st) {
    return launch_rows_args(p, rows_args(p, p->d_S, p->s_pitch, u0, n, d_out, out_pitch), st);
}

// Block size and radices are already chosen; pick the compiled variant and
// size the persistent grid.
int rows_prepare(gbsp_plan_s* p, int sms) {
    int rmax = 0;
    for (int s = 0; s < p->fd.nst; s++) rmax = std::max(rmax, p->fd.R[s]);
    p->rows_ntmax = (rmax > max_radix_for(1024) || p->rows_threads <= 512) ? 512 : 1024;
    if (p->rows_threads > p->rows_ntmax || p->rows_threads < 32 || p->rows_threads % 32)
        return set_error(GBSP_ERR_INVALID, "rows_threads must be a multiple of 32, at most 512 when a "
                                           "radix exceeds 16, at most 1024 otherwise");
    using namespace gbsp;
    if (p->K == 1) p->row_mode = p->direct ? ROW_DIRECT : ROW_SINGLE;
    else if (p->row_mode != ROW_SEQ || p->rows_ntmax != 512) p->row_mode = ROW_CLUSTER;
    if (p->row_mode == ROW_CLUSTER && p->K > MAX_CHANNELS)
        return set_error(GBSP_ERR_UNSUPPORTED, "more than " + std::to_string(MAX_CHANNELS) +
                                                   " channels need sequential channels (512-thread rows)");
    if (p->row_mode == ROW_SEQ && p->K > MAX_CHANNELS) p->row_mode = ROW_SEQW;
    int cap = 0;
    const int rc = rows_capacity(rows_kernel(p), sms, &cap);
    if (rc) return rc;
    if (cap < 1) return set_error(GBSP_ERR_UNSUPPORTED, "row kernel does not fit on an SM");
    p->rows_grid = (p->row_mode == ROW_CLUSTER) ? cap * p->K : cap;
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
    // row indices are checked on the device while they are uploaded (plan_build)
    return GBSP_OK;
}

// Learned planner: the cost model scores every tuning candidate of the
// matrix and the cheapest prediction fills in o's radices, row block and
// pass-1 shape.  A matrix whose candidates leave the model's training range
// (gbsp_cost_model_set_domain) keeps the analytic choice, and o->planner
// says so.  The spectrum does not depend on the choice.
int learned_choice(const gbsp_plan_s* p, const int* col_ptr, size_t smem_cap, gbsp_options* o) {
    if (!gbsp::cost_model_loaded(gbsp::N_FEATURES))
        return set_error(GBSP_ERR_INVALID, "planner: no cost model installed (gbsp_cost_model_set)");
    std::vector<gbsp_options> cands;
    int nr = 0, np = 0;
    gbsp_options base = *o;
    base.planner = GBSP_PLANNER_MODEL;
    if (int rc = gbsp::enumerate_candidates(p->rows, p->cols, &base, smem_cap, 8, &cands, &nr, &np)) return rc;
    std::vector<float> feats(cands.size() * gbsp::N_FEATURES), pred(cands.size());
    for (size_t i = 0; i < cands.size(); i++)
        if (int rc = gbsp::plan_features(p->rows, p->cols, p->n_active, p->nnz, col_ptr, &cands[i], smem_cap,
                                         feats.data() + i * gbsp::N_FEATURES))
            return rc;
    if (!gbsp::cost_model_in_domain(feats.data(), (int)cands.size())) {
        o->planner = GBSP_PLANNER_MODEL;
        return GBSP_OK;
    }
    if (int rc = gbsp::cost_model_predict(feats.data(), (int)cands.size(), pred.data())) return rc;
    const size_t best = std::min_element(pred.begin(), pred.end()) - pred.begin();
    std::memcpy(o->radix, cands[best].radix, sizeof(o->radix));
    o->rows_threads = cands[best].rows_threads;
    o->pass1_shape = cands[best].pass1_shape;
    return GBSP_OK;
}

// force_p1: 1-based pass-1 shape imposed by a batch (one shape for all its
// matrices); 0 leaves the choice to the options.
int plan_build(gbsp_plan_s* p, const int* col_ptr, const int* row_idx, const int* sparse_cols,
               const gbsp_options* o_in, cudaStream_t st, int force_p1 = 0) {
    gbsp_options o = o_in ? *o_in : gbsp_options{};
    if (force_p1) o.pass1_shape = force_p1;
    GB_CUDA(cudaGetDevice(&p->device));
    DeviceLimits lim;
    if (int rc0 = device_limits(p->device, &lim)) return rc0;
    const size_t smem_cap = lim.smem_optin;
    const int sms = lim.sms;
    p->sms = sms;
    const int tmode = o.row_table_mode;
    if (tmode < 0 || tmode > 3) return set_error(GBSP_ERR_INVALID, "row_table_mode must be 0, 1, 2 or 3");
    if (o.pass1_shape < 0 || o.pass1_shape > gbsp::N_P1_SHAPES)
        return set_error(GBSP_ERR_INVALID, "pass1_shape must be 0 (auto) or 1.." + std::to_string(gbsp::N_P1_SHAPES));
    if (o.planner != GBSP_PLANNER_MODEL && o.planner != GBSP_PLANNER_LEARNED)
        return set_error(GBSP_ERR_INVALID, "planner must be GBSP_PLANNER_MODEL or GBSP_PLANNER_LEARNED");
    int rc = GBSP_OK;
    if (o.planner == GBSP_PLANNER_LEARNED && (rc = learned_choice(p, col_ptr, smem_cap, &o))) return rc;
    p->planner = o.planner;

    // ---- lengths, channel split, radices and row block
    gbsp::ChannelSplit sp;
    if ((rc = gbsp::split_channels(p->cols, &o, smem_cap, &sp))) return rc;
    p->L = sp.L;
    p->K = sp.K;
    p->Lp = sp.Lp;
    p->direct = sp.direct;
    p->fd = sp.ranked[0].fd;
    p->rows_threads = sp.ranked[0].nt;
    if (o.stream_tile_rows < GBSP_STREAM_TILE_AUTO)
        return set_error(GBSP_ERR_INVALID, "stream_tile_rows must be >= 0 or GBSP_STREAM_TILE_AUTO");
    if (o.channel_mode < 0 || o.channel_mode > 2)
        return set_error(GBSP_ERR_INVALID, "channel_mode must be 0 (auto), 1 (clusters) or 2 (sequential)");
    // multi-channel rows run sequentially in one CTA unless clusters are asked
    // for (measured on GB300: 1-4 % faster at 2 channels, 10-12 % at 4-5);
    // settled in rows_prepare
    p->row_mode = (o.channel_mode == 1) ? gbsp::ROW_CLUSTER : gbsp::ROW_SEQ;

    p->half_rows = p->rows / 2 + 1;
    p->out_cols = p->cols / 2 + 1;
    p->out_pitch = (p->out_cols + 3) / 4 * 4;
    p->u_tile = (o.u_tile > 0) ? std::min(o.u_tile, p->half_rows) : p->half_rows;
    if (o.exact_phases < 0 || o.exact_phases > 1) return set_error(GBSP_ERR_INVALID, "exact_phases must be 0 or 1");
    p->exact = o.exact_phases;
    p->kahan_min = (o.kahan_min_degree != 0) ? o.kahan_min_degree : 64;
    if (p->kahan_min < 0) p->kahan_min = 0;  // 0 disables compensation in the kernel
    int ib = o.index_bytes ? o.index_bytes : ((p->rows <= 65536 && p->cols <= 65536) ? 2 : 4);
    if (ib != 2 && ib != 4) return set_error(GBSP_ERR_INVALID, "index_bytes must be 2 or 4");
    if (ib == 2 && p->rows > 65536) return set_error(GBSP_ERR_INVALID, "rows > 65536 need 4-byte indices");
    p->idx_bytes = ib;
    p->big = p->rows > 65535;
    p->rows_magic = (p->rows >= 2) ? (uint32_t)(((1ull << 32) + (uint64_t)p->rows - 1) / (uint64_t)p->rows) : 0u;
    p->rows_magic64 = (p->rows >= 2) ? (unsigned long long)((((unsigned __int128)1 << 64) + p->rows - 1) / p->rows) : 0ull;

    // ---- pass-1 configuration: result tile + twiddle table in shared memory
    {
        const std::vector<int> fit = gbsp::fitting_p1_shapes(p->rows, smem_cap, tmode);
        int idx = fit.empty() ? -1 : fit[0];
        if (o.pass1_shape > 0) {
            idx = o.pass1_shape - 1;
            if (std::find(fit.begin(), fit.end(), idx) == fit.end())
                return set_error(GBSP_ERR_UNSUPPORTED, "pass1_shape " + std::to_string(o.pass1_shape) +
                                                           " does not fit this matrix or row_table_mode");
        }
        if (idx < 0) return set_error(GBSP_ERR_UNSUPPORTED, "rows too large for a shared-memory twiddle table");
        const gbsp::P1Shape& sh = gbsp::kP1Shapes[idx];
        p->p1_shape = idx + 1;
        p->p1_ku = sh.ku;
        p->p1_cw = sh.cw;
        p->tab_mode = sh.tab;
        p->ntab = (int)gbsp::row_table_entries(sh.tab, p->rows);
        p->p1_smem = gbsp::p1_smem_bytes(sh, p->rows);
    }
    if ((rc = p1_prepare(p, sms))) return rc;

    // ---- row-kernel configuration
    p->rows_smem = rows_smem_bytes(p->fd);
    if ((rc = rows_prepare(p, sms))) return rc;

    // ---- pass-1 task tables (slot0 | task | task_col, one region): built on
    // the device by k_csc_setup from the compact CSC
    p->s_cols = (p->cols + 1) & ~1;
    const int CW = p->p1_cw, VM = gbsp::p1_vmax(p->p1_cw);
    const int n_win = (p->s_cols + CW - 1) / CW;
    const size_t n_slot = (size_t)n_win * (CW + 1), n_task = (size_t)n_win * VM;
    const size_t off_task = (n_slot + 15) & ~(size_t)15;
    const size_t off_col = off_task + n_task * sizeof(int2);
    const size_t tbl_bytes = off_col + n_task;
    // one device allocation for every buffer of the plan
    {
        // automatic streaming tile: ~half_rows / 9, to the nearest multiple
        // of the SM count (at least one), at most u_tile
        const int t = (p->half_rows + 8) / 9;
        p->stream_tile_auto = std::min(p->u_tile, std::max(sms, (t + sms / 2) / sms * sms));
    }
    const int stream_tile = (o.stream_tile_rows > 0)                       ? std::min(o.stream_tile_rows, p->u_tile)
                            : (o.stream_tile_rows == GBSP_STREAM_TILE_AUTO) ? p->stream_tile_auto
                                                                            : 0;
    const size_t stream_slab = (size_t)2 * stream_tile * p->out_pitch * sizeof(float2);
    p->s_pitch = ((size_t)p->s_cols + 15) & ~(size_t)15;  // 128-byte rows; the bulk copy needs 16
    const size_t s_bytes = (size_t)p->u_tile * p->s_pitch * sizeof(float2);
    // the CSC arrives in a staging area -- the S tile, or a region of its own
    // when the tile is smaller: [int32 row indices (u16 plans narrow them) |
    // col_ptr | sparse_cols]
    const int na = p->n_active;
    auto a256 = [](size_t b) { return (std::max<size_t>(b, 16) + 255) & ~(size_t)255; };
    const size_t idx_in_bytes = (size_t)p->nnz * sizeof(int);
    const size_t st_row = (p->idx_bytes == 2) ? a256(idx_in_bytes) : 0;
    const size_t st_cp = a256((size_t)(na + 1) * sizeof(int)), st_sc = a256((size_t)na * sizeof(int));
    const size_t stage_bytes = st_row + st_cp + st_sc;
    const size_t staging = stage_bytes > s_bytes ? stage_bytes : 0;
    const int K = p->K, Lp = p->Lp, cols = p->cols;
    const int ntw = std::max(fft_tw_count(p->fd), 1);
    {
        const size_t sizes[] = {tbl_bytes, (size_t)std::max(p->nnz, 1) * p->idx_bytes, 4 * sizeof(int),
                                (size_t)p->ntab * sizeof(float2), (size_t)K * cols * sizeof(float2),
                                (size_t)K * cols * sizeof(float2), (size_t)K * Lp * sizeof(float2),
                                (size_t)ntw * sizeof(float2), (size_t)K * Lp * sizeof(double2),
                                (size_t)K * Lp * sizeof(double2), s_bytes, staging,
                                (p->row_mode == gbsp::ROW_SEQ || p->row_mode == gbsp::ROW_SEQW)
                                    ? (size_t)p->rows_grid * (K - 1) * Lp * sizeof(float2)
                                    : 0,
                                stream_slab, stream_slab, p->direct ? (size_t)Lp * sizeof(int) : 0};
        size_t total = 0;
        for (size_t b : sizes) total += a256(b);
        void* base = nullptr;
        cudaMemPool_t pool = nullptr;
        if ((rc = plan_pool(p->device, &pool))) return rc;
        cudaError_t e = pool ? cudaMallocFromPoolAsync(&base, total, pool, st) : cudaMalloc(&base, total);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_error(GBSP_ERR_ALLOC, std::string("plan memory (") + std::to_string(total) +
                                                 " bytes): " + cudaGetErrorString(e));
        }
        if (pool) {
            p->arena_pooled = true;
            pool_account(p->device, (long long)total);
        } else
            p->allocs.push_back(base);
        p->device_bytes += total;
        p->arena = static_cast<char*>(base);
        p->arena_size = total;
        p->arena_off = 0;
    }
    uint8_t* d_tbl = nullptr;
    if ((rc = dev_alloc(p, (void**)&d_tbl, tbl_bytes))) return rc;
    p->d_win_slot0 = d_tbl;
    p->d_win_task = reinterpret_cast<int2*>(d_tbl + off_task);
    p->d_win_task_col = d_tbl + off_col;
    if (stream_slab > 0) {
        for (int b = 0; b < 2; b++)
            if ((rc = dev_alloc(p, &p->stream_slab[b], stream_slab))) return rc;
        p->stream_slab_bytes = stream_slab;
        // the copy stream and its events too, so a streamed transform does
        // no setup of its own
        if ((rc = stream_objects(p))) return rc;
    }
    if ((p->row_mode == gbsp::ROW_SEQ || p->row_mode == gbsp::ROW_SEQW) &&
        (rc = dev_alloc(p, (void**)&p->d_zscratch, (size_t)p->rows_grid * (K - 1) * Lp * sizeof(float2))))
        return rc;
    if ((rc = dev_alloc(p, &p->d_row_idx, (size_t)std::max(p->nnz, 1) * p->idx_bytes))) return rc;
    // [1]: plan-build checks (bit 0 a row index out of range, bit 1 a task
    // overflow); [2], [3]: pass 1's item queue
    if ((rc = dev_alloc(p, (void**)&p->d_err, 4 * sizeof(int)))) return rc;
    if ((rc = dev_alloc(p, (void**)&p->d_S, s_bytes))) return rc;
    char* d_stage = reinterpret_cast<char*>(p->d_S);
    if (staging > 0 && (rc = dev_alloc(p, (void**)&d_stage, staging))) return rc;
    if ((rc = dev_alloc(p, (void**)&p->d_rowtab, (size_t)p->ntab * sizeof(float2)))) return rc;
    if ((rc = dev_alloc(p, (void**)&p->d_pre, (size_t)K * cols * sizeof(float2)))) return rc;
    if ((rc = dev_alloc(p, (void**)&p->d_post, (size_t)K * cols * sizeof(float2)))) return rc;
    if ((rc = dev_alloc(p, (void**)&p->d_filt, (size_t)K * Lp * sizeof(float2)))) return rc;
    if ((rc = dev_alloc(p, (void**)&p->d_fftw, (size_t)ntw * sizeof(float2)))) return rc;
    if (p->direct && (rc = dev_alloc(p, (void**)&p->d_drev, (size_t)Lp * sizeof(int)))) return rc;
    // FP64 filter workspace (ping-pong: the stages run out of place), kept
    // with the plan: freeing it here would synchronise the whole device
    double2* d_spec[2] = {nullptr, nullptr};
    if ((rc = dev_alloc(p, (void**)&d_spec[0], (size_t)K * Lp * sizeof(double2)))) return rc;
    if ((rc = dev_alloc(p, (void**)&d_spec[1], (size_t)K * Lp * sizeof(double2)))) return rc;

    // ---- device work.  The tables (FP64, rounded to FP32) and the filter
    // spectrum (input, DIF stages, final rounding: a chain of dependent
    // launches) need nothing from the host, so they run on the library's
    // helper stream beside the CSC uploads and their setup kernel on `st`;
    // the two join before the synchronisation.
    cudaStream_t hs = nullptr;
    if ((rc = helper_stream(p->device, &hs))) return rc;
    struct Events {  // fork / join, released on every return path
        cudaEvent_t e[2] = {nullptr, nullptr};
        ~Events() {
            for (cudaEvent_t x : e)
                if (x) cudaEventDestroy(x);
        }
    } evs;
    cudaEvent_t* ev = evs.e;
    cudaStream_t fs = st;
    if (hs) {
        GB_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
        GB_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
        GB_CUDA(cudaEventRecord(ev[0], st));  // after the arena's stream-ordered allocation
        GB_CUDA(cudaStreamWaitEvent(hs, ev[0], 0));
        fs = hs;
    }
    {
        gbsp::TableArgs ta;
        ta.rowtab = p->d_rowtab;
        ta.pre = p->d_pre;
        ta.post = p->d_post;
        ta.fftw = p->d_fftw;
        ta.ntab = p->ntab;
        ta.rows = p->rows;
        ta.two_level = p->tab_mode == gbsp::TAB_TWO;
        ta.cols = cols;
        ta.L = p->L;
        ta.K = K;
        ta.fd = p->fd;
        const long n_tab = (long)p->ntab + 2L * K * cols + fft_tw_count(p->fd);
        gbsp::k_tables<<<blocks_for(n_tab, 256), 256, 0, fs>>>(ta);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && p->direct) {  // no filter: the digit-reversal table instead
        gbsp::k_digit_rev<<<blocks_for(Lp, 256), 256, 0, fs>>>(p->d_drev, p->fd);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && !p->direct) {
        gbsp::k_table_filter_input<<<blocks_for((long)K * Lp, 256), 256, 0, fs>>>(d_spec[0], cols, p->L, K, Lp);
        e = cudaGetLastError();
    }
    int cur = 0;
    for (int s = 0; s < p->fd.nst && e == cudaSuccess && !p->direct; s++, cur ^= 1) {
        gbsp::k_dif_stage_f64<<<blocks_for((long)K * Lp, 128), 128, 0, fs>>>(d_spec[cur], d_spec[cur ^ 1], K, Lp,
                                                                             p->fd.R[s], p->fd.m[s]);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && !p->direct) {
        gbsp::k_table_filter_final<<<blocks_for((long)K * Lp, 256), 256, 0, fs>>>(
            p->d_filt, d_spec[cur], K, Lp, p->fd.R[p->fd.nst - 1], 1.0 / (double)p->L);
        e = cudaGetLastError();
    }
    if (hs && e == cudaSuccess) e = cudaEventRecord(ev[1], hs);
    // the CSC: uploads, then one setup kernel (task tables, row-index check)
    int* d_cp = reinterpret_cast<int*>(d_stage + st_row);
    int* d_sc = reinterpret_cast<int*>(d_stage + st_row + st_cp);
    int* d_in = (p->idx_bytes == 2) ? reinterpret_cast<int*>(d_stage) : static_cast<int*>(p->d_row_idx);
    if (e == cudaSuccess) e = cudaMemsetAsync(p->d_err, 0, 4 * sizeof(int), st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_cp, col_ptr, (size_t)(na + 1) * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && na > 0)
        e = cudaMemcpyAsync(d_sc, sparse_cols, (size_t)na * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && p->nnz > 0) e = cudaMemcpyAsync(d_in, row_idx, idx_in_bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        gbsp::CscSetupArgs ca;
        ca.col_ptr = d_cp;
        ca.sparse_cols = d_sc;
        ca.n_active = na;
        ca.cols = cols;
        ca.cw = CW;
        ca.n_win = n_win;
        ca.task_blocks = (int)blocks_for(n_win, gbsp::SETUP_WARPS);
        ca.slot0 = p->d_win_slot0;
        ca.task = p->d_win_task;
        ca.task_col = p->d_win_task_col;
        ca.row_in = d_in;
        ca.row16 = (p->idx_bytes == 2) ? static_cast<uint16_t*>(p->d_row_idx) : nullptr;
        ca.nnz = p->nnz;
        ca.rows = p->rows;
        ca.bad = p->d_err + 1;
        const int row_blocks = (int)std::min<long>(blocks_for(p->nnz, gbsp::SETUP_WARPS * 32), (long)sms * 16);
        gbsp::k_csc_setup<<<ca.task_blocks + std::max(row_blocks, 1), gbsp::SETUP_WARPS * 32, 0, st>>>(ca);
        e = cudaGetLastError();
    }
    if (hs && e == cudaSuccess) e = cudaStreamWaitEvent(st, ev[1], 0);
    int bad = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, p->d_err + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (hs && e != cudaSuccess) cudaStreamSynchronize(hs);  // nothing of this plan may still run
    if (e != cudaSuccess)
        return set_error(GBSP_ERR_CUDA, std::string("plan build: ") + cudaGetErrorString(e));
    if (bad & 1) return set_error(GBSP_ERR_INVALID, "gbsp_plan_create: row index out of range");
    if (bad & 2) return set_error(GBSP_ERR_UNSUPPORTED, "pass-1 window task overflow");
    return GBSP_OK;
}

// Reads and clears the plan's device error word (synchronous) and turns it
// into a status (gbsp_device_flags_status)
int read_device_flags(const gbsp_plan_s* p) {
    int flags = 0;
    GB_CUDA(cudaMemcpy(&flags, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (flags) GB_CUDA(cudaMemset(p->d_err, 0, sizeof(int)));
    return gbsp_device_flags_status(flags);
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

int gbsp_set_memory_cache(size_t bytes) {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    g_cache_limit = bytes;
    for (int d = 0; d < MAX_POOL_DEVICES; d++) {
        if (!g_pool[d]) continue;
        unsigned long long thr = g_pool_live[d] + bytes;
        GB_CUDA(cudaMemPoolSetAttribute(g_pool[d], cudaMemPoolAttrReleaseThreshold, &thr));
        GB_CUDA(cudaMemPoolTrimTo(g_pool[d], thr));
    }
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
    info->row_table_mode = p->tab_mode;
    info->rows_threads = p->rows_threads;
    info->device_bytes = p->device_bytes;
    info->pass1_shape = p->p1_shape;
    info->planner = p->planner;
    info->channel_mode = p->K == 1 ? 0 : (p->row_mode == gbsp::ROW_CLUSTER ? 1 : 2);
    info->exact_phases = p->exact;
    info->direct = p->direct;
    return GBSP_OK;
}

int gbsp_plan_error_flags(gbsp_plan_t p, int* flags) {
    if (!p || !flags) return set_error(GBSP_ERR_INVALID, "gbsp_plan_error_flags: null argument");
    int f = 0;
    GB_CUDA(cudaMemcpy(&f, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    GB_CUDA(cudaMemset(p->d_err, 0, sizeof(int)));
    *flags = f;
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
        if ((rc = launch_pass1(p, u0, n, p->d_S, p->s_pitch, p1_chirp(p), st))) return rc;
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
        rc = launch_pass1(p, u0, n, p->d_S, p->s_pitch, p1_chirp(p), st);
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
    if ((rc = read_device_flags(p))) return rc;
    *ms_pass1 = a;
    *ms_rows = b;
    return GBSP_OK;
}

int gbsp_column_sums(gbsp_plan_t p, int u0, int n_rows, void* d_s, size_t s_pitch, void* stream) {
    if (!p || !d_s) return set_error(GBSP_ERR_INVALID, "gbsp_column_sums: null argument");
    if (u0 < 0 || n_rows < 1 || u0 + n_rows > p->rows || s_pitch < (size_t)p->s_cols)
        return set_error(GBSP_ERR_INVALID, "gbsp_column_sums: bad range or pitch (>= cols rounded up to even)");
    return launch_pass1(p, u0, n_rows, (float2*)d_s, s_pitch, nullptr, (cudaStream_t)stream);
}

}  // extern "C"

// ===========================================================================
// Allocation-free execution.
//
// Some callers must not allocate device memory when they run a transform:
// code whose device memory is owned by a pool with a hard budget (a
// framework's caching allocator that forbids side allocations), latency-
// critical loops where cudaMalloc's implicit synchronisation is not
// acceptable, or code paths that only enqueue work.  For them
// gbsp_execute_noalloc runs the same two kernels as gbsp_execute, but the
// pass-1 intermediate (the S tile the row kernel reads) lives in a fixed
// array compiled into this library instead of a per-plan allocation; it
// calls no allocating routine.  The array is 32 MiB and every GPU that loads
// the library holds it until the process exits.
// ===========================================================================
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = (size_t)32 << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// Device address of g_noalloc_scratch on each device, looked up once per
// device (with that device current) on that device's first call.
constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[NOALLOC_MAX_DEVICES] = {};

int noalloc_scratch_address(int device, void** addr) {
    if (device < 0 || device >= NOALLOC_MAX_DEVICES)
        return set_error(GBSP_ERR_UNSUPPORTED, "gbsp_execute_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return set_error(GBSP_ERR_CUDA, std::string("gbsp_execute_noalloc: cudaGetSymbolAddress: ") +
                                                cudaGetErrorString(e));
        g_noalloc_addr[device] = ptr;
    }
    *addr = g_noalloc_addr[device];
    return GBSP_OK;
}

// the row kernel reading its input rows from an explicit S tile
int launch_rows_from(const gbsp_plan_s* p, const float2* S, size_t s_pitch, int u0, int n, void* d_out,
                     size_t out_pitch, cudaStream_t st) {
    return launch_rows_args(p, rows_args(p, S, s_pitch, u0, n, d_out, out_pitch), st);
}

}  // namespace

extern "C" int gbsp_execute_noalloc(gbsp_plan_t p, void* d_out, size_t out_pitch, void* stream) {
    int rc = check_out(p, d_out, out_pitch, "gbsp_execute_noalloc");
    if (rc) return rc;
    int dev = -1;
    GB_CUDA(cudaGetDevice(&dev));
    if (dev != p->device)
        return set_error(GBSP_ERR_INVALID, "gbsp_execute_noalloc: the plan's device must be current");
    const size_t row_bytes = p->s_pitch * sizeof(float2);
    if (row_bytes > NOALLOC_SCRATCH_BYTES)
        return set_error(GBSP_ERR_UNSUPPORTED,
                         "gbsp_execute_noalloc: one pass-1 row needs " + std::to_string(row_bytes) +
                             " bytes, more than the fixed scratch array (" +
                             std::to_string(NOALLOC_SCRATCH_BYTES) + " bytes)");
    void* scratch = nullptr;
    if ((rc = noalloc_scratch_address(dev, &scratch))) return rc;
    // Tiles sized to the array.  Nothing in it has to start at zero: pass 1
    // writes every element of a tile row that the row kernel reads.  Pass 1
    // computes whole blocks of 32*KU rows, so a tile whose last block would
    // be less than half used is cut back to a whole number of blocks.
    int tile = (int)std::min<size_t>((size_t)p->u_tile, NOALLOC_SCRATCH_BYTES / row_bytes);
    const int ublk = 32 * p->p1_ku;
    if (tile < p->u_tile && tile >= ublk && tile % ublk < ublk / 2) tile -= tile % ublk;
    cudaStream_t st = (cudaStream_t)stream;
    for (int u0 = 0; u0 < p->half_rows; u0 += tile) {
        const int n = std::min(tile, p->half_rows - u0);
        if ((rc = launch_pass1(p, u0, n, (float2*)scratch, p->s_pitch, p1_chirp(p), st))) return rc;
        if ((rc = launch_rows_from(p, (const float2*)scratch, p->s_pitch, u0, n, d_out, out_pitch, st)))
            return rc;
    }
    return GBSP_OK;
}

// ===========================================================================
// Batches: many matrices of uneven size and sparsity in one persistent
// launch per pass, fed by device work queues.
//
// Each matrix gets its own tables and scratch (a plan built with a pass-1
// shape and a block size common to the batch); one descriptor per matrix
// lists them.  gbsp_batch_execute resets the two queue heads and launches
// k_twiddle_sum_batch and k_bluestein_rows_batch once each; matrices whose
// convolution needs several channels run after them through their own plan.
// The three operations capture into a CUDA graph (gbsp_batch_graph_*).
// ===========================================================================
struct gbsp_batch_s {
    int count = 0;
    int device = 0;
    std::vector<gbsp_plan_s*> plans;
    std::vector<int> order;      // queue order (batched matrices, costliest rows first)
    std::vector<int> separate;   // matrices that run through their own plan
    int p1_shape = 1, ku = 8, cw = 32, tab = 0, idx_bytes = 2, big = 0, exact = 0;
    int p1_grid = 0;
    size_t p1_smem = 0;
    // Row launches: one per class of matrices that share a block size and a
    // CTAs-per-SM count, so small rows keep the occupancy they have alone.
    struct RowsClass {
        int nt = 0, grid = 0, begin = 0, end = 0;  // descriptors [begin, end) in queue order
        size_t smem = 0;
    };
    std::vector<RowsClass> classes;
    gbsp::P1Args* d_p1 = nullptr;
    long* d_p1_begin = nullptr;
    gbsp::RowsBatch* d_rows = nullptr;
    long* d_row_begin = nullptr;            // per class: count+1 prefix entries from 0
    unsigned long long* d_queue = nullptr;  // [0] pass 1, [1 + c] rows of class c
    int* d_err = nullptr;
    std::vector<void*> outs;
    std::vector<size_t> pitches;
    bool outputs_set = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<void*> allocs;
};

namespace {

void free_batch(gbsp_batch_s* b) {
    if (!b) return;
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (auto* p : b->plans) free_plan(p);
    for (void* a : b->allocs) cudaFree(a);
    delete b;
}

int batch_alloc(gbsp_batch_s* b, void** ptr, size_t bytes) {
    cudaError_t e = cudaMalloc(ptr, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(GBSP_ERR_ALLOC, std::string("batch cudaMalloc: ") + cudaGetErrorString(e));
    }
    b->allocs.push_back(*ptr);
    return GBSP_OK;
}

// prepare: size the batched pass-1 grid; else launch it
int p1b_dispatch(gbsp_batch_s* b, bool prepare, int sms, cudaStream_t st) {
    const gbsp::P1Kernel k{b->idx_bytes, b->tab, b->big != 0, b->ku, b->exact != 0};
    if (prepare) {
        int nb = 0;
        if (int rc = gbsp::p1_batch_blocks_per_sm(k, b->p1_smem, &nb)) return rc;
        if (nb < 1) return set_error(GBSP_ERR_UNSUPPORTED, "batched pass 1 does not fit on an SM");
        b->p1_grid = nb * sms;
        return GBSP_OK;
    }
    return gbsp::p1_batch_launch(k, b->p1_grid, b->p1_smem, st, b->d_p1, b->d_p1_begin, (int)b->order.size(),
                                 b->d_queue);
}

int batch_launch(gbsp_batch_s* b, cudaStream_t st) {
    if (!b->order.empty()) {
        GB_CUDA(cudaMemsetAsync(b->d_queue, 0, (1 + b->classes.size()) * sizeof(unsigned long long), st));
        int rc = p1b_dispatch(b, false, 0, st);
        if (rc) return rc;
        for (size_t c = 0; c < b->classes.size(); c++) {
            const auto& k = b->classes[c];
            if ((rc = gbsp::rows_batch_launch(k.grid, k.nt, k.smem, st, b->d_rows + k.begin,
                                              b->d_row_begin + k.begin + c, k.end - k.begin, b->d_queue + 1 + c,
                                              b->d_err)))
                return rc;
        }
    }
    for (int m : b->separate) {
        int rc = gbsp_execute(b->plans[m], b->outs[m], b->pitches[m], st);
        if (rc) return rc;
    }
    return GBSP_OK;
}

}  // namespace

extern "C" {

int gbsp_batch_create(int count, const gbsp_matrix* mats, const gbsp_options* opts, void* stream,
                      gbsp_batch_t* out) {
    if (!out || count < 1 || !mats) return set_error(GBSP_ERR_INVALID, "gbsp_batch_create: bad arguments");
    *out = nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    gbsp_batch_s* b = new (std::nothrow) gbsp_batch_s();
    if (!b) return set_error(GBSP_ERR_ALLOC, "gbsp_batch_create: out of host memory");
    b->count = count;
    int rc = GBSP_OK;
    DeviceLimits lim;
    if (cudaGetDevice(&b->device) != cudaSuccess || device_limits(b->device, &lim) != GBSP_OK) {
        free_batch(b);
        return set_error(GBSP_ERR_CUDA, "gbsp_batch_create: no CUDA device");
    }
    const size_t smem_cap = lim.smem_optin;
    const int sms = lim.sms;
    // one pass-1 shape for the batch: the largest row count decides it
    int max_rows = 1;
    bool u32 = false;
    for (int i = 0; i < count; i++) {
        int vr = validate_csc(mats[i].rows, mats[i].cols, mats[i].n_active, mats[i].nnz, mats[i].col_ptr,
                              mats[i].row_idx, mats[i].sparse_cols);
        if (vr) {
            free_batch(b);
            return vr;
        }
        max_rows = std::max(max_rows, mats[i].rows);
        u32 = u32 || mats[i].rows > 65536 || mats[i].cols > 65536 || (opts && opts->index_bytes == 4);
    }
    b->idx_bytes = u32 ? 4 : 2;
    b->big = max_rows > 65535;
    b->exact = (opts && opts->exact_phases == 1) ? 1 : 0;
    {
        const int tmode = opts ? opts->row_table_mode : 0;
        std::vector<int> fit = gbsp::fitting_p1_shapes(max_rows, smem_cap, tmode);
        if (opts && opts->pass1_shape > 0) {
            const int want = opts->pass1_shape - 1;
            fit.erase(std::remove_if(fit.begin(), fit.end(), [&](int i) { return i != want; }), fit.end());
        }
        if (fit.empty()) {
            free_batch(b);
            return set_error(GBSP_ERR_UNSUPPORTED, "gbsp_batch_create: no pass-1 shape fits the largest matrix");
        }
        b->p1_shape = fit[0] + 1;
        b->ku = gbsp::kP1Shapes[fit[0]].ku;
        b->cw = gbsp::kP1Shapes[fit[0]].cw;
        b->tab = gbsp::kP1Shapes[fit[0]].tab;
        b->p1_smem = gbsp::p1_smem_bytes(gbsp::kP1Shapes[fit[0]], max_rows);
    }
    // one plan per matrix with the common pass-1 shape; row blocks of 256 or
    // 512 threads (the planner's automatic choice)
    gbsp_options o = opts ? *opts : gbsp_options{};
    o.u_tile = 0;
    o.index_bytes = b->idx_bytes;
    o.rows_threads = 0;
    o.row_table_mode = 0;
    for (int& r : o.radix) r = 0;  // lengths differ across the batch: per-matrix radices
    b->plans.assign(count, nullptr);
    for (int i = 0; i < count && rc == GBSP_OK; i++) {
        gbsp_plan_s* p = new (std::nothrow) gbsp_plan_s();
        if (!p) { rc = set_error(GBSP_ERR_ALLOC, "gbsp_batch_create: out of host memory"); break; }
        p->rows = mats[i].rows;
        p->cols = mats[i].cols;
        p->nnz = mats[i].nnz;
        p->n_active = mats[i].n_active;
        b->plans[i] = p;
        rc = plan_build(p, mats[i].col_ptr, mats[i].row_idx, mats[i].sparse_cols, &o, st, b->p1_shape);
    }
    if (rc) {
        free_batch(b);
        return rc;
    }
    // Single-channel matrices go through the queues, grouped into classes of
    // (block size, CTAs per SM), classes with the longest rows first, and by
    // decreasing channel length inside a class.
    std::vector<int> per_sm(count, 0);
    for (int i = 0; i < count; i++) {
        const gbsp_plan_s* p = b->plans[i];
        if (p->K != 1 || p->rows_threads > 512) {
            b->separate.push_back(i);
            continue;
        }
        if (gbsp::rows_batch_blocks_per_sm(p->rows_threads, rows_smem_bytes(p->fd), &per_sm[i]) != GBSP_OK ||
            per_sm[i] < 1) {
            free_batch(b);
            return set_error(GBSP_ERR_UNSUPPORTED, "gbsp_batch_create: batched row kernel does not fit");
        }
        b->order.push_back(i);
    }
    std::stable_sort(b->order.begin(), b->order.end(), [&](int x, int y) {
        const gbsp_plan_s *px = b->plans[x], *py = b->plans[y];
        if (per_sm[x] != per_sm[y]) return per_sm[x] < per_sm[y];
        if (px->rows_threads != py->rows_threads) return px->rows_threads > py->rows_threads;
        return px->Lp > py->Lp;
    });
    const int n = (int)b->order.size();
    for (int k = 0; k < n; k++) {
        const gbsp_plan_s* p = b->plans[b->order[k]];
        const int m = b->order[k];
        if (b->classes.empty() || per_sm[b->order[k - 1]] != per_sm[m] ||
            b->plans[b->order[k - 1]]->rows_threads != p->rows_threads) {
            gbsp_batch_s::RowsClass c;
            c.nt = p->rows_threads;
            c.grid = per_sm[m] * sms;
            c.begin = k;
            b->classes.push_back(c);
        }
        b->classes.back().end = k + 1;
        b->classes.back().smem = std::max(b->classes.back().smem, rows_smem_bytes(p->fd));
    }
    const int ncls = (int)b->classes.size();
    if (n > 0) {
        if ((rc = p1b_dispatch(b, true, sms, st)) ||
            (rc = batch_alloc(b, (void**)&b->d_p1, sizeof(gbsp::P1Args) * n)) ||
            (rc = batch_alloc(b, (void**)&b->d_p1_begin, sizeof(long) * (n + 1))) ||
            (rc = batch_alloc(b, (void**)&b->d_rows, sizeof(gbsp::RowsBatch) * n)) ||
            (rc = batch_alloc(b, (void**)&b->d_row_begin, sizeof(long) * (n + ncls)))) {
            free_batch(b);
            return rc;
        }
        // work-queue prefix sums (pass 1 over the whole queue, rows per class)
        std::vector<gbsp::P1Args> p1(n);
        std::vector<long> p1b(n + 1, 0), rb;
        const int ublk = 32 * b->ku;
        for (int k = 0; k < n; k++) {
            const gbsp_plan_s* p = b->plans[b->order[k]];
            p1[k] = p1_args(p, 0, p->half_rows, p->d_S, p->s_pitch, p1_chirp(p));
            p1b[k + 1] = p1b[k] + (long)((p->half_rows + ublk - 1) / ublk) * ((p->s_cols + p->p1_cw - 1) / p->p1_cw);
        }
        for (const auto& c : b->classes) {
            rb.push_back(0);
            for (int k = c.begin; k < c.end; k++) rb.push_back(rb.back() + b->plans[b->order[k]]->half_rows);
        }
        if (cudaMemcpy(b->d_p1, p1.data(), sizeof(gbsp::P1Args) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(b->d_p1_begin, p1b.data(), sizeof(long) * (n + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(b->d_row_begin, rb.data(), sizeof(long) * rb.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
            free_batch(b);
            return set_error(GBSP_ERR_CUDA, "gbsp_batch_create: descriptor upload failed");
        }
    }
    if ((rc = batch_alloc(b, (void**)&b->d_queue, (1 + ncls) * sizeof(unsigned long long))) ||
        (rc = batch_alloc(b, (void**)&b->d_err, sizeof(int)))) {
        free_batch(b);
        return rc;
    }
    cudaMemset(b->d_err, 0, sizeof(int));
    b->outs.assign(count, nullptr);
    b->pitches.assign(count, 0);
    *out = b;
    return GBSP_OK;
}

int gbsp_batch_set_outputs(gbsp_batch_t b, void* const* d_outs, const size_t* out_pitches) {
    if (!b || !d_outs || !out_pitches) return set_error(GBSP_ERR_INVALID, "gbsp_batch_set_outputs: null argument");
    for (int i = 0; i < b->count; i++) {
        int rc = check_out(b->plans[i], d_outs[i], out_pitches[i], "gbsp_batch_set_outputs");
        if (rc) return rc;
    }
    const int n = (int)b->order.size();
    std::vector<gbsp::RowsBatch> rows(n);
    for (int k = 0; k < n; k++) {
        const int m = b->order[k];
        const gbsp_plan_s* p = b->plans[m];
        rows[k].a = rows_args(p, p->d_S, p->s_pitch, 0, p->half_rows, d_outs[m], out_pitches[m]);
        rows[k].fd = p->fd;
    }
    if (n > 0) GB_CUDA(cudaMemcpy(b->d_rows, rows.data(), sizeof(gbsp::RowsBatch) * n, cudaMemcpyHostToDevice));
    for (int i = 0; i < b->count; i++) {
        b->outs[i] = d_outs[i];
        b->pitches[i] = out_pitches[i];
    }
    b->outputs_set = true;
    if (b->graph_exec) {
        cudaGraphExecDestroy(b->graph_exec);
        b->graph_exec = nullptr;
    }
    return GBSP_OK;
}

int gbsp_batch_execute(gbsp_batch_t b, void* stream) {
    if (!b) return set_error(GBSP_ERR_INVALID, "gbsp_batch_execute: null batch");
    if (!b->outputs_set) return set_error(GBSP_ERR_INVALID, "gbsp_batch_execute: outputs not set");
    return batch_launch(b, (cudaStream_t)stream);
}

int gbsp_batch_graph_launch(gbsp_batch_t b, void* stream) {
    if (!b) return set_error(GBSP_ERR_INVALID, "gbsp_batch_graph_launch: null batch");
    if (!b->outputs_set) return set_error(GBSP_ERR_INVALID, "gbsp_batch_graph_launch: outputs not set");
    cudaStream_t st = (cudaStream_t)stream;
    if (!b->graph_exec) {
        // capture on a private stream so the caller's stream state is untouched
        cudaStream_t cs = nullptr;
        GB_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        int rc = (e == cudaSuccess) ? batch_launch(b, cs) : GBSP_ERR_CUDA;
        cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        cudaStreamDestroy(cs);
        if (rc) return rc;
        if (e != cudaSuccess || e2 != cudaSuccess)
            return set_error(GBSP_ERR_CUDA, "gbsp_batch_graph_launch: capture failed");
        e = cudaGraphInstantiate(&b->graph_exec, g, 0);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->graph = g;
        if (e != cudaSuccess) {
            b->graph_exec = nullptr;
            return set_error(GBSP_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
        }
    }
    GB_CUDA(cudaGraphLaunch(b->graph_exec, st));
    return GBSP_OK;
}

int gbsp_batch_error_flags(gbsp_batch_t b, int* flags) {
    if (!b || !flags) return set_error(GBSP_ERR_INVALID, "gbsp_batch_error_flags: null argument");
    int f = 0;
    GB_CUDA(cudaMemcpy(&f, b->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    GB_CUDA(cudaMemset(b->d_err, 0, sizeof(int)));
    for (auto* p : b->plans) {
        int g = 0;
        GB_CUDA(cudaMemcpy(&g, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
        GB_CUDA(cudaMemset(p->d_err, 0, sizeof(int)));
        f |= g;
    }
    *flags = f;
    return GBSP_OK;
}

int gbsp_batch_plan_info(gbsp_batch_t b, int i, gbsp_plan_info* info) {
    if (!b || i < 0 || i >= b->count) return set_error(GBSP_ERR_INVALID, "gbsp_batch_plan_info: bad index");
    return gbsp_plan_get_info(b->plans[i], info);
}

int gbsp_batch_destroy(gbsp_batch_t b) {
    free_batch(b);
    return GBSP_OK;
}

}  // extern "C"

// ===========================================================================
// Streaming to host memory: tiles of Bluestein rows are computed into one of
// two small device slabs (output rows u and rows-u of the tile, remapped by
// the row writer) while the previous slab is copied to the host on a second
// stream.  Device memory beyond the plan: two slabs of 2 x tile x pitch.
// ===========================================================================
namespace {

}  // namespace

extern "C" int gbsp_execute_to_host(gbsp_plan_t p, void* h_out, size_t out_pitch, int tile_rows, void* stream) {
    if (!p || !h_out) return set_error(GBSP_ERR_INVALID, "gbsp_execute_to_host: null argument");
    if (out_pitch < (size_t)p->out_cols || (out_pitch & 1))
        return set_error(GBSP_ERR_INVALID, "gbsp_execute_to_host: out_pitch must be even and >= cols/2+1");
    if (tile_rows < 0) return set_error(GBSP_ERR_INVALID, "gbsp_execute_to_host: tile_rows must be >= 0");
    const int tile = std::min(tile_rows > 0 ? tile_rows : p->stream_tile_auto, p->u_tile);
    cudaStream_t st = (cudaStream_t)stream;
    const size_t slab_bytes = (size_t)2 * tile * out_pitch * sizeof(float2);
    if (int rc0 = stream_objects(p)) return rc0;
    if (p->stream_slab_bytes < slab_bytes) {
        for (int b = 0; b < 2; b++) {
            if (p->stream_slab[b] && p->stream_slab_owned) {
                cudaFree(p->stream_slab[b]);
                p->device_bytes -= p->stream_slab_bytes;
            }
            p->stream_slab[b] = nullptr;
        }
        p->stream_slab_bytes = 0;
        p->stream_slab_owned = true;
        for (int b = 0; b < 2; b++) {
            cudaError_t e = cudaMalloc(&p->stream_slab[b], slab_bytes);
            if (e != cudaSuccess) {
                cudaGetLastError();
                p->stream_slab[b] = nullptr;
                return set_error(GBSP_ERR_ALLOC, std::string("gbsp_execute_to_host: slab: ") + cudaGetErrorString(e));
            }
            p->device_bytes += slab_bytes;
        }
        p->stream_slab_bytes = slab_bytes;
    }
    struct {
        cudaStream_t cs;
        cudaEvent_t* done;
        cudaEvent_t* copied;
        void** slab;
    } r{p->stream_cs, p->stream_done, p->stream_copied, p->stream_slab};
    const size_t row_bytes = out_pitch * sizeof(float2);
    char* host = static_cast<char*>(h_out);
    int rc = GBSP_OK;
    int t = 0;
    // The first tiles ramp up from 256 rows, doubling: the first tile's
    // compute is the only one the copies cannot hide, and a tile computes
    // about as fast as the one before it copies out.  Ramp tiles are
    // multiples of 256 rows (the largest pass-1 row block), so a tile size
    // that is one too starts every tile where the single launch starts a
    // row block, with the same bits.
    int n_ramp = std::min(tile, 256);
    for (int u0 = 0, n = 0; u0 < p->half_rows && rc == GBSP_OK; u0 += n, t++) {
        n = std::min(n_ramp, p->half_rows - u0);
        n_ramp = std::min(tile, 2 * n_ramp);
        const int b = t & 1;
        // rows u in [u0, u0+n) -> slab rows [0, n); their mirrors rows - u
        // (u >= 1, rows - u != u) form [hi_first, rows - u0] -> slab rows n..
        const int u_last = u0 + n - 1;
        int hi_first = p->rows - u_last;
        if (2 * u_last == p->rows) hi_first++;  // the middle row is its own mirror
        const int hi_last = p->rows - std::max(u0, 1);
        const int n_hi = std::max(0, hi_last - hi_first + 1);
        if ((rc = launch_pass1(p, u0, n, p->d_S, p->s_pitch, p1_chirp(p), st))) break;
        // only the row kernel writes the slab: pass 1 overlaps the copy
        // that still drains it
        if (t >= 2) GB_CUDA(cudaStreamWaitEvent(st, r.copied[b], 0));
        const gbsp::RowsArgs a =
            rows_args(p, p->d_S, p->s_pitch, u0, n, r.slab[b], out_pitch, u0 + n, u0, hi_first - n);
        if ((rc = launch_rows_args(p, a, st))) break;
        GB_CUDA(cudaEventRecord(r.done[b], st));
        GB_CUDA(cudaStreamWaitEvent(r.cs, r.done[b], 0));
        GB_CUDA(cudaMemcpy2DAsync(host + (size_t)u0 * row_bytes, row_bytes, r.slab[b], row_bytes, row_bytes, n,
                                  cudaMemcpyDeviceToHost, r.cs));
        if (n_hi > 0)
            GB_CUDA(cudaMemcpy2DAsync(host + (size_t)hi_first * row_bytes, row_bytes,
                                      static_cast<char*>(r.slab[b]) + (size_t)n * row_bytes, row_bytes, row_bytes,
                                      n_hi, cudaMemcpyDeviceToHost, r.cs));
        GB_CUDA(cudaEventRecord(r.copied[b], r.cs));
    }
    cudaError_t e1 = cudaStreamSynchronize(r.cs);
    cudaError_t e2 = cudaStreamSynchronize(st);
    if (rc) return rc;
    if (e1 != cudaSuccess || e2 != cudaSuccess)
        return set_error(GBSP_ERR_CUDA, std::string("gbsp_execute_to_host: ") +
                                            cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
    return read_device_flags(p);
}
