// gbsp_kernels.cuh -- the device side of the binary-sparse 2-D R2C FFT
// (templates and inline device functions only, so several translation units
// can each instantiate their part; the one-time table kernels are in
// gbsp_tables.cuh).
//
//   k_twiddle_sum        pass 1: S[u][j] = sum_{r in column j} W_rows^{u*r}
//   k_bluestein_rows     pre-chirp + FFT + filter + inverse FFT + post-chirp and
//                        the Hermitian-paired R2C row writer, one row per CTA
//                        (or K channels per row: a thread-block cluster, or one
//                        CTA running them in turn)
#pragma once
#include <cooperative_groups.h>
#include "gbsp_fft.cuh"
#include "gbsp_layout.h"

namespace cg = cooperative_groups;

namespace gbsp {

// ---------------------------------------------------------------------------
// Exact integer phase helpers
// ---------------------------------------------------------------------------

// x mod n for any 32-bit x and 2 <= n < 2^31 with magic = ceil(2^32 / n):
// umulhi(x, magic) is floor(x/n) or floor(x/n)+1, corrected by one add.
// (n == 1 uses magic 0 and only ever sees x == 0.)
__device__ __forceinline__ uint32_t mod_magic(uint32_t x, uint32_t n, uint32_t magic) {
    uint32_t q = __umulhi(x, magic);
    uint32_t r = x - q * n;
    return ((int32_t)r < 0) ? r + n : r;
}

// (u*r) mod rows; BIG handles rows > 65535 where u*r may not fit 32 bits:
// the 64-bit product is reduced with magic = ceil(2^64 / rows) as the
// 32-bit case is (u, r < rows < 2^31 keep the quotient estimate within one).
template <bool BIG>
__device__ __forceinline__ uint32_t mulmod_rows(uint32_t u, uint32_t r, uint32_t rows, uint32_t magic,
                                                unsigned long long magic64) {
    if (BIG) {
        const unsigned long long x = (unsigned long long)u * r;
        const unsigned long long q = __umul64hi(x, magic64);
        const long long rem = (long long)(x - q * rows);
        return (uint32_t)(rem < 0 ? rem + rows : rem);
    }
    return mod_magic(u * r, rows, magic);
}

// ---------------------------------------------------------------------------
// mbarrier + bulk-copy helpers (inline PTX).  Every wait is bounded: after
// WAIT_LIMIT polls the kernel records ERR_TIMEOUT in *err and carries on, so
// no barrier can hang the GPU; the host reports the flag as an error.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// true if the phase completed, false after WAIT_LIMIT polls
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (long long i = 0; i < WAIT_LIMIT; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
// global -> this CTA's shared memory, completion counted on bar
__device__ __forceinline__ void bulk_copy_g2s(void* dst_smem, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst_smem)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) accesses
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---------------------------------------------------------------------------
// Pass 1: twiddle sums over each column's nonzero rows, times the chirp.
//
// A work item is (block of 32*KU Bluestein rows, window of cw consecutive
// columns).  On the host each window's nonzeros are cut into at most
// cw + P1_WARPS tasks: a column of degree d becomes ceil(d / T) contiguous
// parts with T = max(32, ceil(window nnz / P1_WARPS)), so no task exceeds a
// warp's fair share.  The warps of the CTA pull tasks from a shared counter
// longest first; lane l owns rows u = ubase + l + 32*kk.  Each task's sums
// land in their own column of a shared-memory tile, and the window is written
// by summing every column's parts in a fixed order (Kahan-compensated when a
// column has several), so the result is balanced and deterministic.
//
// Per nonzero r the lane reduces its phase (u*r) mod rows exactly with an
// integer multiply-high and reads W_rows^p from the table staged in shared
// memory.  The rows u + 32*kk in between follow from the exactly looked-up
// step z = W_rows^{(32*r) mod rows}: the first by one complex product, the
// next ones by the three-term recurrence w[k+1] = 2cos(arg z)*w[k] - w[k-1]
// (two FMAs instead of a four-operation product; its rounding error grows at
// most linearly in the steps taken).  Every P1_RESEED rows the value is
// looked up exactly again, so no twiddle is more than P1_RESEED-1 steps away
// from a correctly rounded table entry.  Sums of a
// batch of 32 nonzeros are added to the task total; for tasks of at least
// kahan_min nonzeros that addition is Kahan-compensated.  The window's
// results (times chirp[c] when a chirp table is given) leave as whole
// 512-byte row segments of S, in column order, zero for empty columns --
// ready for a bulk copy.
//
// The reference evaluates __sincosf of a float angle per (u, nonzero), one
// output row per thread, and writes strided 8-byte values
// (src/sparse_fft_bluestein.cu:366-397).
// ---------------------------------------------------------------------------
// Pass-1 row twiddle tables in shared memory (TAB):
//   TAB_FULL   tab[p] = W^p, p < rows
//   TAB_HALF   tab[p] = W^p, p <= rows/2; the rest by conjugate symmetry
//   TAB_TWO    two levels for tall matrices: tab[i] = W^i (i < TWO_LO),
//              tab[TWO_LO + j] = W^(TWO_LO*j); W^p = hi[p / TWO_LO] * lo[p % TWO_LO]
template <int TAB>
__device__ __forceinline__ float2 row_twiddle(const float2* tab, uint32_t p, uint32_t rows, uint32_t hr) {
    if (TAB == TAB_FULL) return tab[p];
    if (TAB == TAB_TWO) return cmul(tab[TWO_LO + (p >> TWO_LO_BITS)], tab[p & (TWO_LO - 1)]);
    bool hi = p > hr;
    float2 w = tab[hi ? rows - p : p];
    w.y = hi ? -w.y : w.y;
    return w;
}

// one nonzero as a warp shares it: row, reseed step, and -W^{(32*r) mod rows}
struct NzInfo {
    uint32_t r, step;
    float wx, wy;
};

// EXACT: every twiddle is the table entry at its exact phase
// (u*r) mod rows -- the phase of row u + 32*(kk+1) is that of row u + 32*kk
// plus (32*r) mod rows, reduced by one compare -- with no recurrence.
template <typename IDX, int TAB, bool BIG, int KU, bool EXACT>
__device__ __forceinline__ void column_sums_warp(const IDX* __restrict__ row_idx, int beg, int end,
                                                 const float2* tab, NzInfo* info, uint32_t u_lane,
                                                 uint32_t rows, uint32_t magic, unsigned long long magic64,
                                                 int lane, bool compensated,
                                                 float2 (&acc)[KU]) {
    float2 cmp[KU];
#pragma unroll
    for (int i = 0; i < KU; i++) { acc[i] = make_float2(0.f, 0.f); cmp[i] = make_float2(0.f, 0.f); }
    const uint32_t hr = rows / 2;
    for (int p0 = beg; p0 < end; p0 += 32) {
        const int cnt = min(32, end - p0);
        if (lane < cnt) {
            const uint32_t r = (uint32_t)row_idx[p0 + lane];
            const uint32_t d = mulmod_rows<BIG>(32u, r, rows, magic, magic64);
            const float2 wd = row_twiddle<TAB>(tab, d, rows, hr);
            const uint32_t st = EXACT ? d
                                : (KU > P1_RESEED) ? mulmod_rows<BIG>((uint32_t)P1_RESEED, d, rows, magic, magic64) : 0u;
            info[lane] = NzInfo{r, st, -wd.x, -wd.y};  // the step, negated
        }
        __syncwarp();
        if constexpr (EXACT) {
            float2 blk[KU];
#pragma unroll
            for (int i = 0; i < KU; i++) blk[i] = make_float2(0.f, 0.f);
#pragma unroll 2
            for (int i = 0; i < cnt; i++) {
                const NzInfo z = info[i];
                uint32_t p = mulmod_rows<BIG>(u_lane, z.r, rows, magic, magic64);
#pragma unroll
                for (int kk = 0; kk < KU; kk++) {
                    blk[kk] = __fadd2_rn(blk[kk], row_twiddle<TAB>(tab, p, rows, hr));
                    const uint32_t pn = p + z.step;
                    p = min(pn, pn - rows);
                }
            }
            __syncwarp();
            if (compensated) {
#pragma unroll
                for (int kk = 0; kk < KU; kk++) {
                    float y = blk[kk].x - cmp[kk].x;
                    float t = acc[kk].x + y;
                    cmp[kk].x = (t - acc[kk].x) - y;
                    acc[kk].x = t;
                    y = blk[kk].y - cmp[kk].y;
                    t = acc[kk].y + y;
                    cmp[kk].y = (t - acc[kk].y) - y;
                    acc[kk].y = t;
                }
            } else {
#pragma unroll
                for (int kk = 0; kk < KU; kk++) { acc[kk].x += blk[kk].x; acc[kk].y += blk[kk].y; }
            }
            continue;
        }
        // Rows kk = 4g+1 and 4g+2 are carried negated, so every operation
        // below is a plain packed FP32x2 add or FMA with no operand negation:
        //   n1 = w0 * (-z)          = -w1
        //   n2 = c2 * n1 + w0       = -(c2*w1 - w0) = -w2
        //   w3 = (-c2) * n2 + n1    =   c2*w2 - w1
        // Negation is exact and round-to-nearest is symmetric, so each value
        // is bitwise the negative of the one the plain recurrence gives; the
        // negated partial sums are flipped back after the batch.
        static_assert(P1_RESEED == 4 && KU % 4 == 0, "pass-1 rows come in groups of four");
        float2 blk[KU];
#pragma unroll
        for (int i = 0; i < KU; i++) blk[i] = make_float2(0.f, 0.f);
#pragma unroll 4
        for (int i = 0; i < cnt; i++) {
            const NzInfo z = info[i];  // one broadcast 16-byte load
            const float2 nz = make_float2(z.wx, z.wy);
            const float c2 = -2.f * z.wx;  // 2cos(arg z), exact
            const float2 c2p = make_float2(c2, c2), mc2p = make_float2(-c2, -c2);
            uint32_t p = mulmod_rows<BIG>(u_lane, z.r, rows, magic, magic64);
#pragma unroll
            for (int g = 0; g < KU; g += 4) {
                const float2 w0 = row_twiddle<TAB>(tab, p, rows, hr);
                if (g + 4 < KU) {
                    const uint32_t pn = p + z.step;
                    p = min(pn, pn - rows);
                }
                const float2 n1 = cmul(w0, nz);
                const float2 n2 = __ffma2_rn(c2p, n1, w0);
                const float2 w3 = __ffma2_rn(mc2p, n2, n1);
                blk[g] = __fadd2_rn(blk[g], w0);
                blk[g + 1] = __fadd2_rn(blk[g + 1], n1);
                blk[g + 2] = __fadd2_rn(blk[g + 2], n2);
                blk[g + 3] = __fadd2_rn(blk[g + 3], w3);
            }
        }
        __syncwarp();
#pragma unroll
        for (int kk = 0; kk < KU; kk++)
            if (kk % 4 == 1 || kk % 4 == 2) blk[kk] = make_float2(-blk[kk].x, -blk[kk].y);
        if (compensated) {
#pragma unroll
            for (int kk = 0; kk < KU; kk++) {
                float y = blk[kk].x - cmp[kk].x;
                float t = acc[kk].x + y;
                cmp[kk].x = (t - acc[kk].x) - y;
                acc[kk].x = t;
                y = blk[kk].y - cmp[kk].y;
                t = acc[kk].y + y;
                cmp[kk].y = (t - acc[kk].y) - y;
                acc[kk].y = t;
            }
        } else {
#pragma unroll
            for (int kk = 0; kk < KU; kk++) { acc[kk].x += blk[kk].x; acc[kk].y += blk[kk].y; }
        }
    }
}

// One matrix's pass-1 inputs for one tile of Bluestein rows [u0, u0+tile_rows).
// win_slot0[w*(cw+1) + lc]: first tile column of window w's column lc
// (entry cw = tasks in the window); win_task[w*vmax + i] = nonzero range
// (begin, end) and win_task_col[...] its tile column, longest task first.
// S row u-u0 gets columns [0, s_cols), zero past cols.
struct P1Args {
    const void* row_idx;
    const uint8_t* win_slot0;
    const int2* win_task;
    const uint8_t* win_task_col;
    const float2* row_tab;
    const float2* chirp;  // nullptr: raw column sums
    float2* S;
    size_t s_pitch;
    int cw, cols, s_cols, ntab, rows, u0, tile_rows, kahan_min;
    uint32_t magic;
    unsigned long long magic64;  // ceil(2^64 / rows), for rows > 65535
    // k_twiddle_sum's item queue: [0] next item, [1] CTAs done; zero before
    // the first launch, and the last CTA of each launch zeroes it again
    unsigned int* queue;
};

struct P1Shared {
    int next_task;
    unsigned int item;
    int slot0[64 + 1];
    float2 chirp[64];
};

__device__ __forceinline__ long p1_items(const P1Args& a, int ublk) {
    return (long)((a.tile_rows + ublk - 1) / ublk) * ((a.s_cols + a.cw - 1) / a.cw);
}

// Work item `it` of one matrix: all tasks of one (row block, column window),
// then the window's tile written to S.  Whole CTA; tab holds the matrix's
// twiddle table.
template <typename IDX, int TAB, bool BIG, int KU, bool EXACT>
__device__ __forceinline__ void p1_item(const P1Args& a, long it, float2* stage, NzInfo* info_all,
                                        const float2* tab, P1Shared& sh) {
    constexpr int UBLK = 32 * KU;
    const int pitch = p1_pitch(a.cw), vmax = p1_vmax(a.cw), cw = a.cw;
    const int lane = threadIdx.x & 31;
    NzInfo* info = info_all + (threadIdx.x >> 5) * 32;
    const int n_win = (a.s_cols + cw - 1) / cw;
    const int ub = (int)(it / n_win);
    const int w = (int)(it - (long)ub * n_win);
    const int ul0 = ub * UBLK;
    const int c0 = w * cw;
    const uint8_t* slot0 = a.win_slot0 + (size_t)w * (cw + 1);
    if (threadIdx.x <= cw) sh.slot0[threadIdx.x] = slot0[threadIdx.x];
    if (threadIdx.x < cw) {
        const int c = c0 + threadIdx.x;
        sh.chirp[threadIdx.x] = (a.chirp && c < a.cols) ? a.chirp[c] : make_float2(1.f, 0.f);
    }
    const int ntask = slot0[cw];
    const uint32_t u_lane = (uint32_t)(a.u0 + ul0 + lane) % (uint32_t)a.rows;
    const IDX* row_idx = static_cast<const IDX*>(a.row_idx);
    for (;;) {
        int i = 0;
        if (lane == 0) i = atomicAdd(&sh.next_task, 1);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= ntask) break;
        const int2 range = a.win_task[(size_t)w * vmax + i];
        const int col = a.win_task_col[(size_t)w * vmax + i];
        float2 acc[KU];
        column_sums_warp<IDX, TAB, BIG, KU, EXACT>(row_idx, range.x, range.y, tab, info, u_lane,
                                                 (uint32_t)a.rows, a.magic, a.magic64, lane,
                                                 a.kahan_min > 0 && range.y - range.x >= a.kahan_min, acc);
#pragma unroll
        for (int kk = 0; kk < KU; kk++) stage[(lane + 32 * kk) * pitch + col] = acc[kk];
    }
    __syncthreads();
    // The window leaves through S.  Columns of at most one part: each thread
    // keeps one column (the block size is a multiple of cw, so every element
    // it visits has column threadIdx.x % cw) and walks its rows, with the
    // column's part, chirp and S address in registers; a warp stores 32
    // consecutive columns of one row.  Columns of several parts (heavy
    // columns cut for balance) are summed afterwards with one thread per
    // row, so their compensated sums do not hold up the other lanes.
    const int ncol = min(cw, a.s_cols - c0);
    const int cw_log2 = __ffs(cw) - 1;  // every pass-1 shape's window is 16, 32 or 64 columns
    const int rend = min(UBLK, a.tile_rows - ul0);
    const int lc = threadIdx.x & (cw - 1);
    {
        const int p0 = sh.slot0[lc], np = sh.slot0[lc + 1] - p0;
        if (lc < ncol && np <= 1) {
            const float2 ch = sh.chirp[lc];
            const int rstep = blockDim.x >> cw_log2;
            int row = threadIdx.x >> cw_log2;
            float2* dst = a.S + (size_t)(ul0 + row) * a.s_pitch + c0 + lc;
            const size_t dstep = (size_t)rstep * a.s_pitch;
            for (; row < rend; row += rstep, dst += dstep) {
                const float2 v = np > 0 ? stage[row * pitch + p0] : make_float2(0.f, 0.f);
                *dst = cmul(v, ch);
            }
        }
    }
    // the window's several-part columns, as a bit mask (every warp forms it)
    uint64_t multi = 0;
    for (int h = 0; h < cw; h += 32) {
        const int c = h + (int)(threadIdx.x & 31);
        const bool m = c < ncol && sh.slot0[c + 1] - sh.slot0[c] > 1;
        multi |= (uint64_t)__ballot_sync(0xffffffffu, m) << h;
    }
    const int n_multi = __popcll(multi);
    for (int e = threadIdx.x; e < n_multi * UBLK; e += blockDim.x) {
        const int j = e / UBLK, row = e - j * UBLK;
        if (row >= rend) continue;
        uint64_t mm = multi;
        for (int t = 0; t < j; t++) mm &= mm - 1;  // drop the j lowest set bits
        const int c = __ffsll((long long)mm) - 1;
        const int q0 = sh.slot0[c], q1 = sh.slot0[c + 1];
        const float2* srow = stage + row * pitch;
        float2 v = srow[q0], comp = make_float2(0.f, 0.f);
        for (int k = q0 + 1; k < q1; k++) {  // parts in a fixed order, compensated
            float y = srow[k].x - comp.x;
            float t = v.x + y;
            comp.x = (t - v.x) - y;
            v.x = t;
            y = srow[k].y - comp.y;
            t = v.y + y;
            comp.y = (t - v.y) - y;
            v.y = t;
        }
        a.S[(size_t)(ul0 + row) * a.s_pitch + c0 + c] = cmul(v, sh.chirp[c]);
    }
    if (threadIdx.x == 0) sh.next_task = 0;
    __syncthreads();
}

template <typename IDX, int TAB, bool BIG, int KU, bool EXACT>
__global__ void __launch_bounds__(P1_THREADS, 1) k_twiddle_sum(P1Args a) {
    extern __shared__ float4 smem_raw[];
    __shared__ P1Shared sh;
    float2* stage = reinterpret_cast<float2*>(smem_raw);
    NzInfo* info_all = reinterpret_cast<NzInfo*>(stage + (size_t)32 * KU * p1_pitch(a.cw));
    float2* tab = reinterpret_cast<float2*>(info_all + P1_WARPS * 32);
    for (int i = threadIdx.x; i < a.ntab; i += blockDim.x) tab[i] = a.row_tab[i];
    if (threadIdx.x == 0) sh.next_task = 0;
    // Items are handed out one at a time from a device counter, so CTAs
    // whose windows hold fewer nonzeros take more items and all finish
    // together.  p1_item ends on a barrier, so thread 0 rewrites sh.item only
    // after every thread has read it.
    const long nitems = p1_items(a, 32 * KU);
    for (;;) {
        if (threadIdx.x == 0) sh.item = atomicAdd(&a.queue[0], 1u);
        __syncthreads();
        const long it = sh.item;
        if (it >= nitems) break;
        p1_item<IDX, TAB, BIG, KU, EXACT>(a, it, stage, info_all, tab, sh);
    }
    // the last CTA out (every other one has stopped taking items) rearms the
    // queue for the next launch
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&a.queue[1], 1u) == gridDim.x - 1) {
            atomicExch(&a.queue[0], 0u);
            atomicExch(&a.queue[1], 0u);
        }
    }
}

// Batched pass 1: the work items of many matrices (item_begin: first item of
// each matrix, item_begin[nmat] = total) handed out by a device work queue,
// one item per grab.  Items are grabbed in increasing order, so a CTA moves
// forward through the matrices and reloads the twiddle table only when it
// enters a new one.  *queue must be 0 at launch.
template <typename IDX, int TAB, bool BIG, int KU, bool EXACT>
__global__ void __launch_bounds__(P1_THREADS, 1)
k_twiddle_sum_batch(const P1Args* __restrict__ args, const long* __restrict__ item_begin, int nmat,
                    unsigned long long* queue) {
    extern __shared__ float4 smem_raw[];
    __shared__ P1Shared sh;
    __shared__ P1Args cur;
    __shared__ long s_it;
    __shared__ int s_m;
    float2* stage = reinterpret_cast<float2*>(smem_raw);
    int loaded = -1;
    if (threadIdx.x == 0) { sh.next_task = 0; s_m = 0; }
    __syncthreads();
    const long total = item_begin[nmat];
    for (;;) {
        if (threadIdx.x == 0) {
            const long it = (long)atomicAdd(queue, 1ull);
            int m = s_m;
            while (m < nmat && item_begin[m + 1] <= it) m++;
            s_it = it;
            s_m = m;
        }
        __syncthreads();
        const long it = s_it;
        const int m = s_m;
        if (it >= total) break;
        if (m != loaded) {
            if (threadIdx.x == 0) cur = args[m];
            __syncthreads();
            NzInfo* info_all = reinterpret_cast<NzInfo*>(stage + (size_t)32 * KU * p1_pitch(cur.cw));
            float2* tab = reinterpret_cast<float2*>(info_all + P1_WARPS * 32);
            for (int i = threadIdx.x; i < cur.ntab; i += blockDim.x) tab[i] = cur.row_tab[i];
            __syncthreads();
            loaded = m;
        }
        NzInfo* info_all = reinterpret_cast<NzInfo*>(stage + (size_t)32 * KU * p1_pitch(cur.cw));
        float2* tab = reinterpret_cast<float2*>(info_all + P1_WARPS * 32);
        p1_item<IDX, TAB, BIG, KU, EXACT>(cur, it - item_begin[m], stage, info_all, tab, sh);
    }
}

// ---------------------------------------------------------------------------
// Bluestein rows.  Channel q of K (the CTA's rank in its cluster) holds
//   y_q[n] = sum_{c = n mod Lp} pre[q][c] * x[u][c]          (n < Lp)
// where x = S (pass 1 already multiplied by the chirp), runs the forward DIF
// FFT of length Lp, multiplies by the channel's filter spectrum (in the
// network's digit-reversed order, scaled by 1/L), and runs the inverse DIT
// FFT, leaving Z_q[n] in natural order.  The length-L convolution result is
//   y[c] = sum_q post[q][c] * Z_q[c mod Lp]
// read across the cluster's shared memories (DSMEM).  Since the 2-D input is
// real, F[rows-u][v] = conj(F[u][(cols-v) mod cols]), so one Bluestein row u
// (u <= rows/2) writes output rows u and rows-u, each with 16-byte stores of
// two complex values.
//
// A single-channel row arrives with one bulk copy (cp.async.bulk) straight
// into the FFT buffer.  A channel of a multi-channel row whose columns fit
// the channel (columns rounded up to even <= Lp) is read from global memory
// by its first forward stage, pre-twiddle included (no copy, zero fill or
// pre-twiddle pass; with a one-stage network, by the bulk copy); otherwise
// (several columns folding onto one slot) it is added section by section.
//
// Shared memory: the row buffer, then the twiddles of stages >= 1 (loaded
// once per CTA); stage 0's twiddles stream from L2.
//
// The reference runs 2F+4 launches per tile of rows with a global round trip
// per stage (src/sparse_fft_bluestein.cu:2327-2370) and writes 8-byte stores
// in bluestein_finalize_kernel (:469-486).
// ---------------------------------------------------------------------------
// One matrix's row-kernel inputs for one tile of Bluestein rows [u0, u0+tile_rows).
struct RowsArgs {
    const float2* S;
    size_t s_pitch;
    const float2* pre;
    const float2* post;
    const float2* filt;
    const float2* fft_tw;
    float2* out;
    size_t out_pitch;
    int K, rows, cols, u0, tile_rows;
    // output row r goes to out row r - map_lo when r < map_split, else to
    // r - map_hi (identity: map_split = INT_MAX, map_lo = 0); lets a tile of
    // rows u and rows-u land in a small slab for streaming to the host
    int map_split, map_lo, map_hi;
    // ROW_SEQ: per-CTA scratch for the first K-1 channels of a row,
    // (K-1) x Lp complex per CTA, CTA b at zscratch + b*(K-1)*Lp
    float2* zscratch;
    // direct plans (cols smooth: one forward FFT of length cols instead of
    // the Bluestein convolution): drev[c] = where the forward network leaves
    // frequency c; nullptr for Bluestein plans
    const int* drev;
};

// How the K channels of a long row are laid out on the GPU.
//   ROW_SINGLE  K == 1, one CTA per row
//   ROW_CLUSTER one CTA per channel, the K CTAs of a row one thread-block
//               cluster; the output combine reads the peers' buffers (DSMEM)
//   ROW_SEQ     one CTA runs the K channels one after another; the first K-1
//               results wait in an L2-resident scratch for the combine
//   ROW_SEQW    ROW_SEQ for more than MAX_CHANNELS channels (very wide rows;
//               a separate instance, so the common one keeps its registers)
//   ROW_DIRECT  K == 1 and a direct plan (cols smooth: one forward FFT of
//               length cols, no Bluestein convolution), its own instance so
//               the Bluestein one keeps its registers
constexpr int ROW_SINGLE = 0, ROW_CLUSTER = 1, ROW_SEQ = 2, ROW_SEQW = 3, ROW_DIRECT = 4;

// One Bluestein row t of the tile (u = u0 + t), channel q of K: input,
// forward network, filter, inverse network, Hermitian-paired output.  Whole
// CTA (with the cluster when K > 1); ends on a barrier, so the next row may
// overwrite buf at once.  Direct plans (a.drev set, K = 1) run only the
// forward network over the row's cols points and gather the spectrum through
// drev in the writer.
// DIRECT: 0 never (Bluestein), 1 always (ROW_DIRECT), 2 per row from a.drev
// (the batched kernel, whose matrices mix both kinds)
template <int MAXR, int MODE, int DIRECT = (MODE == ROW_DIRECT ? 1 : 0)>
__device__ __forceinline__ void bluestein_row(const RowsArgs& a, const FFTDesc& fd, int t, int q, float2* buf,
                                              const float2* twr, const float2* const* zsrc, uint64_t* bar,
                                              uint32_t& parity, int& err_bits) {
    constexpr bool CLUSTER = MODE == ROW_CLUSTER;
    constexpr bool MULTI = MODE == ROW_CLUSTER || MODE == ROW_SEQ || MODE == ROW_SEQW;
    constexpr bool SEQ = MODE == ROW_SEQ || MODE == ROW_SEQW;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int Lp = fd.Lp, K = a.K, cols = a.cols;
    const int half_slots = (int)(a.out_pitch >> 1);
    const int hc = cols / 2;
    const int cols_even = (cols + 1) & ~1;
    // stage 0 twiddles stream from global memory (read-only path), the rest
    // sit in shared memory
    const float2* tw0 = a.fft_tw + fd.twoff[0];
    auto tw_smem = [&](int s) -> const float2* { return twr + (fd.twoff[s] - fd.rest_base); };
    const int u = a.u0 + t;
    const float2* srow = a.S + (size_t)t * a.s_pitch;
    const bool direct = DIRECT == 1 || (DIRECT == 2 && a.drev != nullptr);
    bool ok = true;
    // ROW_SEQ runs every channel of the row here; the other modes one
    const int q_end = SEQ ? K : q + 1;
    for (int qc = SEQ ? 0 : q; qc < q_end; qc++) {
        const float2* preq = a.pre + (size_t)qc * cols;
        const float2* filtq = a.filt + (size_t)qc * Lp;
        // Sequential channels whose row fits the channel (no fold) and whose
        // network has a separate first stage read the row straight from
        // global memory in that stage, pre-twiddle included
        const int S1 = fd.nst - 1;
        const bool g0 = (SEQ || CLUSTER) && cols_even <= Lp && S1 > 0;
        // (a single channel always has cols_even <= Lp: L >= 2*cols - 1)
        if (g0) {
        } else if (!MULTI || cols_even <= Lp) {
            if (tid == 0) {
                fence_proxy_async_smem();
                mbar_expect_tx(bar, (uint32_t)cols_even * 8u);
                bulk_copy_g2s(buf, srow, (uint32_t)cols_even * 8u, bar);
            }
            for (int i = cols_even + tid; i < Lp; i += nt) buf[i] = make_float2(0.f, 0.f);
            if (!mbar_wait_bounded(bar, parity)) err_bits |= ERR_TIMEOUT;
            parity ^= 1u;
            if (MULTI && qc != 0)  // channel pre-twiddle (channel 0's is 1)
                for (int c = tid; c < cols; c += nt) buf[c] = cmul(buf[c], __ldg(preq + c));
            __syncthreads();
        } else if constexpr (MODE == ROW_SEQW) {
            // Several input columns fold onto one slot: slot n gets
            // sum_j pre[n + j*Lp] * x[n + j*Lp], up to K/2 + 1 sections
            // (very wide rows, K up to MAX_SEQ_CHANNELS); loads of two
            // sections per step
            for (int n = tid; n < Lp; n += nt) {
                float2 acc = make_float2(0.f, 0.f);
                for (int c = n; c < cols; c += 2 * Lp) {
                    const int c2 = c + Lp;
                    const float2 x0 = __ldcg(srow + c), p0 = __ldg(preq + c);
                    const float2 x1 = (c2 < cols) ? __ldcg(srow + c2) : make_float2(0.f, 0.f);
                    const float2 p1 = (c2 < cols) ? __ldg(preq + c2) : make_float2(0.f, 0.f);
                    acc = cadd(acc, cadd(cmul(x0, p0), cmul(x1, p1)));
                }
                buf[n] = acc;
            }
            __syncthreads();
        } else if constexpr (MULTI) {
            // Several input columns fold onto one slot: slot n gets
            // sum_j pre[n + j*Lp] * x[n + j*Lp].  Every channel reads the whole
            // S row, so it is loaded to stay in L2 for the next channel (an
            // evict-first load made each channel re-read it from DRAM).
            // Each thread owns its slots, so
            // no zero fill or barrier between sections; all of a slot's loads
            // are issued before its products.
            // L = K*Lp >= 2*cols - 1 gives cols/Lp <= K/2 + 1/(2Lp): at most
            // K/2 + 1 sections
            constexpr int MAXSEC = MAX_CHANNELS / 2 + 1;
            for (int n = tid; n < Lp; n += nt) {
                float2 xv[MAXSEC], pv[MAXSEC];
#pragma unroll
                for (int j = 0; j < MAXSEC; j++) {
                    const int c = n + j * Lp;
                    const bool ok = c < cols;
                    xv[j] = ok ? __ldcg(srow + c) : make_float2(0.f, 0.f);
                    pv[j] = ok ? __ldg(preq + c) : make_float2(0.f, 0.f);
                }
                float2 acc = make_float2(0.f, 0.f);
#pragma unroll
                for (int j = 0; j < MAXSEC; j++) acc = cadd(acc, cmul(xv[j], pv[j]));
                buf[n] = acc;
            }
            __syncthreads();
        }
        // forward DIF, filter multiply fused with the last stage, inverse DIT
        const float2* none = nullptr;
        // (a direct plan runs the forward network alone, its last stage --
        // span 1, twiddles exactly 1 -- included: X in digit-reversed order)
        const int S_fwd = direct ? S1 + 1 : S1;
        if ((SEQ || CLUSTER) && g0) {
            ok &= (qc == 0) ? fft_stage0_global_dispatch<MAXR, false>(fd.R[0], buf, srow, none, cols, fd.m[0], tw0,
                                                                       tid, nt)
                            : fft_stage0_global_dispatch<MAXR, true>(fd.R[0], buf, srow, preq, cols, fd.m[0], tw0,
                                                                      tid, nt);
            __syncthreads();
        } else if (S_fwd > 0) {
            ok &= fft_stage_dispatch<0, MAXR, true>(fd.R[0], buf, Lp, fd.m[0], fd.magic[0], tw0, none, tid, nt);
            __syncthreads();
        }
        for (int s = 1; s < S_fwd; s++) {
            ok &= fft_stage_dispatch<0, MAXR, false>(fd.R[s], buf, Lp, fd.m[s], fd.magic[s], tw_smem(s), none,
                                                     tid, nt);
            __syncthreads();
        }
        if (direct) continue;
        ok &= fft_stage_dispatch<2, MAXR, false>(fd.R[S1], buf, Lp, 1, 0u, none, filtq, tid, nt);
        __syncthreads();
        for (int s = S1 - 1; s >= 1; s--) {
            ok &= fft_stage_dispatch<1, MAXR, false>(fd.R[s], buf, Lp, fd.m[s], fd.magic[s], tw_smem(s), none,
                                                     tid, nt);
            __syncthreads();
        }
        if (S1 > 0) {
            ok &= fft_stage_dispatch<1, MAXR, true>(fd.R[0], buf, Lp, fd.m[0], fd.magic[0], tw0, none, tid, nt);
            __syncthreads();
        }
        if (SEQ && qc < K - 1) {  // park the channel for the combine
            float2* dst = a.zscratch + ((size_t)blockIdx.x * (K - 1) + qc) * Lp;
            for (int i = tid; i < Lp; i += nt) dst[i] = buf[i];
            __syncthreads();
        }
    }  // channels
    if (!ok) err_bits |= ERR_RADIX;
    if (CLUSTER) cg::this_cluster().sync();

    // Hermitian-paired row writer
    const int u2 = (u == 0) ? 0 : a.rows - u;
    const bool two = (u2 != u);
    const int nslots = two ? 2 * half_slots : half_slots;
    // a cluster splits the row's output slots among its CTAs
    const int qw = CLUSTER ? q : 0, kw = CLUSTER ? K : 1;
    const int lo = (int)((long)qw * nslots / kw), hi = (int)((long)(qw + 1) * nslots / kw);
    if (!MULTI) {
        // Each thread takes WU slots per pass and issues all their loads (post
        // chirp from L2, Z from shared memory) before any product, so the L2
        // latency is paid once per WU slots.
        constexpr int WU = 4;
        for (int s0 = lo + tid; s0 < hi; s0 += WU * nt) {
            int col[WU][2];
            float2 pv[WU][2], zv[WU][2];
#pragma unroll
            for (int w = 0; w < WU; w++) {
                const int s = s0 + w * nt;
                const int sel = s >= half_slots;
                const int v = 2 * (s - sel * half_slots);
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int vv = v + e;
                    const int c = (s >= hi || vv > hc) ? -1 : sel ? (vv == 0 ? 0 : cols - vv) : vv;
                    col[w][e] = c;
                    if (direct) {  // F[u][c] = X[c], no chirp; (1, 0) keeps the product exact
                        pv[w][e] = make_float2(1.f, 0.f);
                        zv[w][e] = buf[c < 0 ? 0 : __ldg(a.drev + c)];
                    } else {
                        pv[w][e] = (c >= 0) ? __ldg(a.post + c) : make_float2(0.f, 0.f);
                        zv[w][e] = buf[c < 0 ? 0 : c];
                    }
                }
            }
#pragma unroll
            for (int w = 0; w < WU; w++) {
                const int s = s0 + w * nt;
                if (s >= hi) break;
                const int sel = s >= half_slots;
                const int v = 2 * (s - sel * half_slots);
                float2 o0 = col[w][0] < 0 ? make_float2(0.f, 0.f) : cmul(zv[w][0], pv[w][0]);
                float2 o1 = col[w][1] < 0 ? make_float2(0.f, 0.f) : cmul(zv[w][1], pv[w][1]);
                if (sel) {
                    o0.y = -o0.y;
                    o1.y = -o1.y;
                }
                const int row = sel ? u2 : u;
                const int drow = row < a.map_split ? row - a.map_lo : row - a.map_hi;
                float4* dst = reinterpret_cast<float4*>(a.out + (size_t)drow * a.out_pitch + v);
                __stcs(dst, make_float4(o0.x, o0.y, o1.x, o1.y));
            }
        }
    } else if constexpr (SEQ) {
        // Sequential channels: channels 0..K-2 wait in this CTA's scratch
        // (global memory, L2-resident), channel K-1 is in buf.  Each thread
        // takes WS slots per pass and, channel by channel, issues all of the
        // slots' loads (parked values and post chirps from L2) before any
        // product, so the L2 latency is paid once per channel and WS slots
        // rather than once per value.  The channels are summed in order.
        constexpr int WS = 4;
        const float2* zs0 = a.zscratch + (size_t)blockIdx.x * (K - 1) * Lp;
        if (K == 2) {
            // Two channels (Lp >= cols, so both read slot c itself): all of
            // a pass's loads are issued before any product, with no channel
            // loop and no wrap of c; the sum runs in the general order.
            const float2* p0 = a.post;
            const float2* p1 = a.post + cols;
            for (int s0 = lo + tid; s0 < hi; s0 += WS * nt) {
                float2 za[WS][2], pa[WS][2], zb[WS][2], pb[WS][2];
#pragma unroll
                for (int w = 0; w < WS; w++) {
                    const int s = s0 + w * nt;
                    const int sel = s >= half_slots;
                    const int v = 2 * (s - sel * half_slots);
#pragma unroll
                    for (int e = 0; e < 2; e++) {
                        const int vv = v + e;
                        const int c = (s >= hi || vv > hc) ? 0 : sel ? (vv == 0 ? 0 : cols - vv) : vv;
                        pa[w][e] = __ldg(p0 + c);
                        za[w][e] = __ldcg(zs0 + c);
                        pb[w][e] = __ldg(p1 + c);
                        zb[w][e] = buf[c];
                    }
                }
#pragma unroll
                for (int w = 0; w < WS; w++) {
                    const int s = s0 + w * nt;
                    if (s >= hi) break;
                    const int sel = s >= half_slots;
                    const int v = 2 * (s - sel * half_slots);
                    float2 o[2];
#pragma unroll
                    for (int e = 0; e < 2; e++) {
                        const float2 y = cadd(cadd(make_float2(0.f, 0.f), cmul(za[w][e], pa[w][e])),
                                              cmul(zb[w][e], pb[w][e]));
                        o[e] = (v + e > hc) ? make_float2(0.f, 0.f) : y;
                        if (sel) o[e].y = -o[e].y;
                    }
                    const int row = sel ? u2 : u;
                    const int drow = row < a.map_split ? row - a.map_lo : row - a.map_hi;
                    float4* dst = reinterpret_cast<float4*>(a.out + (size_t)drow * a.out_pitch + v);
                    __stcs(dst, make_float4(o[0].x, o[0].y, o[1].x, o[1].y));
                }
            }
        } else
        for (int s0 = lo + tid; s0 < hi; s0 += WS * nt) {
            int cc[WS][2], nn[WS][2];
            float2 acc[WS][2];
#pragma unroll
            for (int w = 0; w < WS; w++) {
                const int s = s0 + w * nt;
                const int sel = s >= half_slots;
                const int v = 2 * (s - sel * half_slots);
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int vv = v + e;
                    const int c = (s >= hi || vv > hc) ? -1 : sel ? (vv == 0 ? 0 : cols - vv) : vv;
                    int n = c < 0 ? 0 : c;
                    while (n >= Lp) n -= Lp;  // cols <= (K/2 + 1) * Lp: a few steps at most
                    cc[w][e] = c < 0 ? 0 : c;
                    nn[w][e] = n;
                    acc[w][e] = make_float2(0.f, 0.f);
                }
            }
            for (int qq = 0; qq < K; qq++) {
                const float2* pq = a.post + (size_t)qq * cols;
                const float2* zq = zs0 + (size_t)qq * Lp;
                const bool last = qq == K - 1;
                float2 pv[WS][2], zv[WS][2];
#pragma unroll
                for (int w = 0; w < WS; w++)
#pragma unroll
                    for (int e = 0; e < 2; e++) {
                        pv[w][e] = __ldg(pq + cc[w][e]);
                        zv[w][e] = last ? buf[nn[w][e]] : __ldcg(zq + nn[w][e]);
                    }
#pragma unroll
                for (int w = 0; w < WS; w++)
#pragma unroll
                    for (int e = 0; e < 2; e++) acc[w][e] = cadd(acc[w][e], cmul(zv[w][e], pv[w][e]));
            }
#pragma unroll
            for (int w = 0; w < WS; w++) {
                const int s = s0 + w * nt;
                if (s >= hi) break;
                const int sel = s >= half_slots;
                const int v = 2 * (s - sel * half_slots);
                float2 o0 = (v > hc) ? make_float2(0.f, 0.f) : acc[w][0];
                float2 o1 = (v + 1 > hc) ? make_float2(0.f, 0.f) : acc[w][1];
                if (sel) {
                    o0.y = -o0.y;
                    o1.y = -o1.y;
                }
                const int row = sel ? u2 : u;
                const int drow = row < a.map_split ? row - a.map_lo : row - a.map_hi;
                float4* dst = reinterpret_cast<float4*>(a.out + (size_t)drow * a.out_pitch + v);
                __stcs(dst, make_float4(o0.x, o0.y, o1.x, o1.y));
            }
        }
    } else {
        // clusters: the K channels sit in the shared memories of the cluster
        for (int s = lo + tid; s < hi; s += nt) {
            const int sel = s >= half_slots;
            const int v = 2 * (s - sel * half_slots);
            float2 o[2];
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int vv = v + e;
                float2 val = make_float2(0.f, 0.f);
                if (vv <= hc) {
                    const int c = sel ? (vv == 0 ? 0 : cols - vv) : vv;
                    int n = c;
                    while (n >= Lp) n -= Lp;
                    for (int qq = 0; qq < K; qq++)
                        val = cadd(val, cmul(zsrc[qq][n], __ldg(a.post + (size_t)qq * cols + c)));
                    if (sel) val.y = -val.y;
                }
                o[e] = val;
            }
            const int row = sel ? u2 : u;
            const int drow = row < a.map_split ? row - a.map_lo : row - a.map_hi;
            float4* dst = reinterpret_cast<float4*>(a.out + (size_t)drow * a.out_pitch + v);
            __stcs(dst, make_float4(o[0].x, o[0].y, o[1].x, o[1].y));
        }
    }
    if (CLUSTER) cg::this_cluster().sync();
    else __syncthreads();
}

// MODE: ROW_SINGLE, ROW_DIRECT, ROW_CLUSTER (launched with a K-CTA cluster
// dimension), ROW_SEQ or ROW_SEQW; single-channel plans use the ROW_SINGLE
// (or ROW_DIRECT) instance, which carries no multi-channel code.
template <int NTMAX, int MODE>
__global__ void __launch_bounds__(NTMAX, 1) k_bluestein_rows(RowsArgs a, FFTDesc fd, int* err) {
    extern __shared__ float4 smem_raw[];
    __shared__ uint64_t in_bar;
    float2* buf = reinterpret_cast<float2*>(smem_raw);
    // only a direct row can have odd Lp = cols below its even bulk-copy length
    // (a Bluestein row has Lp >= 2 cols - 1 and the multi-channel loads skip
    // the bulk copy when the row does not fit)
    float2* twr = buf + (MODE == ROW_DIRECT ? row_buf_len(fd.Lp) : fd.Lp);
    for (int i = threadIdx.x; i < fd.rest_len; i += blockDim.x) twr[i] = a.fft_tw[fd.rest_base + i];
    if (threadIdx.x == 0) mbar_init(&in_bar, 1);

    constexpr int MAXR = (NTMAX > 512) ? MAX_RADIX_NT1024 : MAX_RADIX_NT512;
    int q = 0, cid = blockIdx.x, ncl = gridDim.x;
    // the channels' shared-memory buffers across a cluster (ROW_CLUSTER);
    // the other modes read their channels from buf and the scratch directly
    const float2* zsrc[MODE == ROW_CLUSTER ? MAX_CHANNELS : 1];
    if constexpr (MODE == ROW_CLUSTER) {
        const int K = a.K;
        cg::cluster_group cl = cg::this_cluster();
        q = (int)cl.block_rank();
        cid = blockIdx.x / K;
        ncl = gridDim.x / K;
#pragma unroll
        for (int i = 0; i < MAX_CHANNELS; i++)
            zsrc[i] = (i < K) ? cl.map_shared_rank(buf, i) : buf;
    } else {
        zsrc[0] = buf;
    }
    uint32_t parity = 0;
    int err_bits = 0;
    __syncthreads();
    for (int t = cid; t < a.tile_rows; t += ncl)
        bluestein_row<MAXR, MODE>(a, fd, t, q, buf, twr, zsrc, &in_bar, parity, err_bits);
    if (err_bits) atomicOr(err, err_bits);
    if (err_bits & ERR_TIMEOUT) {
        // a copy that never signalled may still be in flight: wait once more
        // (bounded) before the shared memory is released
        mbar_wait_bounded(&in_bar, parity ^ 1u);
    }
}

// Batched rows: the Bluestein rows of many single-channel matrices
// (row_begin: first row of each matrix in the queue, row_begin[nmat] =
// total) handed out one at a time by a device work queue.  A CTA enters the
// matrices in order and reloads the matrix's descriptor and stage twiddles
// only when it moves to the next one.  Shared memory holds the largest
// matrix's row buffer plus its stage twiddles (the twiddles of each matrix
// sit right after its own row buffer).  *queue must be 0 at launch.
struct RowsBatch {
    RowsArgs a;
    FFTDesc fd;
};

template <int NTMAX>
__global__ void __launch_bounds__(NTMAX, 1)
k_bluestein_rows_batch(const RowsBatch* __restrict__ descs, const long* __restrict__ row_begin, int nmat,
                       unsigned long long* queue, int* err) {
    extern __shared__ float4 smem_raw[];
    __shared__ uint64_t in_bar;
    __shared__ RowsBatch cur;
    __shared__ long s_t;
    __shared__ int s_m;
    constexpr int MAXR = (NTMAX > 512) ? MAX_RADIX_NT1024 : MAX_RADIX_NT512;
    float2* buf = reinterpret_cast<float2*>(smem_raw);
    float2* twr = buf;
    if (threadIdx.x == 0) {
        mbar_init(&in_bar, 1);
        s_m = 0;
    }
    const float2* zsrc[1] = {buf};
    uint32_t parity = 0;
    int err_bits = 0;
    int loaded = -1;
    const long total = row_begin[nmat];
    __syncthreads();
    for (;;) {
        if (threadIdx.x == 0) {
            const long t = (long)atomicAdd(queue, 1ull);
            int m = s_m;
            while (m < nmat && row_begin[m + 1] <= t) m++;
            s_t = t;
            s_m = m;
        }
        __syncthreads();
        const long t = s_t;
        const int m = s_m;
        if (t >= total) break;
        if (m != loaded) {
            if (threadIdx.x == 0) cur = descs[m];
            __syncthreads();
            twr = buf + row_buf_len(cur.fd.Lp);
            for (int i = threadIdx.x; i < cur.fd.rest_len; i += blockDim.x)
                twr[i] = cur.a.fft_tw[cur.fd.rest_base + i];
            __syncthreads();
            loaded = m;
        }
        bluestein_row<MAXR, ROW_SINGLE, 2>(cur.a, cur.fd, (int)(t - row_begin[m]), 0, buf, twr, zsrc, &in_bar, parity,
                            err_bits);
    }
    if (err_bits) atomicOr(err, err_bits);
    if (err_bits & ERR_TIMEOUT) mbar_wait_bounded(&in_bar, parity ^ 1u);
}

}  // namespace gbsp
