// gbsp_tables.cuh -- one-time plan tables, FP64 on the GPU, rounded to FP32
// (row twiddles, channel pre/post twiddles, stage twiddles, the filter
// spectrum).  Non-template kernels: included by one translation unit only.
#pragma once
#include "gbsp_kernels.cuh"

namespace gbsp {

// ---------------------------------------------------------------------------
// Plan tables (FP64 -> FP32).  Every phase is reduced exactly in 64-bit
// integers before it becomes a double angle.
// ---------------------------------------------------------------------------

// Row indices arrive as int32 in column order.  Each is checked against
// [0, rows) -- any index outside sets *bad, and the plan is not built, so no
// kernel ever reads a table with it -- and, when dst16 is given, stored as
// u16.  Grid-stride; every thread reaches the warp vote.
__global__ void k_row_index_in(const int* __restrict__ src, uint16_t* __restrict__ dst16, long nnz, int rows,
                               int* bad) {
    int b = 0;
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nnz; i += stride) {
        const int r = src[i];
        b |= (unsigned)r >= (unsigned)rows;
        if (dst16) dst16[i] = (uint16_t)r;
    }
    if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}

// Column c's first nonzero and degree from the compact CSC (deg[] zeroed
// beforehand: columns without nonzeros stay 0).
__global__ void k_column_spans(const int* __restrict__ col_ptr, const int* __restrict__ sparse_cols, int n_active,
                               int* __restrict__ col_begin, int* __restrict__ deg) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_active) return;
    const int c = sparse_cols[j];
    col_begin[c] = col_ptr[j];
    deg[c] = col_ptr[j + 1] - col_ptr[j];
}

// Pass-1 task tables, one warp per window of cw (32 or 64) columns.  With
// T = max(32, ceil(window nonzeros / P1_WARPS)), column lc splits into
// np = ceil(deg / T) tasks at nonzero offsets floor(k * deg / np); the tasks
// take tile columns (slots) in column order, slot0[lc] being column lc's
// first (slot0[cw] = the window's task count), and are listed longest first,
// ties in slot order.  np sums to < window nonzeros / T + cw <= cw + P1_WARPS,
// so the vmax-long list cannot overflow (a violation would set *bad, bit 1).
constexpr int TASK_WARPS = 4;
__global__ void __launch_bounds__(TASK_WARPS * 32)
k_p1_tasks(const int* __restrict__ col_begin, const int* __restrict__ deg, int cols, int cw, int n_win,
           uint8_t* __restrict__ slot0, int2* __restrict__ task, uint8_t* __restrict__ task_col, int* bad) {
    __shared__ int2 s_task[TASK_WARPS][64 + P1_WARPS];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * TASK_WARPS + wl;
    if (w >= n_win) return;  // warp-uniform
    const int vmax = p1_vmax(cw);
    const int halves = cw / 32;  // columns lane and lane + 32
    int d[2] = {0, 0};
    for (int h = 0; h < halves; h++) {
        const int c = w * cw + h * 32 + lane;
        d[h] = c < cols ? deg[c] : 0;
    }
    int sum = d[0] + d[1];
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    const int T = max(32, (sum + P1_WARPS - 1) / P1_WARPS);
    int first[2] = {0, 0}, np[2] = {0, 0};
    int base = 0;
    for (int h = 0; h < halves; h++) {
        np[h] = (d[h] + T - 1) / T;
        int incl = np[h];
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        first[h] = base + incl - np[h];
        base += __shfl_sync(0xffffffffu, incl, 31);
    }
    const int nt = base;
    uint8_t* s0 = slot0 + (size_t)w * (cw + 1);
    for (int h = 0; h < halves; h++) s0[h * 32 + lane] = (uint8_t)min(first[h], vmax);
    if (lane == 0) s0[cw] = (uint8_t)min(nt, vmax);
    if (nt > vmax) {
        if (lane == 0) atomicOr(bad, 2);
        return;
    }
    for (int h = 0; h < halves; h++) {
        const int c = w * cw + h * 32 + lane;
        if (np[h] == 0) continue;
        const int b0 = col_begin[c];
        for (int k = 0; k < np[h]; k++)
            s_task[wl][first[h] + k] = make_int2(b0 + (int)((long long)k * d[h] / np[h]),
                                                 b0 + (int)((long long)(k + 1) * d[h] / np[h]));
    }
    __syncwarp();
    int2* tw = task + (size_t)w * vmax;
    uint8_t* tc = task_col + (size_t)w * vmax;
    for (int i = lane; i < vmax; i += 32) {
        if (i >= nt) {
            tw[i] = make_int2(0, 0);
            tc[i] = 0;
        }
    }
    for (int i = lane; i < nt; i += 32) {
        const int2 t = s_task[wl][i];
        const int len = t.y - t.x;
        int rank = 0;
        for (int j = 0; j < nt; j++) {
            const int lj = s_task[wl][j].y - s_task[wl][j].x;
            rank += (lj > len) || (lj == len && j < i);
        }
        tw[rank] = t;
        tc[rank] = (uint8_t)i;
    }
}

// tab[p] = exp(-2*pi*i*p/rows), p < ntab
// two_level: entries TWO_LO.. hold W^(TWO_LO*j) (layout of TAB_TWO)
__global__ void k_table_rows(float2* __restrict__ tab, int ntab, int rows, int two_level) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntab) return;
    const long long p = (two_level && i >= TWO_LO) ? (long long)(i - TWO_LO) * TWO_LO % rows : i;
    double s, c;
    sincospi(-2.0 * (double)p / (double)rows, &s, &c);
    tab[i] = make_float2((float)c, (float)s);
}

// Chirp exp(-i*pi*c^2/cols) times W_L^{+c*q} (sign = +1) or W_L^{-c*q} (sign = -1),
// W_L = exp(-2*pi*i/L); c^2 mod 2*cols and c*q mod L are reduced exactly.
__device__ __forceinline__ float2 chirp_twiddle(long long c, int q, int cols, int L, int sign) {
    long long c2 = (c * c) % (2LL * cols);
    long long cq = (c * (long long)q) % (long long)L;
    double a = -(double)c2 / (double)cols - sign * 2.0 * (double)cq / (double)L;
    double s, co;
    sincospi(a, &s, &co);
    return make_float2((float)co, (float)s);
}

// pre[q][c] = W_L^{+c*q}  (channel pre-twiddle; the chirp is applied by pass 1)
__global__ void k_table_pre(float2* __restrict__ pre, int cols, int L, int K) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)K * cols) return;
    int q = (int)(idx / cols);
    long long c = idx - (long)q * cols;
    long long cq = (c * (long long)q) % (long long)L;
    double s, co;
    sincospi(-2.0 * (double)cq / (double)L, &s, &co);
    pre[idx] = make_float2((float)co, (float)s);
}

// post[q][c] = chirp(c) * W_L^{-c*q}  (column order)
__global__ void k_table_post(float2* __restrict__ post, int cols, int L, int K) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)K * cols) return;
    int q = (int)(idx / cols);
    int c = (int)(idx - (long)q * cols);
    post[idx] = chirp_twiddle(c, q, cols, L, -1);
}

// Stage twiddles, q-major: tw[off + (q-1)*m + k] = W_{Lp}^{q*k*l}, l = Lp/(R*m).
__global__ void k_table_fft(float2* __restrict__ tw, int Lp, int R, int m, int off) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= m * (R - 1)) return;
    int q = idx / m + 1;
    int k = idx - (q - 1) * m;
    long long l = Lp / (R * m);
    long long e = ((long long)q * k * l) % Lp;
    double s, c;
    sincospi(-2.0 * (double)e / (double)Lp, &s, &c);
    tw[off + idx] = make_float2((float)c, (float)s);
}

// Channel-q filter input: bq[q][n] = sum_{c = n mod Lp, c < L} b[c] * W_L^{c*q}
// where b[c] = exp(+i*pi*c^2/cols) for c < cols, b[L-c] = b[c] for 0 < c < cols.
// (reference: make_bluestein_b, include/sparse_fft_internal.cuh:179-191)
__global__ void k_table_filter_input(double2* __restrict__ bq, int cols, int L, int K, int Lp) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)K * Lp) return;
    int q = (int)(idx / Lp);
    int n = (int)(idx - (long)q * Lp);
    double ax = 0.0, ay = 0.0;
    for (int s = 0; s < K; s++) {
        long long c = (long long)s * Lp + n;
        long long k;
        if (c < cols) k = c;
        else if (c > 0 && L - c < cols) k = L - c;
        else continue;
        long long k2 = (k * k) % (2LL * cols);
        long long cq = (c * (long long)q) % (long long)L;
        double sn, cs;
        sincospi((double)k2 / (double)cols - 2.0 * (double)cq / (double)L, &sn, &cs);
        ax += cs;
        ay += sn;
    }
    bq[idx] = make_double2(ax, ay);
}

// One forward DIF stage (any radix R <= MAX_RADIX) over K channels in global
// memory, FP64, out of place: one thread per output element, which sums its
// butterfly's R inputs against the R-point roots by definition and applies
// the stage twiddle, every root evaluated from an exactly reduced integer
// phase.  Used once per plan for the filter spectrum, so it follows the row
// kernel's network.  (One thread per element keeps every SM busy: FP64 runs
// at a small fraction of the FP32 rate on this part.)
constexpr int MAX_RADIX = 64;
__global__ void k_dif_stage_f64(const double2* __restrict__ src, double2* __restrict__ dst, int K, int Lp, int R,
                                int m) {
    __shared__ double2 root[MAX_RADIX];  // W_R^e, e < R
    if (R > MAX_RADIX) return;
    for (int e = threadIdx.x; e < R; e += blockDim.x) {
        double sn, cs;
        sincospi(-2.0 * (double)e / (double)R, &sn, &cs);
        root[e] = make_double2(cs, sn);
    }
    __syncthreads();
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)K * Lp) return;
    const int ch = (int)(idx / Lp);
    const int pos = (int)(idx - (long)ch * Lp);  // = j*R*m + q*m + k
    const int span = R * m;
    const int j = pos / span, rem = pos - j * span, q = rem / m, k = rem - q * m;
    const double2* x = src + (size_t)ch * Lp + (size_t)j * span + k;
    double2 acc = make_double2(0.0, 0.0);
    for (int s = 0, e = 0; s < R; s++, e = (e + q) % R) acc = cadd(acc, cmul(x[(size_t)s * m], root[e]));
    const long long l = Lp / span;
    const long long ph = ((long long)q * k * l) % Lp;
    double sn, cs;
    sincospi(-2.0 * (double)ph / (double)Lp, &sn, &cs);
    dst[idx] = cmul(acc, make_double2(cs, sn));
}

// filt[ch][q*(Lp/R) + t] = (float)(spec[ch][t*R + q] * scale): the filter in the
// thread order of the fused last stage (radix R, span 1).
__global__ void k_table_filter_final(float2* __restrict__ filt, const double2* __restrict__ spec,
                                     int K, int Lp, int R, double scale) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)K * Lp) return;
    int ch = (int)(idx / Lp);
    int pos = (int)(idx - (long)ch * Lp);
    int t = pos / R, q = pos - (pos / R) * R;
    double2 v = spec[idx];
    filt[(size_t)ch * Lp + (size_t)q * (Lp / R) + t] = make_float2((float)(v.x * scale), (float)(v.y * scale));
}

}  // namespace gbsp
