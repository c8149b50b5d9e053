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

// The CSC half of a plan's build, one launch:
//
// Blocks [0, task_blocks): the pass-1 task tables, one warp per window of cw
// (16, 32 or 64) columns.  The window's active columns are found in sparse_cols
// (strictly increasing) by a binary search for its first column.  With
// T = max(32, ceil(window nonzeros / P1_WARPS)), column lc splits into
// np = ceil(deg / T) tasks at nonzero offsets floor(k * deg / np); the tasks
// take tile columns (slots) in column order, slot0[lc] being column lc's
// first (slot0[cw] = the window's task count), and are listed longest first,
// ties in slot order.  np sums to < window nonzeros / T + cw <= cw + P1_WARPS,
// so the vmax-long list cannot overflow (a violation would set *bad, bit 1).
//
// Blocks [task_blocks, gridDim.x): the row indices, int32 in column order,
// each checked against [0, rows) -- one outside sets *bad (bit 0) and the
// plan is not built, so no kernel ever reads a table with it -- and, when
// row16 is given, stored as u16.  Grid-stride; every thread of these blocks
// reaches the warp vote.
constexpr int SETUP_WARPS = 4;
struct CscSetupArgs {
    const int* col_ptr;      // n_active + 1
    const int* sparse_cols;  // n_active, strictly increasing
    int n_active, cols, cw, n_win, task_blocks;
    uint8_t* slot0;
    int2* task;
    uint8_t* task_col;
    const int* row_in;  // nnz int32
    uint16_t* row16;    // nullptr: 4-byte indices, checked in place
    long nnz;
    int rows;
    int* bad;
};
__global__ void __launch_bounds__(SETUP_WARPS * 32) k_csc_setup(CscSetupArgs a) {
    if ((int)blockIdx.x >= a.task_blocks) {
        int b = 0;
        const long stride = (long)(gridDim.x - a.task_blocks) * blockDim.x;
        for (long i = (long)(blockIdx.x - a.task_blocks) * blockDim.x + threadIdx.x; i < a.nnz; i += stride) {
            const int r = a.row_in[i];
            b |= (unsigned)r >= (unsigned)a.rows;
            if (a.row16) a.row16[i] = (uint16_t)r;
        }
        if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(a.bad, 1);
        return;
    }
    __shared__ int2 s_task[SETUP_WARPS][64 + P1_WARPS];
    __shared__ int s_deg[SETUP_WARPS][64], s_beg[SETUP_WARPS][64];
    const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * SETUP_WARPS + wl;
    if (w >= a.n_win) return;  // warp-uniform
    const int cw = a.cw, vmax = p1_vmax(cw);
    const int halves = (cw + 31) / 32;  // columns lane and lane + 32; lanes >= cw idle when cw = 16
    const int c0 = w * cw;
    // first active column >= c0
    int lo = 0, hi = a.n_active;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a.sparse_cols[mid] < c0) lo = mid + 1;
        else hi = mid;
    }
    for (int h = 0; h < halves; h++) s_deg[wl][h * 32 + lane] = 0;
    __syncwarp();
    for (int h = 0; h < halves; h++) {
        const int j = lo + h * 32 + lane;
        if (j < a.n_active) {
            const int c = a.sparse_cols[j];
            if (c < c0 + cw) {
                s_deg[wl][c - c0] = a.col_ptr[j + 1] - a.col_ptr[j];
                s_beg[wl][c - c0] = a.col_ptr[j];
            }
        }
    }
    __syncwarp();
    int d[2] = {0, 0};
    for (int h = 0; h < halves; h++) d[h] = s_deg[wl][h * 32 + lane];
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
    uint8_t* s0 = a.slot0 + (size_t)w * (cw + 1);
    for (int h = 0; h < halves; h++)
        if (h * 32 + lane < cw) s0[h * 32 + lane] = (uint8_t)min(first[h], vmax);
    if (lane == 0) s0[cw] = (uint8_t)min(nt, vmax);
    if (nt > vmax) {
        if (lane == 0) atomicOr(a.bad, 2);
        return;
    }
    for (int h = 0; h < halves; h++) {
        if (np[h] == 0) continue;
        const int b0 = s_beg[wl][h * 32 + lane];
        for (int k = 0; k < np[h]; k++)
            s_task[wl][first[h] + k] = make_int2(b0 + (int)((long long)k * d[h] / np[h]),
                                                 b0 + (int)((long long)(k + 1) * d[h] / np[h]));
    }
    __syncwarp();
    int2* tw = a.task + (size_t)w * vmax;
    uint8_t* tc = a.task_col + (size_t)w * vmax;
    for (int i = nt + lane; i < vmax; i += 32) {
        tw[i] = make_int2(0, 0);
        tc[i] = 0;
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

// Direct plans: drev[f] = position of frequency f after the forward DIF
// network, sum over stages s of digit_s(f) * m_s, where digit_s(f) =
// (f / (R_0 ... R_{s-1})) mod R_s (the stage-s output q lands at q * m_s).
__global__ void k_digit_rev(int* drev, FFTDesc fd) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= fd.Lp) return;
    int t = f, pos = 0;
    for (int s = 0; s < fd.nst; s++) {
        pos += (t % fd.R[s]) * fd.m[s];
        t /= fd.R[s];
    }
    drev[f] = pos;
}

// exp(-2*pi*i*e/n) for an exactly reduced integer phase e < n
__device__ __forceinline__ float2 root_f32(long long e, long long n) {
    double s, c;
    sincospi(-2.0 * (double)e / (double)n, &s, &c);
    return make_float2((float)c, (float)s);
}

// The single-precision plan tables in one launch, one entry per thread over
// the concatenated index ranges
//   rowtab[p] = W_rows^p, p < ntab (two_level: entries TWO_LO.. hold
//              W_rows^(TWO_LO*j), the layout of TAB_TWO)
//   pre[q][c] = W_L^{+c*q}              (channel pre-twiddle)
//   post[q][c] = chirp(c) * W_L^{-c*q}  (column order)
//   fftw: stage s's twiddles, q-major, tw[twoff[s] + (q-1)*m + k] =
//         W_Lp^{q*k*l}, l = Lp/(R*m)
struct TableArgs {
    float2* rowtab;
    float2* pre;
    float2* post;
    float2* fftw;
    int ntab, rows, two_level, cols, L, K;
    FFTDesc fd;
};
__global__ void k_tables(TableArgs a) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.ntab) {
        const long long p = (a.two_level && i >= TWO_LO) ? (long long)(i - TWO_LO) * TWO_LO % a.rows : i;
        a.rowtab[i] = root_f32(p, a.rows);
        return;
    }
    i -= a.ntab;
    const long kc = (long)a.K * a.cols;
    if (i < 2 * kc) {
        const bool post = i >= kc;
        const long idx = post ? i - kc : i;
        const int q = (int)(idx / a.cols);
        const long long c = idx - (long)q * a.cols;
        if (post)
            a.post[idx] = chirp_twiddle(c, q, a.cols, a.L, -1);
        else
            a.pre[idx] = root_f32((c * (long long)q) % (long long)a.L, a.L);
        return;
    }
    i -= 2 * kc;
    for (int s = 0; s < a.fd.nst; s++) {
        const int R = a.fd.R[s], m = a.fd.m[s];
        const long n = (long)(R - 1) * m;
        if (i < n) {
            const int q = (int)(i / m) + 1;
            const int k = (int)(i - (long)(q - 1) * m);
            const long long l = a.fd.Lp / (R * m);
            a.fftw[a.fd.twoff[s] + i] = root_f32(((long long)q * k * l) % a.fd.Lp, a.fd.Lp);
            return;
        }
        i -= n;
    }
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
    // inputs in groups of 8 loads issued together (R is a runtime value: a
    // load-multiply chain would pay the L2 latency R times); sum order s = 0..R-1
    double2 acc = make_double2(0.0, 0.0);
    int e = 0;
    for (int s0 = 0; s0 < R; s0 += 8) {
        double2 xv[8];
#pragma unroll
        for (int i = 0; i < 8; i++) xv[i] = (s0 + i < R) ? x[(size_t)(s0 + i) * m] : make_double2(0.0, 0.0);
#pragma unroll
        for (int i = 0; i < 8; i++) {
            if (s0 + i < R) {
                acc = cadd(acc, cmul(xv[i], root[e]));
                e += q;
                if (e >= R) e -= R;
            }
        }
    }
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
