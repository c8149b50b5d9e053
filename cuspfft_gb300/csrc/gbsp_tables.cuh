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
