// gbsp_kernels.cuh -- the device side of the binary-sparse 2-D R2C FFT.
//
//   k_table_*            one-time plan tables, FP64 on the GPU, rounded to FP32
//   k_twiddle_sum        pass 1: S[u][j] = sum_{r in column j} W_rows^{u*r}
//   k_bluestein_rows     pre-chirp + FFT + filter + inverse FFT + post-chirp and
//                        the Hermitian-paired R2C row writer, one row per CTA
//                        (or per thread-block cluster when the convolution is
//                        longer than one CTA's shared memory)
#pragma once
#include <cooperative_groups.h>
#include "gbsp_fft.cuh"

namespace cg = cooperative_groups;

namespace gbsp {

constexpr int MAX_STAGES = 16;
constexpr int MAX_CHANNELS = 8;
constexpr int ROWS_THREADS = 1024;  // k_bluestein_rows block size
constexpr int PASS1_KU = 4;         // Bluestein rows per lane in k_twiddle_sum
constexpr int PASS1_UBLK = 32 * PASS1_KU;

struct FFTDesc {
    int Lp;
    int nst;
    int R[MAX_STAGES];
    int m[MAX_STAGES];
    uint32_t magic[MAX_STAGES];
    int twoff[MAX_STAGES];
};

// ---------------------------------------------------------------------------
// Exact integer phase helpers
// ---------------------------------------------------------------------------

// x mod n for x < n^2 (so the true quotient is < n <= 65536): a float
// estimate of the quotient is off by at most one, corrected both ways.
__device__ __forceinline__ uint32_t mod_small(uint32_t x, uint32_t n, float inv_n) {
    uint32_t q = __float2uint_rz(__uint2float_rz(x) * inv_n);
    int32_t r = (int32_t)(x - q * n);
    r += (r < 0) ? (int32_t)n : 0;
    r -= (r >= (int32_t)n) ? (int32_t)n : 0;
    return (uint32_t)r;
}

// ---------------------------------------------------------------------------
// Plan tables (FP64 -> FP32).  Every phase is reduced exactly in 64-bit
// integers before it becomes a double angle.
// ---------------------------------------------------------------------------

// tab[p] = exp(-2*pi*i*p/rows), p < ntab
__global__ void k_table_rows(float2* __restrict__ tab, int ntab, int rows) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= ntab) return;
    double s, c;
    sincospi(-2.0 * (double)p / (double)rows, &s, &c);
    tab[p] = make_float2((float)c, (float)s);
}

// pre[q][c]  = exp(-i*pi*c^2/cols) * W_L^{+c*q}   (chirp, channel pre-twiddle)
// post[q][c] = exp(-i*pi*c^2/cols) * W_L^{-c*q}   (chirp, channel recombination)
// with W_L = exp(-2*pi*i/L).  The chirp phase uses c^2 mod 2*cols exactly.
__global__ void k_table_chirp(float2* __restrict__ pre, float2* __restrict__ post,
                              int cols, int L, int K) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)K * cols) return;
    int q = (int)(idx / cols);
    int c = (int)(idx - (long)q * cols);
    long long c2 = ((long long)c * (long long)c) % (2LL * cols);
    long long cq = ((long long)c * (long long)q) % (long long)L;
    double a = -(double)c2 / (double)cols;          // chirp: angle = pi * a
    double b = -2.0 * (double)cq / (double)L;       // W_L^{cq}: angle = pi * b
    double s, co;
    sincospi(a + b, &s, &co);
    pre[idx] = make_float2((float)co, (float)s);
    sincospi(a - b, &s, &co);
    post[idx] = make_float2((float)co, (float)s);
}

// Stage twiddles tw[off + k*(R-1) + q-1] = W_{Lp}^{q*k*l}, l = Lp/(R*m).
__global__ void k_table_fft(float2* __restrict__ tw, int Lp, int R, int m, int off) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= m * (R - 1)) return;
    int k = idx / (R - 1);
    int q = idx - k * (R - 1) + 1;
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

// One forward DIF stage over K channels in global memory, FP64, twiddles
// evaluated on the fly.  Used once per plan for the filter spectrum.
template <int R>
__device__ __forceinline__ void dif_stage_f64_one(double2* __restrict__ x, int Lp, int m, int t) {
    int j = t / m, k = t - (t / m) * m;
    int base = j * R * m + k;
    long long l = Lp / (R * m);
    double2 a[R];
#pragma unroll
    for (int s = 0; s < R; s++) a[s] = x[base + s * m];
    SmallDFT<R, false, double2>::run(a);
#pragma unroll
    for (int q = 1; q < R; q++) {
        long long e = ((long long)q * k * l) % Lp;
        double sn, cs;
        sincospi(-2.0 * (double)e / (double)Lp, &sn, &cs);
        a[q] = cmul(a[q], make_double2(cs, sn));
    }
#pragma unroll
    for (int s = 0; s < R; s++) x[base + s * m] = a[s];
}

__global__ void k_dif_stage_f64(double2* __restrict__ data, int K, int Lp, int R, int m) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    int nb = Lp / R;
    if (idx >= (long)K * nb) return;
    int ch = (int)(idx / nb);
    int t = (int)(idx - (long)ch * nb);
    double2* x = data + (size_t)ch * Lp;
    switch (R) {
        case 2: dif_stage_f64_one<2>(x, Lp, m, t); break;
        case 3: dif_stage_f64_one<3>(x, Lp, m, t); break;
        case 4: dif_stage_f64_one<4>(x, Lp, m, t); break;
        case 5: dif_stage_f64_one<5>(x, Lp, m, t); break;
        case 7: dif_stage_f64_one<7>(x, Lp, m, t); break;
        case 8: dif_stage_f64_one<8>(x, Lp, m, t); break;
        default: break;
    }
}

// filt = (float)(spec * scale)
__global__ void k_table_filter_final(float2* __restrict__ filt, const double2* __restrict__ spec,
                                     long n, double scale) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    double2 v = spec[idx];
    filt[idx] = make_float2((float)(v.x * scale), (float)(v.y * scale));
}

// ---------------------------------------------------------------------------
// Pass 1: twiddle sums over each active column's nonzero rows.
//
// Work item = (block of PASS1_UBLK Bluestein rows, one active column) handled
// by one warp; lane l owns rows u = ubase + l + 32*i (i < KU).  Per nonzero r
// the lane computes its phase (u*r) mod rows once with exact integer
// arithmetic and then steps it by (32*r) mod rows, so only one modular
// multiply is spent per KU twiddles.  Twiddles come from a table staged in
// shared memory: the whole circle (TAB_HALF = false) or the half circle
// p <= rows/2 with W^{rows-p} = conj(W^p).  Columns with at least
// kahan_min nonzeros accumulate with Kahan-compensated FP32 additions.
//
// The reference evaluates __sincosf of a float angle per (u, nonzero) and
// does one output row per thread (src/sparse_fft_bluestein.cu:366-397).
// ---------------------------------------------------------------------------
template <bool TAB_HALF>
__device__ __forceinline__ float2 row_twiddle(const float2* tab, uint32_t p, uint32_t rows, uint32_t hr) {
    if (!TAB_HALF) return tab[p];
    bool hi = p > hr;
    float2 w = tab[hi ? rows - p : p];
    w.y = hi ? -w.y : w.y;
    return w;
}

// (u*r) mod rows; BIG handles rows > 65536 where u*r no longer fits 32 bits.
template <bool BIG>
__device__ __forceinline__ uint32_t mulmod_rows(uint32_t u, uint32_t r, uint32_t rows, float inv_rows) {
    if (BIG) return (uint32_t)(((uint64_t)u * (uint64_t)r) % (uint64_t)rows);
    return mod_small(u * r, rows, inv_rows);
}

template <typename IDX, bool TAB_HALF, bool KAHAN, bool BIG>
__device__ __forceinline__ void column_sum_loop(const IDX* __restrict__ row_idx, int beg, int end,
                                                const float2* tab, uint32_t u_lane, uint32_t rows,
                                                float inv_rows, int lane, float (&ax)[PASS1_KU],
                                                float (&ay)[PASS1_KU]) {
    float cx[PASS1_KU], cy[PASS1_KU];
#pragma unroll
    for (int i = 0; i < PASS1_KU; i++) { cx[i] = 0.f; cy[i] = 0.f; }
    const uint32_t hr = rows / 2;
    for (int p0 = beg; p0 < end; p0 += 32) {
        int cnt = min(32, end - p0);
        uint32_t rl = 0, dl = 0;
        if (lane < cnt) {
            rl = (uint32_t)row_idx[p0 + lane];
            dl = mulmod_rows<BIG>(32u, rl, rows, inv_rows);
        }
        for (int i = 0; i < cnt; i++) {
            uint32_t r = __shfl_sync(0xffffffffu, rl, i);
            uint32_t d = __shfl_sync(0xffffffffu, dl, i);
            uint32_t p = mulmod_rows<BIG>(u_lane, r, rows, inv_rows);
#pragma unroll
            for (int kk = 0; kk < PASS1_KU; kk++) {
                float2 w = row_twiddle<TAB_HALF>(tab, p, rows, hr);
                if (KAHAN) {
                    float y = w.x - cx[kk];
                    float t = ax[kk] + y;
                    cx[kk] = (t - ax[kk]) - y;
                    ax[kk] = t;
                    y = w.y - cy[kk];
                    t = ay[kk] + y;
                    cy[kk] = (t - ay[kk]) - y;
                    ay[kk] = t;
                } else {
                    ax[kk] += w.x;
                    ay[kk] += w.y;
                }
                uint32_t pn = p + d;
                p = min(pn, pn - rows);
            }
        }
    }
}

template <typename IDX, bool TAB_HALF, bool BIG>
__global__ void __launch_bounds__(512)
k_twiddle_sum(const int* __restrict__ col_ptr, const IDX* __restrict__ row_idx, int n_active,
              const float2* __restrict__ row_tab, int ntab, int rows, float inv_rows,
              int u0, int tile_rows, float2* __restrict__ S, size_t s_pitch, int kahan_min) {
    extern __shared__ float4 smem_raw[];
    float2* tab = reinterpret_cast<float2*>(smem_raw);
    for (int i = threadIdx.x; i < ntab; i += blockDim.x) tab[i] = row_tab[i];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const long gw = (long)blockIdx.x * wpb + (threadIdx.x >> 5);
    const long nw = (long)gridDim.x * wpb;
    const int n_ublk = (tile_rows + PASS1_UBLK - 1) / PASS1_UBLK;
    const long nitems = (long)n_ublk * n_active;

    for (long it = gw; it < nitems; it += nw) {
        const int ub = (int)(it / n_active);
        const int j = (int)(it - (long)ub * n_active);
        const int ul0 = ub * PASS1_UBLK;
        uint32_t u_lane = (uint32_t)(u0 + ul0 + lane) % (uint32_t)rows;
        const int beg = col_ptr[j], end = col_ptr[j + 1];
        float ax[PASS1_KU], ay[PASS1_KU];
#pragma unroll
        for (int i = 0; i < PASS1_KU; i++) { ax[i] = 0.f; ay[i] = 0.f; }
        if (kahan_min > 0 && end - beg >= kahan_min)
            column_sum_loop<IDX, TAB_HALF, true, BIG>(row_idx, beg, end, tab, u_lane, (uint32_t)rows,
                                                 inv_rows, lane, ax, ay);
        else
            column_sum_loop<IDX, TAB_HALF, false, BIG>(row_idx, beg, end, tab, u_lane, (uint32_t)rows,
                                                  inv_rows, lane, ax, ay);
#pragma unroll
        for (int kk = 0; kk < PASS1_KU; kk++) {
            int ul = ul0 + lane + 32 * kk;
            if (ul < tile_rows) S[(size_t)ul * s_pitch + j] = make_float2(ax[kk], ay[kk]);
        }
    }
}

// ---------------------------------------------------------------------------
// Bluestein rows.  Channel q of K (the CTA's rank in its cluster) holds
//   y_q[n] = sum_{c = n mod Lp} pre[q][c] * S[u][c]          (n < Lp)
// runs the forward DIF FFT of length Lp, multiplies by the channel's filter
// spectrum (digit-reversed, scaled by 1/L), and runs the inverse DIT FFT,
// leaving Z_q[n] in natural order.  The length-L convolution result is then
//   y[c] = sum_q post[q][c] * Z_q[c mod Lp]
// read across the cluster's shared memories (DSMEM).  Since the 2-D input is
// real, F[rows-u][v] = conj(F[u][(cols-v) mod cols]), so one Bluestein row u
// (u <= rows/2) writes output rows u and rows-u, each with 16-byte stores of
// two complex values.
//
// The reference runs 2F+4 launches per tile of rows with a global round trip
// per stage (src/sparse_fft_bluestein.cu:2327-2370) and writes 8-byte stores
// in bluestein_finalize_kernel (:469-486).
// ---------------------------------------------------------------------------
template <bool CLUSTER>
__global__ void __launch_bounds__(ROWS_THREADS, 1)
k_bluestein_rows(const float2* __restrict__ S, size_t s_pitch, int n_active,
                 const int* __restrict__ sparse_cols, const float2* __restrict__ pre,
                 const float2* __restrict__ post, const float2* __restrict__ filt,
                 const float2* __restrict__ fft_tw, FFTDesc fd, int K, int rows, int cols,
                 int u0, int tile_rows, float2* __restrict__ out, size_t out_pitch) {
    extern __shared__ float4 smem_raw[];
    float2* buf = reinterpret_cast<float2*>(smem_raw);
    const int Lp = fd.Lp;
    const int tid = threadIdx.x, nt = blockDim.x;

    int q = 0, cid = blockIdx.x, ncl = gridDim.x;
    const float2* zsrc[MAX_CHANNELS];
    if (CLUSTER) {
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
    const float2* preq = pre + (size_t)q * cols;
    const float2* filtq = filt + (size_t)q * Lp;
    const int half_slots = (int)(out_pitch >> 1);
    const int hc = cols / 2;
    const bool wrap_in = cols > Lp;

    for (int t = cid; t < tile_rows; t += ncl) {
        const int u = u0 + t;
        for (int i = tid; i < Lp; i += nt) buf[i] = make_float2(0.f, 0.f);
        __syncthreads();
        const float2* srow = S + (size_t)t * s_pitch;
        if (!wrap_in) {
            for (int j = tid; j < n_active; j += nt) {
                int c = sparse_cols[j];
                buf[c] = cmul(srow[j], preq[c]);
            }
            __syncthreads();
        } else {
            // several input columns fold onto one slot: add section by section
            for (int sec = 0; sec * Lp < cols; sec++) {
                const int lo = sec * Lp, hi = lo + Lp;
                for (int j = tid; j < n_active; j += nt) {
                    int c = sparse_cols[j];
                    if (c >= lo && c < hi) buf[c - lo] = cadd(buf[c - lo], cmul(srow[j], preq[c]));
                }
                __syncthreads();
            }
        }
        // forward DIF, filter multiply fused with the last stage, inverse DIT
        const int S1 = fd.nst - 1;
        for (int s = 0; s < S1; s++) {
            fft_stage_dispatch<0>(fd.R[s], buf, Lp, fd.m[s], fd.magic[s], fft_tw + fd.twoff[s],
                                  (const float2*)nullptr, tid, nt);
            __syncthreads();
        }
        fft_stage_dispatch<2>(fd.R[S1], buf, Lp, fd.m[S1], fd.magic[S1], fft_tw + fd.twoff[S1],
                              filtq, tid, nt);
        __syncthreads();
        for (int s = S1 - 1; s >= 0; s--) {
            fft_stage_dispatch<1>(fd.R[s], buf, Lp, fd.m[s], fd.magic[s], fft_tw + fd.twoff[s],
                                  (const float2*)nullptr, tid, nt);
            __syncthreads();
        }
        if (CLUSTER) cg::this_cluster().sync();

        // Hermitian-paired row writer
        const int u2 = (u == 0) ? 0 : rows - u;
        const bool two = (u2 != u);
        const int nslots = two ? 2 * half_slots : half_slots;
        const int lo = (int)((long)q * nslots / K), hi = (int)((long)(q + 1) * nslots / K);
        for (int s = lo + tid; s < hi; s += nt) {
            const int sel = s >= half_slots;
            const int v = 2 * (s - sel * half_slots);
            float2 o[2];
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int vv = v + e;
                float2 val = make_float2(0.f, 0.f);
                if (vv <= hc) {
                    int c = sel ? (vv == 0 ? 0 : cols - vv) : vv;
                    int n = c;
                    while (n >= Lp) n -= Lp;
                    if (CLUSTER) {
                        for (int qq = 0; qq < K; qq++)
                            val = cadd(val, cmul(zsrc[qq][n], post[(size_t)qq * cols + c]));
                    } else {
                        val = cmul(buf[n], post[c]);
                    }
                    if (sel) val.y = -val.y;
                }
                o[e] = val;
            }
            const int row = sel ? u2 : u;
            float4* dst = reinterpret_cast<float4*>(out + (size_t)row * out_pitch + v);
            *dst = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
        }
        if (CLUSTER) cg::this_cluster().sync();
        else __syncthreads();
    }
}

}  // namespace gbsp
