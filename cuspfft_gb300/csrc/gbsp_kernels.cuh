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
constexpr int P1_THREADS = 512;     // k_twiddle_sum block size
constexpr int P1_WARPS = P1_THREADS / 32;
constexpr int P1_KU = 8;            // Bluestein rows per lane in k_twiddle_sum
constexpr int P1_UBLK = 32 * P1_KU; // Bluestein rows per work item
constexpr int P1_RESEED = 4;        // exact table lookup every P1_RESEED rows
constexpr int P1_STAGE_PITCH = P1_WARPS + 1;
constexpr size_t P1_STAGE_BYTES = (size_t)P1_UBLK * P1_STAGE_PITCH * 8;

struct FFTDesc {
    int Lp;                     // channel FFT length
    int nst;                    // stages
    int R[MAX_STAGES];          // radix per stage
    int m[MAX_STAGES];          // span per stage
    uint32_t magic[MAX_STAGES]; // ceil(2^32 / m)
    int twoff[MAX_STAGES];      // stage twiddle offset in the global table (q-major blocks)
    int rest_base;              // first twiddle of stage 1 (stages >= 1 are staged in smem)
    int rest_len;               // twiddles of stages >= 1
};

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

// (u*r) mod rows; BIG handles rows > 65535 where u*r may not fit 32 bits.
template <bool BIG>
__device__ __forceinline__ uint32_t mulmod_rows(uint32_t u, uint32_t r, uint32_t rows, uint32_t magic) {
    if (BIG) return (uint32_t)(((uint64_t)u * (uint64_t)r) % (uint64_t)rows);
    return mod_magic(u * r, rows, magic);
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

// pre[q][j]  = chirp(c_j) * W_L^{+c_j*q}, c_j = slot_col[j]  (slot order)
__global__ void k_table_pre(float2* __restrict__ pre, const int* __restrict__ slot_col, int n_slots,
                            int cols, int L, int K) {
    long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)K * n_slots) return;
    int q = (int)(idx / n_slots);
    int j = (int)(idx - (long)q * n_slots);
    pre[idx] = chirp_twiddle(slot_col[j], q, cols, L, +1);
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

// ---------------------------------------------------------------------------
// Pass 1: twiddle sums over each active column's nonzero rows.
//
// Columns live in "slots" sorted by degree (descending), so the P1_WARPS
// columns of one work item have nearly equal nonzero counts.  A work item is
// (block of P1_UBLK Bluestein rows, group of P1_WARPS slots); warp w owns
// slot g*P1_WARPS + w and lane l owns rows u = ubase + l + 32*kk (kk < KU).
//
// Per nonzero r the lane reduces its phase (u*r) mod rows exactly with an
// integer multiply-high and reads W_rows^p from the table staged in shared
// memory.  The rows u + 32*kk in between reuse the exactly looked-up
// W_rows^{(32*r) mod rows} as a complex multiplier, and every P1_RESEED rows
// the value is looked up exactly again, so no twiddle is more than
// P1_RESEED-1 products away from a correctly rounded table entry.  Sums of a
// batch of 32 nonzeros are added to the column total; for columns with at
// least kahan_min nonzeros that addition is Kahan-compensated.  Results pass
// through a shared-memory tile so every S row segment is written as whole
// 128-byte lines.
//
// The reference evaluates __sincosf of a float angle per (u, nonzero), one
// output row per thread, and writes strided 8-byte values
// (src/sparse_fft_bluestein.cu:366-397).
// ---------------------------------------------------------------------------
template <bool TAB_HALF>
__device__ __forceinline__ float2 row_twiddle(const float2* tab, uint32_t p, uint32_t rows, uint32_t hr) {
    if (!TAB_HALF) return tab[p];
    bool hi = p > hr;
    float2 w = tab[hi ? rows - p : p];
    w.y = hi ? -w.y : w.y;
    return w;
}

template <typename IDX, bool TAB_HALF, bool BIG>
__device__ __forceinline__ void column_sums_warp(const IDX* __restrict__ row_idx, int beg, int end,
                                                 const float2* tab, uint32_t u_lane, uint32_t rows,
                                                 uint32_t magic, int lane, bool compensated,
                                                 float2 (&acc)[P1_KU]) {
    float2 cmp[P1_KU];
#pragma unroll
    for (int i = 0; i < P1_KU; i++) { acc[i] = make_float2(0.f, 0.f); cmp[i] = make_float2(0.f, 0.f); }
    const uint32_t hr = rows / 2;
    for (int p0 = beg; p0 < end; p0 += 32) {
        const int cnt = min(32, end - p0);
        uint32_t rl = 0, sl = 0;
        float2 wl = make_float2(1.f, 0.f);
        if (lane < cnt) {
            rl = (uint32_t)row_idx[p0 + lane];
            const uint32_t d = mulmod_rows<BIG>(32u, rl, rows, magic);
            wl = row_twiddle<TAB_HALF>(tab, d, rows, hr);
            sl = mulmod_rows<BIG>((uint32_t)P1_RESEED, d, rows, magic);
        }
        float2 blk[P1_KU];
#pragma unroll
        for (int i = 0; i < P1_KU; i++) blk[i] = make_float2(0.f, 0.f);
        for (int i = 0; i < cnt; i++) {
            const uint32_t r = __shfl_sync(0xffffffffu, rl, i);
            const uint32_t step = __shfl_sync(0xffffffffu, sl, i);
            const float2 wd = make_float2(__shfl_sync(0xffffffffu, wl.x, i),
                                          __shfl_sync(0xffffffffu, wl.y, i));
            uint32_t p = mulmod_rows<BIG>(u_lane, r, rows, magic);
            float2 w = make_float2(1.f, 0.f);
#pragma unroll
            for (int kk = 0; kk < P1_KU; kk++) {
                if (kk % P1_RESEED == 0) {
                    w = row_twiddle<TAB_HALF>(tab, p, rows, hr);
                    const uint32_t pn = p + step;
                    p = min(pn, pn - rows);
                } else {
                    w = cmul(w, wd);
                }
                blk[kk].x += w.x;
                blk[kk].y += w.y;
            }
        }
        if (compensated) {
#pragma unroll
            for (int kk = 0; kk < P1_KU; kk++) {
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
            for (int kk = 0; kk < P1_KU; kk++) { acc[kk].x += blk[kk].x; acc[kk].y += blk[kk].y; }
        }
    }
}

template <typename IDX, bool TAB_HALF, bool BIG>
__global__ void __launch_bounds__(P1_THREADS)
k_twiddle_sum(const int* __restrict__ slot_ptr, const IDX* __restrict__ row_idx, int n_slots,
              const float2* __restrict__ row_tab, int ntab, int rows, uint32_t magic,
              int u0, int tile_rows, float2* __restrict__ S, size_t s_pitch, int kahan_min) {
    extern __shared__ float4 smem_raw[];
    float2* stage = reinterpret_cast<float2*>(smem_raw);
    float2* tab = stage + P1_UBLK * P1_STAGE_PITCH;
    for (int i = threadIdx.x; i < ntab; i += blockDim.x) tab[i] = row_tab[i];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int n_ublk = (tile_rows + P1_UBLK - 1) / P1_UBLK;
    const int n_grp = (n_slots + P1_WARPS - 1) / P1_WARPS;
    const long nitems = (long)n_ublk * n_grp;

    for (long it = blockIdx.x; it < nitems; it += gridDim.x) {
        const int ub = (int)(it / n_grp);
        const int g = (int)(it - (long)ub * n_grp);
        const int ul0 = ub * P1_UBLK;
        const int j = g * P1_WARPS + warp;
        if (j < n_slots) {
            const uint32_t u_lane = (uint32_t)(u0 + ul0 + lane) % (uint32_t)rows;
            const int beg = slot_ptr[j], end = slot_ptr[j + 1];
            float2 acc[P1_KU];
            column_sums_warp<IDX, TAB_HALF, BIG>(row_idx, beg, end, tab, u_lane, (uint32_t)rows, magic,
                                                 lane, kahan_min > 0 && end - beg >= kahan_min, acc);
#pragma unroll
            for (int kk = 0; kk < P1_KU; kk++) stage[(lane + 32 * kk) * P1_STAGE_PITCH + warp] = acc[kk];
        }
        __syncthreads();
        for (int e = threadIdx.x; e < P1_UBLK * P1_WARPS; e += blockDim.x) {
            const int row = e / P1_WARPS, col = e - (e / P1_WARPS) * P1_WARPS;
            const int ul = ul0 + row, jj = g * P1_WARPS + col;
            if (ul < tile_rows && jj < n_slots)
                S[(size_t)ul * s_pitch + jj] = stage[row * P1_STAGE_PITCH + col];
        }
        __syncthreads();
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
// Shared memory: the padded row buffer, then the twiddles of stages >= 1
// (loaded once per CTA); stage 0's twiddles stream from L2.
//
// The reference runs 2F+4 launches per tile of rows with a global round trip
// per stage (src/sparse_fft_bluestein.cu:2327-2370) and writes 8-byte stores
// in bluestein_finalize_kernel (:469-486).
// ---------------------------------------------------------------------------
template <bool CLUSTER>
__global__ void __launch_bounds__(ROWS_THREADS, 1)
k_bluestein_rows(const float2* __restrict__ S, size_t s_pitch, int n_slots,
                 const int* __restrict__ slot_col, const float2* __restrict__ pre,
                 const float2* __restrict__ post, const float2* __restrict__ filt,
                 const float2* __restrict__ fft_tw, FFTDesc fd, int K, int rows, int cols,
                 int u0, int tile_rows, float2* __restrict__ out, size_t out_pitch) {
    extern __shared__ float4 smem_raw[];
    float2* buf = reinterpret_cast<float2*>(smem_raw);
    const int Lp = fd.Lp;
    const int Lpad = padded_len(Lp);
    float2* twr = buf + Lpad;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < fd.rest_len; i += nt) twr[i] = fft_tw[fd.rest_base + i];

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
    const float2* preq = pre + (size_t)q * n_slots;
    const float2* filtq = filt + (size_t)q * Lp;
    const int half_slots = (int)(out_pitch >> 1);
    const int hc = cols / 2;
    const bool wrap_in = cols > Lp;
    // stage 0 twiddles stream from global memory, the rest sit in shared memory
    auto tw_of = [&](int s) -> const float2* {
        return (s == 0) ? fft_tw + fd.twoff[0] : twr + (fd.twoff[s] - fd.rest_base);
    };

    for (int t = cid; t < tile_rows; t += ncl) {
        const int u = u0 + t;
        for (int i = tid; i < Lpad; i += nt) buf[i] = make_float2(0.f, 0.f);
        __syncthreads();
        const float2* srow = S + (size_t)t * s_pitch;
        if (!wrap_in) {
            for (int j = tid; j < n_slots; j += nt) {
                const int c = slot_col[j];
                buf[pad16(c)] = cmul(srow[j], preq[j]);
            }
            __syncthreads();
        } else {
            // several input columns fold onto one slot: add section by section
            for (int sec = 0; sec * Lp < cols; sec++) {
                const int lo = sec * Lp, hi = lo + Lp;
                for (int j = tid; j < n_slots; j += nt) {
                    const int c = slot_col[j];
                    if (c >= lo && c < hi) {
                        float2* d = buf + pad16(c - lo);
                        *d = cadd(*d, cmul(srow[j], preq[j]));
                    }
                }
                __syncthreads();
            }
        }
        // forward DIF, filter multiply fused with the last stage, inverse DIT
        const int S1 = fd.nst - 1;
        for (int s = 0; s < S1; s++) {
            fft_stage_dispatch<0>(fd.R[s], buf, Lp, fd.m[s], fd.magic[s], tw_of(s),
                                  (const float2*)nullptr, tid, nt);
            __syncthreads();
        }
        fft_stage_dispatch<2>(fd.R[S1], buf, Lp, fd.m[S1], fd.magic[S1], tw_of(S1), filtq, tid, nt);
        __syncthreads();
        for (int s = S1 - 1; s >= 0; s--) {
            fft_stage_dispatch<1>(fd.R[s], buf, Lp, fd.m[s], fd.magic[s], tw_of(s),
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
                    const int c = sel ? (vv == 0 ? 0 : cols - vv) : vv;
                    int n = c;
                    while (n >= Lp) n -= Lp;
                    const int pn = pad16(n);
                    if (CLUSTER) {
                        for (int qq = 0; qq < K; qq++)
                            val = cadd(val, cmul(zsrc[qq][pn], post[(size_t)qq * cols + c]));
                    } else {
                        val = cmul(buf[pn], post[c]);
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
