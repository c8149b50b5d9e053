// gbsp_layout.h -- sizes and descriptors shared by the kernels and the host
// planner (no device code, so host-only translation units can include it).
#pragma once
#include <cstddef>
#include <cstdint>

#ifdef __CUDACC__
#define GBSP_HD __host__ __device__
#else
#define GBSP_HD
#endif

namespace gbsp {

constexpr int MAX_STAGES = 16;
constexpr int MAX_CHANNELS = 8;       // channels a thread-block cluster can hold
constexpr int MAX_SEQ_CHANNELS = 64;  // channels one CTA runs in turn (very wide matrices)
constexpr int P1_THREADS = 512;     // k_twiddle_sum block size
constexpr int P1_WARPS = P1_THREADS / 32;
constexpr int P1_RESEED = 4;        // exact table lookup every P1_RESEED rows
// k_twiddle_sum shapes: KU Bluestein rows per lane (32*KU per work item) and
// windows of cw consecutive columns cut into at most cw + P1_WARPS tasks
GBSP_HD constexpr int p1_vmax(int cw) { return cw + P1_WARPS; }
GBSP_HD constexpr int p1_pitch(int cw) { return p1_vmax(cw) + 1; }
// shared memory before the twiddle table: result tile + per-warp nonzero data
GBSP_HD constexpr size_t p1_head_bytes(int ku, int cw) {
    return (size_t)32 * ku * p1_pitch(cw) * 8 + (size_t)P1_WARPS * 32 * 16;
}
// complex slots of the row kernel's shared-memory row buffer for a channel of
// Lp points: rounded up to even, so the bulk copy of an odd-length row (which
// moves whole 16-byte pairs) stays inside the buffer
GBSP_HD constexpr int row_buf_len(int Lp) { return (Lp + 1) & ~1; }
// pass-1 twiddle table layouts (see row_twiddle)
constexpr int TAB_FULL = 0, TAB_HALF = 1, TAB_TWO = 2;
constexpr int TWO_LO_BITS = 8, TWO_LO = 1 << TWO_LO_BITS;
constexpr long long WAIT_LIMIT = 1LL << 26;  // bounded spin on an mbarrier (~seconds)
constexpr int ERR_TIMEOUT = 1;              // bit set in the plan's error word
constexpr int ERR_RADIX = 2;                // a stage radix the kernel was not compiled for

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

}  // namespace gbsp
