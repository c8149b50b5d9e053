// gbsp_planner.cu -- host-side planning (no kernels): channel split, radix
// sequences and row-block sizes ranked by an analytic model, pass-1 shapes,
// tuning candidates and the feature vector of the learned cost model.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gbsp_fft.cuh"
#include "gbsp_internal.h"
#include "gbsp_launch.h"
#include "gbsp_planner.h"

namespace gbsp {

// Stage descriptor for a given radix sequence (product must be Lp).
int build_fft_desc(int Lp, const std::vector<int>& rs, FFTDesc* fd) {
    if ((int)rs.size() > MAX_STAGES || rs.empty()) return GBSP_ERR_UNSUPPORTED;
    long prod = 1;
    for (int r : rs) {
        if (!radix_supported(r)) return GBSP_ERR_UNSUPPORTED;
        prod *= r;
    }
    if (prod != Lp) return GBSP_ERR_UNSUPPORTED;
    fd->Lp = Lp;
    fd->nst = (int)rs.size();
    int l = 1, off = 0;
    for (int s = 0; s < fd->nst; s++) {
        const int R = rs[s];
        const int m = Lp / (l * R);
        fd->R[s] = R;
        fd->m[s] = m;
        // divisor of the stage's thread -> butterfly mapping (see fft_stage)
        const int lcount = Lp / (R * m);
        const int div = (m == 1) ? 0 : (stage_j_fastest(R, m, lcount) ? lcount : m);
        fd->magic[s] = (div <= 1) ? 0u : (uint32_t)(((1ull << 32) + (uint64_t)div - 1) / (uint64_t)div);
        fd->twoff[s] = off;
        off += (R - 1) * m;
        l *= R;
    }
    fd->rest_base = (fd->R[0] - 1) * fd->m[0];
    fd->rest_len = off - fd->rest_base;
    return GBSP_OK;
}

int fft_tw_count(const FFTDesc& fd) { return fd.rest_base + fd.rest_len; }

size_t rows_smem_bytes(const FFTDesc& fd) {
    return ((size_t)row_buf_len(fd.Lp) + (size_t)fd.rest_len) * sizeof(float2);
}

// ---- radix planning -------------------------------------------------------
// Every multiset of supported radices whose product is the channel length
// (at most 7 stages) is ordered even radices first, odd radices last (an odd
// radix at span 1 keeps the last stage free of bank conflicts) and scored by
// a model fitted to GB300 measurements of the row kernel: a stage costs
// (rounds of the block over its butterflies) x radix, forward and inverse
// stages twice, the fused middle stage 1.6 times, radices above 32 a little
// more (register pressure), plus a fixed cost per stage; the row time is that
// cost divided by the CTAs resident per SM (a 512-thread block at 128
// registers fills an SM's register file, smaller blocks can pair up when
// shared memory allows).  Block sizes 256 and 512 are considered; 1024 only
// on request.  The tuner can override the choice by measurement.
static const int kRadices[] = {40, 35, 32, 28, 25, 24, 21, 20, 16, 15, 12, 9, 8, 7, 5, 4, 3, 2};

static void factorizations(int rem, int maxr, std::vector<int>& cur, std::vector<std::vector<int>>& out) {
    if (rem == 1) {
        if (!cur.empty()) out.push_back(cur);
        return;
    }
    if ((int)cur.size() >= 7) return;
    for (int r : kRadices) {
        if (r > maxr || rem % r) continue;
        cur.push_back(r);
        factorizations(rem / r, r, cur, out);
        cur.pop_back();
    }
}

static std::vector<int> order_radices(std::vector<int> rs) {
    std::stable_sort(rs.begin(), rs.end(), [](int a, int b) {
        const bool ea = (a % 2 == 0), eb = (b % 2 == 0);
        if (ea != eb) return ea;
        return a > b;
    });
    return rs;
}

// largest radix a block of the given maximum size can hold in registers
int max_radix_for(int nt_max) { return nt_max > 512 ? MAX_RADIX_NT1024 : MAX_RADIX_NT512; }

// SM limits the model uses (GB300: 228 KB shared memory, 64K registers, 2048 threads per SM)
constexpr size_t kSmemPerSM = 233472;
constexpr int kRegsPerSM = 65536;

double rows_cost(const FFTDesc& fd, int nt, size_t smem_per_cta, bool direct) {
    double cost = 0.0;
    for (int s = 0; s < fd.nst; s++) {
        const int R = fd.R[s], m = fd.m[s], nb = fd.Lp / R, l = nb / m;
        const double rounds = std::ceil((double)nb / (double)nt);
        // radices 35 and 40 spill at 128 registers a thread: weight 1.5,
        // fitted to the tuner's timings of 2200 matrices (mean row-kernel
        // regret of the first pick 4.1 % -> 3.7 %).  A fused last stage of
        // radix 2 or 3 costs twice its share (the filter load and the pairing
        // are paid per element, with little arithmetic to hide them): 1890
        // timed matrices 3.4 -> 3.1 %, and on GB300 every x,..,3 plan measured
        // against its replacement was slower (3460^2 10 %, 40421^2 3-smooth 8 %)
        const bool last = s == fd.nst - 1;
        double per = rounds * R * (R > 32 ? 1.5 : 1.0) * (last && R <= 3 ? 2.0 : 1.0);
        const bool strided = (m == 1 && R % 2 == 0) ||
                             (m > 1 && m < 16 && l > 1 && !stage_j_fastest(R, m, l));
        if (direct && m == 1 && R % 2 == 0) {
            // A span-1 stage of even radix reads buf[t*R + s]: its bank
            // conflicts grow with R's power-of-two part.  Fitted on direct
            // plans only (GB300, 4001 rows, eight candidates each at seven
            // smooth lengths): the first pick's mean regret 11.1 -> 3.5 %
            // (cols 4096: [16, 16, 16] 0.121 ms -> [16, 8, 8, 4] 0.094 ms).
            per *= std::max(1.5, (double)(R & -R) / 4.0);
        } else if (strided) {
            per *= 1.5;
        }
        cost += (last ? 1.6 : 2.0) * per + 12.0;
    }
    const int regs = nt <= 512 ? 128 : 64;
    int ctas = std::min({(int)(kSmemPerSM / (smem_per_cta + 1024)), 2048 / nt, kRegsPerSM / (nt * regs)});
    ctas = std::max(ctas, 1);
    return cost / ctas;
}

std::vector<RadixPlan> rank_radices(int Lp, size_t smem_cap, const int* radix_opt, int nt_opt, bool direct) {
    std::vector<std::vector<int>> cands;
    if (radix_opt && radix_opt[0] > 0) {
        std::vector<int> rs;
        for (int i = 0; i < 8 && radix_opt[i] > 0; i++) rs.push_back(radix_opt[i]);
        cands.push_back(rs);
    } else {
        std::vector<int> cur;
        factorizations(Lp, 64, cur, cands);
        for (auto& c : cands) c = order_radices(c);
    }
    std::vector<RadixPlan> out;
    for (const auto& rs : cands) {
        FFTDesc fd{};
        if (build_fft_desc(Lp, rs, &fd) != GBSP_OK) continue;
        if (rows_smem_bytes(fd) > smem_cap) continue;
        const int rmax = *std::max_element(rs.begin(), rs.end());
        const int nt_hi = rmax > max_radix_for(1024) ? 512 : 1024;
        if (rmax > max_radix_for(512)) continue;
        for (int nt : {256, 512, 1024, nt_opt}) {
            if (nt <= 0 || nt > nt_hi || (nt_opt > 0 && nt != nt_opt) || (nt_opt == 0 && nt == 1024)) continue;
            if (nt_opt > 0 && !out.empty() && out.back().nt == nt && std::memcmp(&out.back().fd, &fd, sizeof(fd)) == 0)
                continue;  // nt_opt listed twice
            RadixPlan rp;
            rp.fd = fd;
            rp.nt = nt;
            rp.cost = rows_cost(fd, nt, rows_smem_bytes(fd), direct);
            out.push_back(rp);
        }
    }
    std::stable_sort(out.begin(), out.end(), [](const RadixPlan& a, const RadixPlan& b) { return a.cost < b.cost; });
    return out;
}

int split_channels(int cols, const gbsp_options* o, size_t smem_cap, ChannelSplit* out) {
    const int policy = (o && o->length_policy) ? o->length_policy : GBSP_LEN_3SMOOTH;
    if (policy != GBSP_LEN_3SMOOTH && policy != GBSP_LEN_7SMOOTH && policy != GBSP_LEN_POW2)
        return set_error(GBSP_ERR_INVALID, "length_policy must be 2, 3 or 7");
    const int nt_opt = o ? o->rows_threads : 0;
    if (nt_opt < 0 || nt_opt % 32 || nt_opt > 1024)
        return set_error(GBSP_ERR_INVALID, "rows_threads must be 0 or a multiple of 32 up to 1024");
    // By default a channel is as long as shared memory allows (the row
    // buffer plus the inner stages' twiddles, about 28k points on GB300):
    // fewer channels were faster at every length measured (a cap of 24000
    // had split cols 25000 into four channels, 1.88 ms against 0.37 ms for
    // the direct FFT in one; 40421^2 into five, 32.6 against 30.5 ms for three)
    const int maxLp = (o && o->max_channel_len > 0) ? o->max_channel_len : 0;
    auto channel_fits = [&](long lp) {
        return lp >= 2 && (maxLp == 0 || lp <= maxLp) && (size_t)row_buf_len((int)lp) * sizeof(float2) <= smem_cap;
    };
    // Direct: when cols itself has the policy's smoothness and fits one CTA,
    // the row DFT is one forward FFT of length cols -- the same DFT as the
    // Bluestein convolution, with a quarter of its FFT work and less rounding
    out->direct = 0;
    if (!(o && o->force_bluestein) && channel_fits(cols) && next_smooth(cols, policy) == cols) {
        auto ranked = rank_radices(cols, smem_cap, o ? o->radix : nullptr, nt_opt, true);
        if (!ranked.empty()) {
            out->L = cols;
            out->K = 1;
            out->Lp = cols;
            out->direct = 1;
            out->ranked = std::move(ranked);
            return GBSP_OK;
        }
    }
    long L = next_smooth(2L * cols - 1, policy);
    if (L < 2) L = 2;
    if (L > (1L << 28)) return set_error(GBSP_ERR_UNSUPPORTED, "fft_len too large");
    out->L = (int)L;
    out->K = 0;
    // more than MAX_CHANNELS channels only run sequentially in one CTA
    const int kmax = (o && o->channel_mode == 1) ? MAX_CHANNELS : MAX_SEQ_CHANNELS;
    for (int k = 1; k <= kmax; k++) {
        if (L % k || !channel_fits(L / k)) continue;
        auto ranked = rank_radices((int)(L / k), smem_cap, o ? o->radix : nullptr, nt_opt);
        if (ranked.empty()) continue;
        out->K = k;
        out->Lp = (int)(L / k);
        out->ranked = std::move(ranked);
        return GBSP_OK;
    }
    return set_error(GBSP_ERR_UNSUPPORTED, "fft_len " + std::to_string(L) + " does not split into <= " +
                                               std::to_string(kmax) + " channels" +
                                               (maxLp > 0 ? " of <= " + std::to_string(maxLp) : std::string()) +
                                               " that fit in shared memory");
}

// Shapes by index (the 1-based gbsp_options.pass1_shape minus one).  Window
// widths must be 16, 32 or 64: the pass-1 window epilogue indexes its tile
// by shift and mask.  A 16-column window halves the result tile (256 x 33
// entries), which lets the full twiddle table fit for up to ~16.9k rows.
const P1Shape kP1Shapes[N_P1_SHAPES] = {{8, 32, TAB_FULL}, {8, 32, TAB_HALF}, {4, 64, TAB_FULL}, {8, 16, TAB_FULL},
                                        {8, 16, TAB_HALF}, {4, 32, TAB_HALF}, {8, 32, TAB_TWO},  {4, 32, TAB_TWO}};
// Preference order of the automatic choice, measured on GB300: 256-row items
// with the full table, then with the half table, then with the two-level
// table (its small table leaves room for 256-row items where the half table
// only allows 128: 40421^2 pass 1 6.03 ms against 6.93 ms), then the rest.
static const int kP1Preference[N_P1_SHAPES] = {0, 1, 6, 2, 3, 4, 5, 7};

size_t row_table_entries(int tab, int rows) {
    if (tab == TAB_HALF) return (size_t)(rows / 2 + 1);
    if (tab == TAB_TWO) return (size_t)TWO_LO + (size_t)(rows + TWO_LO - 1) / TWO_LO;
    return (size_t)rows;
}

size_t p1_smem_bytes(const P1Shape& sh, int rows) {
    return p1_head_bytes(sh.ku, sh.cw) + row_table_entries(sh.tab, rows) * 8;
}

std::vector<int> fitting_p1_shapes(int rows, size_t smem_cap, int table_mode) {
    std::vector<int> out;
    for (int pi = 0; pi < N_P1_SHAPES; pi++) {
        const int i = kP1Preference[pi];
        const P1Shape& sh = kP1Shapes[i];
        if (table_mode == 1 && sh.tab != TAB_FULL) continue;
        if (table_mode == 2 && sh.tab != TAB_HALF) continue;
        if (table_mode == 3 && sh.tab != TAB_TWO) continue;
        if (p1_smem_bytes(sh, rows) + 1024 > smem_cap) continue;  // + static shared variables
        out.push_back(i);
    }
    return out;
}

int device_limits(int dev, DeviceLimits* out) {
    constexpr int kMaxDev = 64;
    static std::mutex mu;
    static DeviceLimits cache[kMaxDev];
    if (dev < 0 || dev >= kMaxDev) return set_error(GBSP_ERR_UNSUPPORTED, "device index out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (cache[dev].sms == 0) {
        int optin = 0, sms = 0;
        GB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        cache[dev].smem_optin = (size_t)optin;
        cache[dev].sms = sms;
    }
    *out = cache[dev];
    return GBSP_OK;
}

int allow_full_smem(const void* kern) {
    static std::mutex mu;
    static std::vector<std::pair<const void*, int>> done;  // (kernel, device) already raised
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    const std::pair<const void*, int> key(kern, dev);
    std::lock_guard<std::mutex> lk(mu);
    if (std::find(done.begin(), done.end(), key) != done.end()) return GBSP_OK;
    cudaFuncAttributes fa;
    DeviceLimits lim;
    GB_CUDA(cudaFuncGetAttributes(&fa, kern));
    if (int rc = device_limits(dev, &lim)) return rc;
    GB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)lim.smem_optin - (int)fa.sharedSizeBytes));
    done.push_back(key);
    return GBSP_OK;
}

size_t device_smem_cap() {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess && optin > 0)
        return (size_t)optin;
    cudaGetLastError();
    return 232448;
}

int enumerate_candidates(int rows, int cols, const gbsp_options* base, size_t smem_cap, int max_rows,
                         std::vector<gbsp_options>* out, int* n_rows, int* n_p1) {
    if (rows < 1 || cols < 1 || max_rows < 1) return set_error(GBSP_ERR_INVALID, "enumerate_candidates: bad sizes");
    gbsp_options o = base ? *base : gbsp_options{};
    ChannelSplit sp;
    if (int rc = split_channels(cols, &o, smem_cap, &sp)) return rc;
    const int tmode = o.row_table_mode;
    std::vector<int> shapes;
    if (o.pass1_shape > 0) {
        if (o.pass1_shape > N_P1_SHAPES) return set_error(GBSP_ERR_INVALID, "pass1_shape out of range");
        shapes.push_back(o.pass1_shape - 1);
    } else {
        shapes = fitting_p1_shapes(rows, smem_cap, tmode);
    }
    if (shapes.empty()) return set_error(GBSP_ERR_UNSUPPORTED, "rows too large for a shared-memory twiddle table");
    const int nr = std::min<int>(max_rows, (int)sp.ranked.size());
    out->clear();
    for (int i = 0; i < nr; i++) {
        for (int j : shapes) {
            gbsp_options c = o;
            std::memset(c.radix, 0, sizeof(c.radix));
            const FFTDesc& fd = sp.ranked[i].fd;
            if (fd.nst > 8) return set_error(GBSP_ERR_UNSUPPORTED, "more than 8 radix stages");
            for (int s = 0; s < fd.nst; s++) c.radix[s] = fd.R[s];
            c.rows_threads = sp.ranked[i].nt;
            c.pass1_shape = j + 1;
            out->push_back(c);
        }
    }
    *n_rows = nr;
    *n_p1 = (int)shapes.size();
    return GBSP_OK;
}

static int largest_prime_factor(int n) {
    int best = 1;
    for (int p = 2; (long)p * p <= n; p++)
        while (n % p == 0) {
            best = p;
            n /= p;
        }
    return n > 1 ? std::max(best, n) : best;
}

static float lg2(double x) { return (float)std::log2(std::max(x, 1e-30)); }

int plan_features(int rows, int cols, int n_active, int nnz, const int* col_ptr, const gbsp_options* cand,
                  size_t smem_cap, float* f) {
    if (!cand || !f || rows < 1 || cols < 1 || n_active < 0 || nnz < 0 || (n_active > 0 && !col_ptr))
        return set_error(GBSP_ERR_INVALID, "plan_features: bad arguments");
    ChannelSplit sp;
    if (int rc = split_channels(cols, cand, smem_cap, &sp)) return rc;
    const RadixPlan& rp = sp.ranked[0];  // radix and rows_threads of cand restrict the ranking to one choice
    const int sh_idx = cand->pass1_shape - 1;
    if (sh_idx < 0 || sh_idx >= N_P1_SHAPES) return set_error(GBSP_ERR_INVALID, "plan_features: pass1_shape unset");
    const P1Shape& sh = kP1Shapes[sh_idx];
    const int half_rows = rows / 2 + 1;
    std::fill(f, f + N_FEATURES, 0.f);
    // matrix
    int maxdeg = 0;
    double hist[6] = {0, 0, 0, 0, 0, 0};
    for (int j = 0; j < n_active; j++) {
        const int d = col_ptr[j + 1] - col_ptr[j];
        maxdeg = std::max(maxdeg, d);
        const int b = d <= 1 ? 0 : d <= 3 ? 1 : d <= 7 ? 2 : d <= 15 ? 3 : d <= 63 ? 4 : 5;
        hist[b] += 1.0;
    }
    f[0] = lg2(rows);
    f[1] = lg2(cols);
    f[2] = lg2(nnz + 1.0);
    f[3] = lg2(n_active + 1.0);
    f[4] = lg2((nnz + 1.0) / ((double)rows * cols));
    f[5] = lg2(largest_prime_factor(rows));
    f[6] = lg2(largest_prime_factor(cols));
    f[7] = lg2(sp.L);
    f[8] = (float)sp.K;
    f[9] = lg2(maxdeg + 1.0);
    for (int b = 0; b < 6; b++) f[10 + b] = n_active ? (float)(hist[b] / n_active) : 0.f;
    f[16] = lg2((double)half_rows * cols);
    f[17] = lg2((double)nnz * half_rows + 1.0);
    // row choice
    const FFTDesc& fd = rp.fd;
    int rmax = 0;
    for (int s = 0; s < fd.nst; s++) rmax = std::max(rmax, fd.R[s]);
    f[18] = rp.nt / 512.f;
    f[19] = (float)fd.nst;
    for (int s = 0; s < 4 && s < fd.nst; s++) f[20 + s] = lg2(fd.R[s]);
    f[24] = lg2(rmax);
    f[25] = lg2((double)rows_smem_bytes(fd));
    const int regs = rp.nt <= 512 ? 128 : 64;
    f[26] = (float)std::max(1, std::min({(int)(233472 / (rows_smem_bytes(fd) + 1024)), 2048 / rp.nt,
                                         65536 / (rp.nt * regs)}));
    // (the Bluestein form of the row model for every plan: the feature the
    // cost model was trained on)
    f[27] = lg2(rows_cost(fd, rp.nt, rows_smem_bytes(fd)));
    // pass-1 shape (the two-level shapes share the slot of their half-table
    // twin: the model never saw them, and they only appear when nothing else fits)
    f[28 + (sh_idx == 6 ? 1 : sh_idx == 7 ? 5 : sh_idx)] = 1.f;
    const int s_cols = (cols + 1) & ~1;
    const double items = std::ceil(half_rows / (32.0 * sh.ku)) * std::ceil((double)s_cols / sh.cw);
    f[34] = lg2(items);
    f[35] = lg2((double)p1_smem_bytes(sh, rows));
    return GBSP_OK;
}

}  // namespace gbsp

using gbsp::set_error;

extern "C" {

int gbsp_plan_candidates(int rows, int cols, const gbsp_options* base, int max_rows_cands, gbsp_options* out,
                         int cap, int* n_rows_cands, int* n_p1_cands) {
    if (!n_rows_cands || !n_p1_cands || (cap > 0 && !out))
        return set_error(GBSP_ERR_INVALID, "gbsp_plan_candidates: null argument");
    std::vector<gbsp_options> c;
    int nr = 0, np = 0;
    if (int rc = gbsp::enumerate_candidates(rows, cols, base, gbsp::device_smem_cap(), max_rows_cands, &c, &nr, &np))
        return rc;
    *n_rows_cands = nr;
    *n_p1_cands = np;
    if ((int)c.size() > cap)
        return set_error(GBSP_ERR_INVALID, "gbsp_plan_candidates: cap < " + std::to_string(c.size()));
    std::copy(c.begin(), c.end(), out);
    return GBSP_OK;
}

int gbsp_plan_features(int rows, int cols, int n_active, int nnz, const int* col_ptr, const gbsp_options* cand,
                       float* out) {
    return gbsp::plan_features(rows, cols, n_active, nnz, col_ptr, cand, gbsp::device_smem_cap(), out);
}

int gbsp_autotune(int rows, int cols, int n_active, int nnz, const int* col_ptr, const int* row_idx,
                  const int* sparse_cols, const gbsp_options* base, int max_rows_cands, int reps, void* stream,
                  gbsp_options* best, gbsp_tune_entry* entries, int cap, int* n_rows_cands, int* n_p1_cands) {
    if (!best || !n_rows_cands || !n_p1_cands || reps < 1 || (cap > 0 && !entries))
        return set_error(GBSP_ERR_INVALID, "gbsp_autotune: bad arguments");
    gbsp_options b = base ? *base : gbsp_options{};
    b.planner = GBSP_PLANNER_MODEL;
    std::vector<gbsp_options> c;
    int nr = 0, np = 0;
    if (int rc = gbsp::enumerate_candidates(rows, cols, &b, gbsp::device_smem_cap(), max_rows_cands, &c, &nr, &np))
        return rc;
    *n_rows_cands = nr;
    *n_p1_cands = np;
    if (cap > 0 && (int)c.size() > cap)
        return set_error(GBSP_ERR_INVALID, "gbsp_autotune: cap < " + std::to_string(c.size()));
    const size_t pitch = (size_t)((cols / 2 + 1 + 3) / 4 * 4);
    void* d_out = nullptr;
    cudaError_t e = cudaMalloc(&d_out, (size_t)rows * pitch * 8);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(GBSP_ERR_ALLOC, std::string("gbsp_autotune: output buffer: ") + cudaGetErrorString(e));
    }
    std::vector<float> p1(np, INFINITY), rw(nr, INFINITY);
    int rc = GBSP_OK;
    const int T = std::max(nr, np);
    for (int t = 0; t < T && rc == GBSP_OK; t++) {
        const int i = t % nr, j = t % np;
        gbsp_plan_t pl = nullptr;
        rc = gbsp_plan_create(rows, cols, n_active, nnz, col_ptr, row_idx, sparse_cols, &c[(size_t)i * np + j], stream,
                              &pl);
        if (rc) break;
        rc = gbsp_execute(pl, d_out, pitch, stream);  // warm-up
        for (int r = 0; r < reps && rc == GBSP_OK; r++) {
            float a = 0.f, q = 0.f;
            rc = gbsp_execute_profiled(pl, d_out, pitch, stream, &a, &q);
            p1[j] = std::min(p1[j], a);
            rw[i] = std::min(rw[i], q);
        }
        gbsp_plan_destroy(pl);
    }
    if (rc) {
        cudaFree(d_out);
        return rc;
    }
    int bi = 0, bj = 0;
    for (int i = 0; i < nr; i++)
        for (int j = 0; j < np; j++) {
            if (cap > 0) {
                gbsp_tune_entry& en = entries[(size_t)i * np + j];
                en.opts = c[(size_t)i * np + j];
                en.ms_pass1 = p1[j];
                en.ms_rows = rw[i];
            }
            if (p1[j] + rw[i] < p1[bj] + rw[bi]) {
                bi = i;
                bj = j;
            }
        }
    *best = c[(size_t)bi * np + bj];
    // The --csc-tile analogue: Bluestein rows per tile, at most the caller's
    // u_tile (0 = all rows); smaller tiles bound the scratch memory, and the
    // fastest of {limit, limit/2, limit/4} is kept.
    {
        const int half_rows = rows / 2 + 1;
        const int limit = (b.u_tile > 0) ? std::min(b.u_tile, half_rows) : half_rows;
        float best_ms = INFINITY;
        int best_tile = limit;
        for (int div = 1; div <= 4 && rc == GBSP_OK; div *= 2) {
            const int tile = std::max(1, limit / div);
            if (div > 1 && tile == limit / (div / 2)) break;
            gbsp_options o = *best;
            o.u_tile = tile;
            gbsp_plan_t pl = nullptr;
            if ((rc = gbsp_plan_create(rows, cols, n_active, nnz, col_ptr, row_idx, sparse_cols, &o, stream, &pl)))
                break;
            rc = gbsp_execute(pl, d_out, pitch, stream);
            float tot = INFINITY;
            for (int r = 0; r < reps && rc == GBSP_OK; r++) {
                float x = 0.f, y = 0.f;
                rc = gbsp_execute_profiled(pl, d_out, pitch, stream, &x, &y);
                tot = std::min(tot, x + y);
            }
            gbsp_plan_destroy(pl);
            if (tot < best_ms) {
                best_ms = tot;
                best_tile = tile;
            }
        }
        if (rc == GBSP_OK) best->u_tile = (best_tile == half_rows) ? 0 : best_tile;
    }
    cudaFree(d_out);
    return rc;
}

}  // extern "C"
