// gbsp_planner.h -- host-side planning: channel split, radix sequences and
// row-block sizes ranked by an analytic model, pass-1 shapes, the tuning
// candidates of a matrix and the features the learned cost model reads.
#pragma once
#include <cstddef>
#include <vector>

#include "gbspfft.h"
#include "gbsp_layout.h"

namespace gbsp {

// ---- channel FFT
int build_fft_desc(int Lp, const std::vector<int>& rs, FFTDesc* fd);
int fft_tw_count(const FFTDesc& fd);
size_t rows_smem_bytes(const FFTDesc& fd);
int max_radix_for(int nt_max);  // largest radix a block of at most nt_max threads holds
// direct: the plan is one forward FFT (no Bluestein convolution)
double rows_cost(const FFTDesc& fd, int nt, size_t smem_per_cta, bool direct = false);

struct RadixPlan {
    FFTDesc fd{};
    int nt = 0;
    double cost = 1e300;
};
// Every (radix sequence, block size) for channel length Lp that fits in
// smem_cap, cheapest first by rows_cost.  radix_opt (0-terminated, may be
// null) and nt_opt (0 = automatic: 256 or 512) restrict the set.
std::vector<RadixPlan> rank_radices(int Lp, size_t smem_cap, const int* radix_opt, int nt_opt,
                                    bool direct = false);

// Channel split of the length-L convolution: the smallest K (<= MAX_CHANNELS
// for clusters, MAX_SEQ_CHANNELS for sequential channels)
// whose channel length fits; ranked radix choices for that channel.
struct ChannelSplit {
    int L = 0, K = 0, Lp = 0;
    int direct = 0;  // 1: one forward FFT of length cols (cols smooth), no Bluestein
    std::vector<RadixPlan> ranked;
};
int split_channels(int cols, const gbsp_options* o, size_t smem_cap, ChannelSplit* out);

// ---- pass 1 shapes: {rows per lane, window width, twiddle table layout
// (TAB_FULL, TAB_HALF, TAB_TWO)}
struct P1Shape {
    int ku, cw, tab;
};
constexpr int N_P1_SHAPES = 8;
extern const P1Shape kP1Shapes[N_P1_SHAPES];
size_t row_table_entries(int tab, int rows);
size_t p1_smem_bytes(const P1Shape& sh, int rows);
// Indices (0-based, preference order) of the shapes that fit for `rows`
// under the table mode (0 auto, 1 full, 2 half, 3 two-level).
std::vector<int> fitting_p1_shapes(int rows, size_t smem_cap, int table_mode);

// Shared memory per CTA available to the kernels: the current device's
// opt-in limit, or GB300's 232448 bytes when no device is visible.
size_t device_smem_cap();

// ---- tuning candidates and cost-model features
// Candidates for a matrix: the `max_rows` cheapest (radix, block) choices
// crossed with every fitting pass-1 shape; out[i * n_p1 + j] pairs row
// choice i with shape j.  Each is `base` with radix, rows_threads and
// pass1_shape filled in.
int enumerate_candidates(int rows, int cols, const gbsp_options* base, size_t smem_cap, int max_rows,
                         std::vector<gbsp_options>* out, int* n_rows, int* n_p1);

constexpr int N_FEATURES = 36;
// Feature vector of (matrix, candidate): [0,18) matrix, [18,28) row
// choice, [28,36) pass-1 shape.  col_ptr: compact CSC (n_active + 1).
int plan_features(int rows, int cols, int n_active, int nnz, const int* col_ptr, const gbsp_options* cand,
                  size_t smem_cap, float* out);

// ---- learned cost model (gbsp_mlp.cu)
bool cost_model_loaded(int n_in);
// false when a feature of the n candidates lies outside the installed
// training range by more than DOMAIN_MARGIN of its width (always true when
// no range is installed)
constexpr float DOMAIN_MARGIN = 0.1f;
bool cost_model_in_domain(const float* feats, int n);
// Predicted log-latency of n candidates (raw features, n x N_FEATURES).
int cost_model_predict(const float* feats, int n, float* out);

}  // namespace gbsp
