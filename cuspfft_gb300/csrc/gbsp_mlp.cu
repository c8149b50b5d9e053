// gbsp_mlp.cu -- the learned cost model: a small MLP (n_in -> 64 -> 64 -> 1,
// ReLU, FP32) with hand-written forward, backward and Adam kernels, and the
// model GBSP_PLANNER_LEARNED consults when a plan is created.
//
// Parameters, packed: W1[n_in][64], b1[64], W2[64][64], b2[64], w3[64], b3.
// One CTA of 64 threads works on tiles of TB samples, thread j owning hidden
// unit j.  The backward kernel runs on a fixed grid; each CTA sums its tiles'
// gradients in a fixed order and a second kernel adds the CTAs' partial sums
// in CTA order, so gradients are bit-reproducible.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "gbspfft.h"
#include "gbsp_internal.h"
#include "gbsp_planner.h"

namespace gbsp {
namespace {

constexpr int H = GBSP_MLP_HIDDEN;
constexpr int TB = 16;          // samples per tile
constexpr int MAX_IN = 48;      // largest n_in the kernels take (static shared memory)
constexpr int BWD_GRID = 256;   // CTAs of the backward kernel (fixed: reduction order)

struct Layout {
    size_t w1, b1, w2, b2, w3, b3, total;
};
__host__ __device__ inline Layout layout(int n_in) {
    Layout l;
    l.w1 = 0;
    l.b1 = l.w1 + (size_t)n_in * H;
    l.w2 = l.b1 + H;
    l.b2 = l.w2 + (size_t)H * H;
    l.w3 = l.b2 + H;
    l.b3 = l.w3 + H;
    l.total = l.b3 + 1;
    return l;
}

struct TileBufs {
    float xs[TB][MAX_IN];
    float h1[TB][H + 1];
    float h2[TB][H + 1];  // after the output layer: d2 = dL/d(pre-activation 2)
    float ys[TB];
};

// Forward pass of one tile starting at sample s0; leaves h1, h2, ys in smem.
__device__ void tile_forward(const float* __restrict__ P, const Layout& L, int n_in, const float* __restrict__ x,
                             int n, int s0, TileBufs& b) {
    const int j = threadIdx.x;
    for (int e = j; e < TB * n_in; e += H) {
        const int s = e / n_in, k = e - s * n_in;
        b.xs[s][k] = (s0 + s < n) ? x[(size_t)(s0 + s) * n_in + k] : 0.f;
    }
    __syncthreads();
    float acc[TB];
#pragma unroll
    for (int s = 0; s < TB; s++) acc[s] = P[L.b1 + j];
    for (int k = 0; k < n_in; k++) {
        const float w = P[L.w1 + (size_t)k * H + j];
#pragma unroll
        for (int s = 0; s < TB; s++) acc[s] = fmaf(b.xs[s][k], w, acc[s]);
    }
#pragma unroll
    for (int s = 0; s < TB; s++) b.h1[s][j] = fmaxf(acc[s], 0.f);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < TB; s++) acc[s] = P[L.b2 + j];
    for (int k = 0; k < H; k++) {
        const float w = P[L.w2 + (size_t)k * H + j];
#pragma unroll
        for (int s = 0; s < TB; s++) acc[s] = fmaf(b.h1[s][k], w, acc[s]);
    }
#pragma unroll
    for (int s = 0; s < TB; s++) b.h2[s][j] = fmaxf(acc[s], 0.f);
    __syncthreads();
    if (j < TB) {
        float y = P[L.b3];
        for (int k = 0; k < H; k++) y = fmaf(b.h2[j][k], P[L.w3 + k], y);
        b.ys[j] = y;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(H) k_mlp_forward(const float* __restrict__ P, int n_in, const float* __restrict__ x,
                                                   int n, float* __restrict__ y) {
    __shared__ TileBufs b;
    const Layout L = layout(n_in);
    for (int s0 = blockIdx.x * TB; s0 < n; s0 += gridDim.x * TB) {
        tile_forward(P, L, n_in, x, n, s0, b);
        if (threadIdx.x < TB && s0 + threadIdx.x < n) y[s0 + threadIdx.x] = b.ys[threadIdx.x];
        __syncthreads();
    }
}

// Per-CTA gradient sums over its tiles (tiles blockIdx.x, +gridDim.x, ...):
// part[blockIdx.x][0, total) in parameter layout, part[..][total] = sum of
// squared errors.
__global__ void __launch_bounds__(H) k_mlp_backward(const float* __restrict__ P, int n_in,
                                                    const float* __restrict__ x, const float* __restrict__ t, int n,
                                                    float* __restrict__ part) {
    __shared__ TileBufs b;
    __shared__ float d1[TB][H + 1];
    __shared__ float dy[TB];
    __shared__ float gw1[MAX_IN][H];
    __shared__ float gw2[H][H];
    const Layout L = layout(n_in);
    const int j = threadIdx.x;
    for (int k = 0; k < n_in; k++) gw1[k][j] = 0.f;
    for (int k = 0; k < H; k++) gw2[k][j] = 0.f;
    float gb1 = 0.f, gb2 = 0.f, gw3 = 0.f, gb3 = 0.f, sse = 0.f;
    const float scale = 2.f / (float)n;
    const float w3j = P[L.w3 + j];
    for (int s0 = blockIdx.x * TB; s0 < n; s0 += gridDim.x * TB) {
        tile_forward(P, L, n_in, x, n, s0, b);
        if (j < TB) {
            const bool ok = s0 + j < n;
            const float e = ok ? b.ys[j] - t[s0 + j] : 0.f;
            dy[j] = scale * e;
            b.ys[j] = e * e;
        }
        __syncthreads();
        if (j == 0)
            for (int s = 0; s < TB; s++) {
                sse += b.ys[s];
                gb3 += dy[s];
            }
        // output layer and second hidden layer (thread j owns column j)
#pragma unroll 4
        for (int s = 0; s < TB; s++) {
            const float h = b.h2[s][j];
            gw3 = fmaf(dy[s], h, gw3);
            const float d = (h > 0.f) ? dy[s] * w3j : 0.f;
            b.h2[s][j] = d;
            gb2 += d;
        }
        __syncthreads();
        for (int k = 0; k < H; k++) {
            float g = 0.f;
#pragma unroll
            for (int s = 0; s < TB; s++) g = fmaf(b.h1[s][k], b.h2[s][j], g);
            gw2[k][j] += g;
        }
        // first hidden layer: thread j now owns input unit j of layer 2
        {
            float acc[TB];
#pragma unroll
            for (int s = 0; s < TB; s++) acc[s] = 0.f;
            for (int q = 0; q < H; q++) {
                const float w = P[L.w2 + (size_t)j * H + q];
#pragma unroll
                for (int s = 0; s < TB; s++) acc[s] = fmaf(b.h2[s][q], w, acc[s]);
            }
#pragma unroll
            for (int s = 0; s < TB; s++) {
                const float d = (b.h1[s][j] > 0.f) ? acc[s] : 0.f;
                d1[s][j] = d;
                gb1 += d;
            }
        }
        __syncthreads();
        for (int k = 0; k < n_in; k++) {
            float g = 0.f;
#pragma unroll
            for (int s = 0; s < TB; s++) g = fmaf(b.xs[s][k], d1[s][j], g);
            gw1[k][j] += g;
        }
        __syncthreads();
    }
    float* out = part + (size_t)blockIdx.x * (L.total + 1);
    for (int k = 0; k < n_in; k++) out[L.w1 + (size_t)k * H + j] = gw1[k][j];
    for (int k = 0; k < H; k++) out[L.w2 + (size_t)k * H + j] = gw2[k][j];
    out[L.b1 + j] = gb1;
    out[L.b2 + j] = gb2;
    out[L.w3 + j] = gw3;
    if (j == 0) {
        out[L.b3] = gb3;
        out[L.total] = sse / (float)n;
    }
}

// grad[p] = sum over CTAs b = 0, 1, ... of part[b][p]; loss likewise.
__global__ void k_mlp_reduce(const float* __restrict__ part, int nblk, size_t total, float* __restrict__ grad,
                             float* __restrict__ loss) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p > total) return;
    float acc = 0.f;
    for (int b = 0; b < nblk; b++) acc += part[(size_t)b * (total + 1) + p];
    if (p < total) grad[p] = acc;
    else *loss = acc;
}

__global__ void k_mlp_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                           float* __restrict__ v, size_t n, float lr, float b1, float b2, float eps, float c1,
                           float c2) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

#define MLP_CUDA(call)                                                                             \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return set_error(GBSP_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int check_n_in(int n_in) {
    if (n_in < 1 || n_in > MAX_IN) return set_error(GBSP_ERR_INVALID, "mlp: n_in must be in [1, 48]");
    return GBSP_OK;
}

int forward_grid(int n) { return std::max(1, std::min((n + TB - 1) / TB, 4096)); }

// ---- installed model
std::mutex g_model_mu;
std::vector<float> g_params, g_mean, g_scale;
std::vector<float> g_lo, g_hi;  // feature range of the training candidates (empty: no limit)
int g_n_in = 0;

}  // namespace

bool cost_model_in_domain(const float* feats, int n) {
    std::lock_guard<std::mutex> lk(g_model_mu);
    if (g_lo.empty()) return true;
    for (int i = 0; i < n; i++)
        for (int k = 0; k < g_n_in; k++) {
            const float f = feats[(size_t)i * g_n_in + k];
            const float margin = DOMAIN_MARGIN * (g_hi[k] - g_lo[k]);
            if (!(f >= g_lo[k] - margin && f <= g_hi[k] + margin)) return false;
        }
    return true;
}

bool cost_model_loaded(int n_in) {
    std::lock_guard<std::mutex> lk(g_model_mu);
    return g_n_in == n_in && !g_params.empty();
}

int cost_model_predict(const float* feats, int n, float* out) {
    std::vector<float> params, mean, scale;
    int n_in;
    {
        std::lock_guard<std::mutex> lk(g_model_mu);
        params = g_params;
        mean = g_mean;
        scale = g_scale;
        n_in = g_n_in;
    }
    if (params.empty() || n < 1) return set_error(GBSP_ERR_INVALID, "cost model: nothing installed or no input");
    std::vector<float> xs((size_t)n * n_in);
    for (int i = 0; i < n; i++)
        for (int k = 0; k < n_in; k++)
            xs[(size_t)i * n_in + k] = (feats[(size_t)i * n_in + k] - mean[k]) / scale[k];
    float *dp = nullptr, *dx = nullptr, *dy = nullptr;
    int rc = GBSP_OK;
    cudaError_t e = cudaMalloc((void**)&dp, params.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&dx, xs.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&dy, (size_t)n * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(dp, params.data(), params.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dx, xs.data(), xs.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_mlp_forward<<<forward_grid(n), H>>>(dp, n_in, dx, n, dy);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dy, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) rc = set_error(GBSP_ERR_CUDA, std::string("cost model inference: ") + cudaGetErrorString(e));
    cudaFree(dp);
    cudaFree(dx);
    cudaFree(dy);
    return rc;
}

}  // namespace gbsp

using gbsp::set_error;

extern "C" {

size_t gbsp_mlp_param_count(int n_in) { return gbsp::layout(n_in).total; }

size_t gbsp_mlp_work_floats(int n_in) { return (size_t)gbsp::BWD_GRID * (gbsp::layout(n_in).total + 1); }

int gbsp_mlp_forward(const float* d_params, int n_in, const float* d_x, int n, float* d_y, void* stream) {
    if (int rc = gbsp::check_n_in(n_in)) return rc;
    if (!d_params || !d_x || !d_y || n < 0) return set_error(GBSP_ERR_INVALID, "gbsp_mlp_forward: bad arguments");
    if (n == 0) return GBSP_OK;
    gbsp::k_mlp_forward<<<gbsp::forward_grid(n), gbsp::H, 0, (cudaStream_t)stream>>>(d_params, n_in, d_x, n, d_y);
    MLP_CUDA(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_mlp_backward(const float* d_params, int n_in, const float* d_x, const float* d_target, int n,
                      float* d_grad, float* d_loss, float* d_work, void* stream) {
    if (int rc = gbsp::check_n_in(n_in)) return rc;
    if (!d_params || !d_x || !d_target || !d_grad || !d_loss || !d_work || n < 1)
        return set_error(GBSP_ERR_INVALID, "gbsp_mlp_backward: bad arguments");
    const cudaStream_t st = (cudaStream_t)stream;
    const size_t total = gbsp::layout(n_in).total;
    gbsp::k_mlp_backward<<<gbsp::BWD_GRID, gbsp::H, 0, st>>>(d_params, n_in, d_x, d_target, n, d_work);
    MLP_CUDA(cudaGetLastError());
    gbsp::k_mlp_reduce<<<(unsigned)((total + 1 + 255) / 256), 256, 0, st>>>(d_work, gbsp::BWD_GRID, total, d_grad,
                                                                           d_loss);
    MLP_CUDA(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_mlp_adam(float* d_params, const float* d_grad, float* d_m, float* d_v, size_t n_params, float lr,
                  float beta1, float beta2, float eps, int step, void* stream) {
    if (!d_params || !d_grad || !d_m || !d_v || step < 1 || n_params == 0)
        return set_error(GBSP_ERR_INVALID, "gbsp_mlp_adam: bad arguments");
    const float c1 = 1.f - std::pow(beta1, (float)step), c2 = 1.f - std::pow(beta2, (float)step);
    gbsp::k_mlp_adam<<<(unsigned)((n_params + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        d_params, d_grad, d_m, d_v, n_params, lr, beta1, beta2, eps, c1, c2);
    MLP_CUDA(cudaGetLastError());
    return GBSP_OK;
}

int gbsp_cost_model_set(const float* params, int n_in, const float* feat_mean, const float* feat_scale) {
    if (n_in != GBSP_N_FEATURES || !params || !feat_mean || !feat_scale)
        return set_error(GBSP_ERR_INVALID, "gbsp_cost_model_set: n_in must be GBSP_N_FEATURES and arrays non-null");
    for (int k = 0; k < n_in; k++)
        if (!(feat_scale[k] > 0.f)) return set_error(GBSP_ERR_INVALID, "gbsp_cost_model_set: feat_scale must be > 0");
    std::lock_guard<std::mutex> lk(gbsp::g_model_mu);
    gbsp::g_params.assign(params, params + gbsp::layout(n_in).total);
    gbsp::g_mean.assign(feat_mean, feat_mean + n_in);
    gbsp::g_scale.assign(feat_scale, feat_scale + n_in);
    gbsp::g_lo.clear();  // a new model's domain comes with it
    gbsp::g_hi.clear();
    gbsp::g_n_in = n_in;
    return GBSP_OK;
}

int gbsp_cost_model_set_domain(int n_in, const float* feat_lo, const float* feat_hi) {
    std::lock_guard<std::mutex> lk(gbsp::g_model_mu);
    if (!feat_lo && !feat_hi) {
        gbsp::g_lo.clear();
        gbsp::g_hi.clear();
        return GBSP_OK;
    }
    if (gbsp::g_params.empty() || n_in != gbsp::g_n_in || !feat_lo || !feat_hi)
        return set_error(GBSP_ERR_INVALID, "gbsp_cost_model_set_domain: install the model first; n_in must match");
    for (int k = 0; k < n_in; k++)
        if (!(feat_lo[k] <= feat_hi[k]))
            return set_error(GBSP_ERR_INVALID, "gbsp_cost_model_set_domain: feat_lo must be <= feat_hi");
    gbsp::g_lo.assign(feat_lo, feat_lo + n_in);
    gbsp::g_hi.assign(feat_hi, feat_hi + n_in);
    return GBSP_OK;
}

}  // extern "C"
