// ref_gpu_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Runs the reference's own GPU kernels for its two hot methods on this GPU,
// so the library's spectra can be checked against the reference's real GPU
// output (and the reference's GPU time measured on the same device):
//
//   method 3: sparse_fft_csc_bluestein_mixed_radix  src/sparse_fft_bluestein.cu:2256-2392
//   method 7: sparse_fft_csc_bluestein_cufft_smooth src/sparse_fft_bluestein.cu:2557-2719
//
// The kernels come from oracle/_ref/ref_kernels.fatbin, which
// oracle/build_ref.sh compiles for sm_103a from the reference's own
// src/sparse_fft_bluestein.cu (device code only, so the file runs on a GPU
// host of any CPU architecture).  They are looked up by name in the loaded
// module and launched through the CUDA driver API.  This file restates only
// the host orchestration around them, step for step:
//   CSC upload (u16 indices when can_pack_u16), chirp upload, FFT(b) by the
//   method's own FFT (run_fft_mixed_23 :2215-2254 or one cuFFT C2C plan),
//   then per tile of u_tile output rows: memset of the signal tile (:2330),
//   pass 1 (csc_build_bluestein_input[_packed]_kernel, grid n_sp x
//   ceil(tile/128), block 128), forward FFT, pointwise_mul_batched_kernel,
//   inverse FFT (+ scale_complex_kernel by 1/fft_len), and
//   bluestein_finalize_kernel (block 32 x 8).
// The host-side inputs (compact CSC, chirp and b tables, radix list) are
// passed in by the caller; oracle/ref_port.py restates the reference's host
// functions for them and is pinned bit for bit to the reference's compiled
// host code.
//
// cuFFT is called here because the reference's second method calls it; the
// library itself never does.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;

struct Kernels {
    CUmodule mod = nullptr;
    CUfunction build = nullptr, build_packed = nullptr, radix2 = nullptr, radix3 = nullptr, radix9 = nullptr,
               scale = nullptr, pointwise = nullptr, finalize = nullptr;
} g_k;

constexpr int CSC_BU = 128;  // include/sparse_fft_internal.cuh:73

#define DRV(x)                                                                              \
    do {                                                                                    \
        CUresult r_ = (x);                                                                  \
        if (r_ != CUDA_SUCCESS) {                                                           \
            const char* s_ = nullptr;                                                       \
            cuGetErrorString(r_, &s_);                                                      \
            g_err = std::string(#x) + ": " + (s_ ? s_ : "?");                               \
            throw 1;                                                                        \
        }                                                                                   \
    } while (0)
#define RT(x)                                                                               \
    do {                                                                                    \
        cudaError_t e_ = (x);                                                               \
        if (e_ != cudaSuccess) {                                                            \
            g_err = std::string(#x) + ": " + cudaGetErrorString(e_);                        \
            throw 1;                                                                        \
        }                                                                                   \
    } while (0)
#define FFTCHK(x)                                                                           \
    do {                                                                                    \
        cufftResult c_ = (x);                                                               \
        if (c_ != CUFFT_SUCCESS) {                                                          \
            g_err = std::string(#x) + ": cufft error " + std::to_string((int)c_);           \
            throw 1;                                                                        \
        }                                                                                   \
    } while (0)

// Itanium-mangled names of free functions start with _Z<length><name>
bool name_is(const char* mangled, const char* plain) {
    const std::string pre = "_Z" + std::to_string(std::strlen(plain)) + plain;
    return std::strncmp(mangled, pre.c_str(), pre.size()) == 0;
}

void launch(CUfunction f, dim3 grid, dim3 block, void** args) {
    DRV(cuLaunchKernel(f, grid.x, grid.y, grid.z, block.x, block.y, block.z, 0, nullptr, args, nullptr));
}

template <typename T>
struct DevArr {
    T* p = nullptr;
    explicit DevArr(size_t n) { RT(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T))); }
    ~DevArr() { cudaFree(p); }
};

// run_fft_mixed_23 (src/sparse_fft_bluestein.cu:2215-2254): one launch per
// radix (9, 3, 2), out of place, ping-pong; inverse scaled by 1/n
float2* fft_mixed_23(float2* d_in, float2* d_tmp, int n, const std::vector<int>& factors, int batch, bool inverse) {
    float2* src = d_in;
    float2* dst = d_tmp;
    int l = 1;
    int inv = inverse ? 1 : 0;
    for (int radix : factors) {
        int m = n / (l * radix);
        const int total = (n / radix) * batch;
        const unsigned blocks = (unsigned)((total + 255) / 256);
        CUfunction f = radix == 2 ? g_k.radix2 : radix == 3 ? g_k.radix3 : radix == 9 ? g_k.radix9 : nullptr;
        if (!f) {
            g_err = "unsupported radix";
            throw 1;
        }
        void* args[] = {&src, &dst, &n, &l, &m, &batch, &inv};
        launch(f, dim3(blocks), dim3(256), args);
        l *= radix;
        std::swap(src, dst);
    }
    if (inverse) {
        int total = n * batch;
        float scale = 1.f / (float)n;
        void* args[] = {&src, &total, &scale};
        launch(g_k.scale, dim3((unsigned)((total + 255) / 256)), dim3(256), args);
    }
    return src;
}

}  // namespace

extern "C" {

const char* refgpu_last_error() { return g_err.c_str(); }

// Loads the fatbin and resolves the reference's kernels.  Returns 0 on success.
int refgpu_init(const char* fatbin_path) {
    try {
        if (g_k.mod) return 0;
        RT(cudaFree(nullptr));  // primary context current
        std::FILE* f = std::fopen(fatbin_path, "rb");
        if (!f) {
            g_err = std::string("cannot open ") + fatbin_path;
            return 1;
        }
        std::vector<char> image;
        char buf[1 << 16];
        size_t n;
        while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) image.insert(image.end(), buf, buf + n);
        std::fclose(f);
        DRV(cuModuleLoadData(&g_k.mod, image.data()));
        unsigned count = 0;
        DRV(cuModuleGetFunctionCount(&count, g_k.mod));
        std::vector<CUfunction> fs(count);
        DRV(cuModuleEnumerateFunctions(fs.data(), count, g_k.mod));
        for (CUfunction fn : fs) {
            const char* nm = nullptr;
            DRV(cuFuncGetName(&nm, fn));
            if (!nm) continue;
            if (name_is(nm, "csc_build_bluestein_input_kernel")) g_k.build = fn;
            else if (name_is(nm, "csc_build_bluestein_input_packed_kernel")) g_k.build_packed = fn;
            else if (name_is(nm, "stockham_stage_kernel")) g_k.radix2 = fn;
            else if (name_is(nm, "stockham_radix3_stage_kernel")) g_k.radix3 = fn;
            else if (name_is(nm, "stockham_radix9_stage_kernel")) g_k.radix9 = fn;
            else if (name_is(nm, "scale_complex_kernel")) g_k.scale = fn;
            else if (name_is(nm, "pointwise_mul_batched_kernel")) g_k.pointwise = fn;
            else if (name_is(nm, "bluestein_finalize_kernel")) g_k.finalize = fn;
        }
        if (!g_k.build || !g_k.build_packed || !g_k.radix2 || !g_k.radix3 || !g_k.radix9 || !g_k.scale ||
            !g_k.pointwise || !g_k.finalize) {
            g_err = "a reference kernel is missing from the fatbin";
            return 1;
        }
        return 0;
    } catch (int) {
        return 1;
    }
}

// One call of the reference method (3: mixed radix, 7: cuFFT smooth) on a
// compact CSC.  chirp: cols (re, im) pairs; b: fft_len pairs (the reference's
// make_bluestein_b); factors: factor_3_smooth(fft_len) for method 3.  Runs
// the timed tile loop 1 + n_times times (the first is a warm-up) and stores
// each timed loop's milliseconds (CUDA events, as the reference times it) in
// times[]; the spectrum of the last loop goes to h_out (rows x stride
// complex64; pad columns zero).
int refgpu_run(int method, int rows, int cols, int n_sp, const int* col_ptr, const int* row_idx,
               const int* sparse_cols, const float* chirp, const float* b, int fft_len, const int* factors,
               int n_factors, int u_tile, float* h_out, int stride, int n_times, float* times) {
    cufftHandle plan_b = 0, plan_full = 0, plan_last = 0;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    int status = 1;
    try {
        if (!g_k.mod) {
            g_err = "refgpu_init was not called";
            return 1;
        }
        if (u_tile <= 0 || n_sp <= 0 || (method != 3 && method != 7)) {
            g_err = "bad arguments";
            return 1;
        }
        const int output_cols = cols / 2 + 1;
        const int nnz = col_ptr[n_sp];
        const bool packed = rows <= 65536 && cols <= 65536;  // can_pack_u16
        DevArr<int> d_col_ptr(n_sp + 1);
        RT(cudaMemcpy(d_col_ptr.p, col_ptr, (n_sp + 1) * sizeof(int), cudaMemcpyHostToDevice));
        DevArr<uint16_t> d_ri16(packed ? nnz : 1), d_sc16(packed ? n_sp : 1);
        DevArr<int> d_ri(packed ? 1 : nnz), d_sc(packed ? 1 : n_sp);
        if (packed) {
            std::vector<uint16_t> ri(row_idx, row_idx + nnz), sc(sparse_cols, sparse_cols + n_sp);
            RT(cudaMemcpy(d_ri16.p, ri.data(), nnz * sizeof(uint16_t), cudaMemcpyHostToDevice));
            RT(cudaMemcpy(d_sc16.p, sc.data(), n_sp * sizeof(uint16_t), cudaMemcpyHostToDevice));
        } else {
            RT(cudaMemcpy(d_ri.p, row_idx, (size_t)nnz * sizeof(int), cudaMemcpyHostToDevice));
            RT(cudaMemcpy(d_sc.p, sparse_cols, (size_t)n_sp * sizeof(int), cudaMemcpyHostToDevice));
        }
        DevArr<float2> d_chirp(cols), d_b_fft(fft_len);
        RT(cudaMemcpy(d_chirp.p, chirp, (size_t)cols * sizeof(float2), cudaMemcpyHostToDevice));
        const int max_tile = std::min(u_tile, rows);
        DevArr<float2> d_signal((size_t)max_tile * fft_len);
        DevArr<float2> d_work(method == 3 ? (size_t)max_tile * fft_len : 1);
        DevArr<float2> d_out((size_t)rows * stride);
        RT(cudaMemset(d_out.p, 0, (size_t)rows * stride * sizeof(float2)));
        std::vector<int> fac(factors, factors + n_factors);
        if (method == 3) {
            RT(cudaMemcpy(d_signal.p, b, (size_t)fft_len * sizeof(float2), cudaMemcpyHostToDevice));
            float2* res = fft_mixed_23(d_signal.p, d_work.p, fft_len, fac, 1, false);
            RT(cudaMemcpy(d_b_fft.p, res, (size_t)fft_len * sizeof(float2), cudaMemcpyDeviceToDevice));
        } else {
            RT(cudaMemcpy(d_b_fft.p, b, (size_t)fft_len * sizeof(float2), cudaMemcpyHostToDevice));
            int fl = fft_len;
            FFTCHK(cufftPlanMany(&plan_b, 1, &fl, nullptr, 1, fft_len, nullptr, 1, fft_len, CUFFT_C2C, 1));
            FFTCHK(cufftExecC2C(plan_b, (cufftComplex*)d_b_fft.p, (cufftComplex*)d_b_fft.p, CUFFT_FORWARD));
            FFTCHK(cufftPlanMany(&plan_full, 1, &fl, nullptr, 1, fft_len, nullptr, 1, fft_len, CUFFT_C2C,
                                 max_tile));
            const int last = rows % u_tile;
            if (last != 0 && last != max_tile)
                FFTCHK(cufftPlanMany(&plan_last, 1, &fl, nullptr, 1, fft_len, nullptr, 1, fft_len, CUFFT_C2C,
                                     last));
        }
        RT(cudaDeviceSynchronize());
        RT(cudaEventCreate(&t0));
        RT(cudaEventCreate(&t1));
        for (int rep = 0; rep <= n_times; rep++) {
            RT(cudaEventRecord(t0));
            for (int u_base = 0; u_base < rows; u_base += u_tile) {
                int tile_rows = std::min(u_tile, rows - u_base);
                RT(cudaMemset(d_signal.p, 0, (size_t)tile_rows * fft_len * sizeof(float2)));
                int rws = rows, nsp = n_sp, fl = fft_len, ub = u_base;
                float inv_rows = 1.f / (float)rows;
                const void* cp = d_col_ptr.p;
                const void* ri = packed ? (const void*)d_ri16.p : (const void*)d_ri.p;
                const void* sc = packed ? (const void*)d_sc16.p : (const void*)d_sc.p;
                const void* ch = d_chirp.p;
                void* sig = d_signal.p;
                void* a1[] = {&cp, &ri, &sc, &ch, &sig, &rws, &nsp, &fl, &ub, &tile_rows, &inv_rows};
                launch(packed ? g_k.build_packed : g_k.build,
                       dim3((unsigned)n_sp, (unsigned)((tile_rows + CSC_BU - 1) / CSC_BU)), dim3(CSC_BU), a1);
                int total = tile_rows * fft_len;
                float2* conv = nullptr;
                if (method == 3) {
                    float2* fwd = fft_mixed_23(d_signal.p, d_work.p, fft_len, fac, tile_rows, false);
                    float2* other = (fwd == d_signal.p) ? d_work.p : d_signal.p;
                    const void* bf = d_b_fft.p;
                    void* a2[] = {&fwd, &bf, &fl, &tile_rows};
                    launch(g_k.pointwise, dim3((unsigned)((total + 255) / 256)), dim3(256), a2);
                    conv = fft_mixed_23(fwd, other, fft_len, fac, tile_rows, true);
                } else {
                    cufftHandle tp = (plan_last && tile_rows != max_tile) ? plan_last : plan_full;
                    FFTCHK(cufftExecC2C(tp, (cufftComplex*)d_signal.p, (cufftComplex*)d_signal.p, CUFFT_FORWARD));
                    const void* bf = d_b_fft.p;
                    void* a2[] = {&sig, &bf, &fl, &tile_rows};
                    launch(g_k.pointwise, dim3((unsigned)((total + 255) / 256)), dim3(256), a2);
                    FFTCHK(cufftExecC2C(tp, (cufftComplex*)d_signal.p, (cufftComplex*)d_signal.p, CUFFT_INVERSE));
                    float scale = 1.f / (float)fft_len;
                    void* a3[] = {&sig, &total, &scale};
                    launch(g_k.scale, dim3((unsigned)((total + 255) / 256)), dim3(256), a3);
                    conv = d_signal.p;
                }
                int oc = output_cols, os = stride;
                void* out = d_out.p;
                void* a4[] = {&conv, &ch, &out, &rws, &os, &oc, &fl, &ub, &tile_rows};
                launch(g_k.finalize, dim3((unsigned)((output_cols + 31) / 32), (unsigned)((tile_rows + 7) / 8)),
                       dim3(32, 8), a4);
            }
            RT(cudaDeviceSynchronize());
            RT(cudaEventRecord(t1));
            RT(cudaEventSynchronize(t1));
            float ms = 0.f;
            RT(cudaEventElapsedTime(&ms, t0, t1));
            if (rep > 0 && times) times[rep - 1] = ms;
        }
        RT(cudaMemcpy(h_out, d_out.p, (size_t)rows * stride * sizeof(float2), cudaMemcpyDeviceToHost));
        status = 0;
    } catch (int) {
        status = 1;
    }
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (plan_b) cufftDestroy(plan_b);
    if (plan_full) cufftDestroy(plan_full);
    if (plan_last) cufftDestroy(plan_last);
    return status;
}

}  // extern "C"
