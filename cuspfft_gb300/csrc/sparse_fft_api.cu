// sparse_fft_api.cu -- the reference-compatible C++ API (include/sparse_fft.h,
// include/mtx_reader.h, include/sparse_fft_csc.h) over the C ABI.
//
// Status codes become std::runtime_error here, as the reference's
// CUDA_CHECK does (include/sparse_fft_internal.cuh:16-22), so callers
// written against the reference (try / catch / cudaGetLastError) behave the
// same way.  Every device buffer is owned by an RAII holder, so a throw
// leaks nothing (the reference leaks on throw).
#include <algorithm>

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "gbspfft.h"
#include "sparse_fft.h"
#include "sparse_fft_csc.h"

namespace {

std::string last_error() {
    char buf[512];
    gbsp_last_error(buf, sizeof(buf));
    return std::string(buf);
}

void check(int status, const char* what) {
    if (status != GBSP_OK)
        throw std::runtime_error(std::string(what) + ": " + gbsp_status_string(status) + ": " +
                                 last_error());
}

void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error: ") + what + ": " +
                                                   cudaGetErrorString(e));
}

struct PlanHolder {
    gbsp_plan_t p = nullptr;
    ~PlanHolder() { if (p) gbsp_plan_destroy(p); }
};
struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    void* release() { void* r = p; p = nullptr; return r; }
};
struct Events {
    cudaEvent_t a = nullptr, b = nullptr;
    Events() {
        cuda_check(cudaEventCreate(&a), "cudaEventCreate");
        cuda_check(cudaEventCreate(&b), "cudaEventCreate");
    }
    ~Events() { cudaEventDestroy(a); cudaEventDestroy(b); }
};
struct StreamHolder {
    cudaStream_t s = nullptr;
    ~StreamHolder() { if (s) cudaStreamDestroy(s); }
};
struct GraphHolder {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t e = nullptr;
    ~GraphHolder() {
        if (e) cudaGraphExecDestroy(e);
        if (g) cudaGraphDestroy(g);
    }
};

// The reference's memory metric (DeviceMemPeak, src/sparse_fft_bluestein.cu:7-20)
// is the cudaMemGetInfo delta at the end of the call: every buffer the call
// still holds then (tables, scratch, output).  Here those are the plan's
// device memory and the output, counted directly: a cudaMemGetInfo delta
// cannot see plan memory that the library's pool hands out again, so from
// the second call on it would report little more than the output.
size_t working_set(gbsp_plan_t p, size_t out_bytes) {
    gbsp_plan_info info;
    check(gbsp_plan_get_info(p, &info), "gbsp_plan_get_info");
    return info.device_bytes + out_bytes;
}

// Reads and clears the plan's device error word once the call's work is
// done (outside the timed region) and throws if a kernel reported one, as
// the reference throws on a CUDA failure (include/sparse_fft_internal.cuh:16-22).
void check_device_flags(gbsp_plan_t p, const char* who) {
    int flags = 0;
    check(gbsp_plan_error_flags(p, &flags), "gbsp_plan_error_flags");
    check(gbsp_device_flags_status(flags), who);
}

// stream_tile > 0 reserves the streaming slabs (and copy stream) with the
// plan, outside the timed transform
void make_plan(const COOMatrix& coo, int u_tile, int policy, PlanHolder& ph, gbsp_plan_info& info,
               int stream_tile = 0) {
    if (u_tile <= 0) throw std::runtime_error("CSC tile size must be positive");
    CompactCSC csc = make_compact_csc(coo);
    gbsp_options o = {};
    o.length_policy = policy;
    o.u_tile = u_tile;
    o.stream_tile_rows = stream_tile;
    check(gbsp_plan_create(coo.rows, coo.cols, csc.n_sparse_cols, coo.nnz, csc.col_ptr.data(),
                           csc.row_idx.data(), csc.sparse_cols.data(), &o, nullptr, &ph.p),
          "gbsp_plan_create");
    check(gbsp_plan_get_info(ph.p, &info), "gbsp_plan_get_info");
}

SparseFFTResult run_method(const COOMatrix& coo, int u_tile, int policy) {
    PlanHolder ph;
    gbsp_plan_info info;
    make_plan(coo, u_tile, policy, ph, info);
    DevBuf out;
    cuda_check(cudaMalloc(&out.p, (size_t)coo.rows * info.output_pitch * sizeof(cuFloatComplex)),
               "cudaMalloc(d_output)");
    cuda_check(cudaDeviceSynchronize(), "setup");
    Events ev;
    cuda_check(cudaEventRecord(ev.a, nullptr), "cudaEventRecord");
    check(gbsp_execute(ph.p, out.p, (size_t)info.output_pitch, nullptr), "gbsp_execute");
    cuda_check(cudaEventRecord(ev.b, nullptr), "cudaEventRecord");
    cuda_check(cudaEventSynchronize(ev.b), "cudaEventSynchronize");
    float ms = 0.f;
    cuda_check(cudaEventElapsedTime(&ms, ev.a, ev.b), "cudaEventElapsedTime");
    check_device_flags(ph.p, "gbsp_execute");
    SparseFFTResult r;
    r.mem_bytes = working_set(ph.p, (size_t)coo.rows * info.output_pitch * sizeof(cuFloatComplex));
    r.output_cols = info.output_pitch;
    r.ms = ms;
    r.d_output = (cuFloatComplex*)out.release();
    return r;
}

SparseFFTResult run_graph(const COOMatrix& coo, int u_tile, int policy) {
    PlanHolder ph;
    gbsp_plan_info info;
    make_plan(coo, u_tile, policy, ph, info);
    DevBuf out;
    cuda_check(cudaMalloc(&out.p, (size_t)coo.rows * info.output_pitch * sizeof(cuFloatComplex)),
               "cudaMalloc(d_output)");
    cuda_check(cudaDeviceSynchronize(), "setup");
    StreamHolder sh;
    cuda_check(cudaStreamCreateWithFlags(&sh.s, cudaStreamNonBlocking), "cudaStreamCreate");
    GraphHolder gh;
    cuda_check(cudaStreamBeginCapture(sh.s, cudaStreamCaptureModeThreadLocal), "BeginCapture");
    int st = gbsp_execute(ph.p, out.p, (size_t)info.output_pitch, sh.s);
    cudaError_t ce = cudaStreamEndCapture(sh.s, &gh.g);
    check(st, "gbsp_execute (capture)");
    cuda_check(ce, "cudaStreamEndCapture");
    cuda_check(cudaGraphInstantiate(&gh.e, gh.g, 0), "cudaGraphInstantiate");
    Events ev;
    cuda_check(cudaEventRecord(ev.a, sh.s), "cudaEventRecord");
    cuda_check(cudaGraphLaunch(gh.e, sh.s), "cudaGraphLaunch");
    cuda_check(cudaEventRecord(ev.b, sh.s), "cudaEventRecord");
    cuda_check(cudaEventSynchronize(ev.b), "cudaEventSynchronize");
    float ms = 0.f;
    cuda_check(cudaEventElapsedTime(&ms, ev.a, ev.b), "cudaEventElapsedTime");
    check_device_flags(ph.p, "graph replay");
    SparseFFTResult r;
    r.mem_bytes = working_set(ph.p, (size_t)coo.rows * info.output_pitch * sizeof(cuFloatComplex));
    r.output_cols = info.output_pitch;
    r.ms = ms;
    r.d_output = (cuFloatComplex*)out.release();
    return r;
}

struct PinnedBuf {
    void* p = nullptr;
    ~PinnedBuf() {
        if (p) cudaFreeHost(p);
    }
};

// Streaming form: the spectrum goes tile by tile into pinned host memory and
// is returned in h_output with d_output = nullptr, as the reference's
// streaming methods do (src/sparse_fft_bluestein.cu:1276-1296).
SparseFFTResult run_streaming(const COOMatrix& coo, int u_tile, int policy) {
    PlanHolder ph;
    gbsp_plan_info info;
    make_plan(coo, u_tile, policy, ph, info, u_tile);
    const size_t n = (size_t)coo.rows * info.output_pitch;
    PinnedBuf host;
    cuda_check(cudaMallocHost(&host.p, std::max<size_t>(n, 1) * sizeof(cuFloatComplex)), "cudaMallocHost");
    cuda_check(cudaDeviceSynchronize(), "setup");
    Events ev;
    cuda_check(cudaEventRecord(ev.a, nullptr), "cudaEventRecord");
    check(gbsp_execute_to_host(ph.p, host.p, (size_t)info.output_pitch, u_tile, nullptr), "gbsp_execute_to_host");
    cuda_check(cudaEventRecord(ev.b, nullptr), "cudaEventRecord");
    cuda_check(cudaEventSynchronize(ev.b), "cudaEventSynchronize");
    float ms = 0.f;
    cuda_check(cudaEventElapsedTime(&ms, ev.a, ev.b), "cudaEventElapsedTime");
    SparseFFTResult r;
    r.mem_bytes = working_set(ph.p, 0);  // the spectrum is in host memory
    r.output_cols = info.output_pitch;
    r.ms = ms;
    r.d_output = nullptr;
    const cuFloatComplex* h = static_cast<const cuFloatComplex*>(host.p);
    r.h_output.assign(h, h + n);
    return r;
}

}  // namespace

// ---- mtx_reader.h ----------------------------------------------------------
COOMatrix read_mtx(const std::string& path) {
    int rows = 0, cols = 0, nnz = 0;
    int *ri = nullptr, *ci = nullptr;
    int st = gbsp_read_mtx(path.c_str(), &rows, &cols, &nnz, &ri, &ci);
    if (st != GBSP_OK) throw std::runtime_error(last_error());
    COOMatrix coo;
    coo.rows = rows;
    coo.cols = cols;
    coo.nnz = nnz;
    coo.row_idx.assign(ri, ri + nnz);
    coo.col_idx.assign(ci, ci + nnz);
    gbsp_free(ri);
    gbsp_free(ci);
    return coo;
}

CSRMatrix coo_to_csr(const COOMatrix& coo) {
    CSRMatrix csr;
    csr.rows = coo.rows;
    csr.cols = coo.cols;
    csr.nnz = coo.nnz;
    csr.col_idx = coo.col_idx;
    csr.row_ptr.assign(coo.rows + 1, 0);
    for (int i = 0; i < coo.nnz; i++) csr.row_ptr[coo.row_idx[i] + 1]++;
    for (int r = 0; r < coo.rows; r++) csr.row_ptr[r + 1] += csr.row_ptr[r];
    return csr;
}

// ---- sparse_fft_csc.h --------------------------------------------------------
CompactCSC make_compact_csc(const COOMatrix& coo) {
    CompactCSC csc;
    std::vector<int> sc(std::max(coo.cols, 1)), cp(coo.cols + 1), ri(std::max(coo.nnz, 1));
    int na = 0;
    check(gbsp_build_compact_csc(coo.rows, coo.cols, coo.nnz, coo.row_idx.data(), coo.col_idx.data(),
                                 &na, sc.data(), cp.data(), ri.data()),
          "make_compact_csc");
    csc.n_sparse_cols = na;
    csc.sparse_cols.assign(sc.begin(), sc.begin() + na);
    csc.col_ptr.assign(cp.begin(), cp.begin() + na + 1);
    csc.row_idx.assign(ri.begin(), ri.begin() + coo.nnz);
    return csc;
}

// ---- sparse_fft.h ----------------------------------------------------------
SparseFFTResult sparse_fft_csc_bluestein_mixed_radix(const COOMatrix& coo, int u_tile) {
    return run_method(coo, u_tile, GBSP_LEN_3SMOOTH);
}
SparseFFTResult sparse_fft_csc_bluestein_mixed_radix_graph(const COOMatrix& coo, int u_tile) {
    return run_graph(coo, u_tile, GBSP_LEN_3SMOOTH);
}
SparseFFTResult sparse_fft_csc_bluestein_cufft_smooth(const COOMatrix& coo, int u_tile) {
    return run_method(coo, u_tile, GBSP_LEN_7SMOOTH);
}

// The reference's power-of-two methods (fft_len = next_power_of_two(2 cols - 1),
// src/sparse_fft_bluestein.cu:687, 918, 1160, 1500, 1767).  use_stockham and
// fft_backend only pick the reference's FFT implementation (Stockham loop,
// shared-memory Stockham, cuFFT); the byte-mask LUT methods differ from it
// only in how pass 1 forms the twiddle sums.  Every one computes the same
// spectrum, here with the sm_103a kernels at the method's own length.
SparseFFTResult sparse_fft_csc_bluestein(const COOMatrix& coo, int u_tile, bool, int) {
    return run_method(coo, u_tile, GBSP_LEN_POW2);
}
SparseFFTResult sparse_fft_csc_bluestein_smem(const COOMatrix& coo, int u_tile) {
    return run_method(coo, u_tile, GBSP_LEN_POW2);
}
SparseFFTResult sparse_fft_csc_bluestein_cufft(const COOMatrix& coo, int u_tile) {
    return run_method(coo, u_tile, GBSP_LEN_POW2);
}
// Streaming methods: output to pinned host memory, returned in h_output.
SparseFFTResult sparse_fft_csc_stockham_streaming(const COOMatrix& coo, int u_tile, int) {
    return run_streaming(coo, u_tile, GBSP_LEN_POW2);
}
SparseFFTResult sparse_fft_csc_bluestein_cufft_streaming(const COOMatrix& coo, int u_tile) {
    return run_streaming(coo, u_tile, GBSP_LEN_POW2);
}
SparseFFTResult sparse_fft_csc_stockham_graph(const COOMatrix& coo, int u_tile) {
    return run_streaming(coo, u_tile, GBSP_LEN_POW2);
}
SparseFFTResult sparse_fft_csc_bluestein_binary_lut(const COOMatrix& coo, int u_tile) {
    return run_streaming(coo, u_tile, GBSP_LEN_POW2);
}
SparseFFTResult sparse_fft_csc_stockham_binary_smem(const COOMatrix& coo, int u_tile) {
    return run_method(coo, u_tile, GBSP_LEN_POW2);
}
