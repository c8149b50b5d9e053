/*
 * gbspfft.h -- C ABI of the GB300-native binary-sparse 2-D R2C FFT.
 *
 * Plain pointers, sizes and int status codes only: no C++ types, no torch
 * types, no exceptions cross this boundary.  The C++ drop-in layer
 * (include/sparse_fft.h, include/mtx_reader.h) and the Python package are
 * both written on top of these entry points.
 *
 * What is computed (same as the reference's two hot methods,
 * src/sparse_fft_bluestein.cu:2256-2392 and :2557-2719):
 *   F[u][v] = sum over nonzeros (r,c) of exp(-2*pi*i*(r*u/rows + c*v/cols))
 * for u in [0,rows), v in [0, cols/2], written row-major as complex64
 * (interleaved float re, im) with a caller-chosen row pitch.
 *
 * All functions return GBSP_OK (0) on success or a positive GBSP_ERR_* code;
 * gbsp_last_error() returns a message for the calling thread's last failure.
 */
#ifndef GBSPFFT_H
#define GBSPFFT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    GBSP_OK = 0,
    GBSP_ERR_INVALID = 1,     /* bad argument (sizes, pointers, options)      */
    GBSP_ERR_CUDA = 2,        /* a CUDA runtime call or kernel launch failed  */
    GBSP_ERR_ALLOC = 3,       /* device or host allocation failed             */
    GBSP_ERR_UNSUPPORTED = 4, /* shape outside what this library handles      */
    GBSP_ERR_IO = 5,          /* file could not be opened / parsed            */
    GBSP_ERR_NOT_BUILT = 6    /* entry point exists for link compatibility only */
};

/* Length policy of the Bluestein convolution along the column axis.
 *   GBSP_LEN_3SMOOTH: fft_len = next 2^a*3^b >= 2*cols-1
 *                     (reference: next_3_smooth, src/sparse_fft_bluestein.cu:1975-1982,
 *                      used by sparse_fft_csc_bluestein_mixed_radix)
 *   GBSP_LEN_7SMOOTH: fft_len = next 2^a*3^b*5^c*7^d >= 2*cols-1
 *                     (reference: next_7_smooth, :1987-1994,
 *                      used by sparse_fft_csc_bluestein_cufft_smooth) */
/*   GBSP_LEN_POW2:    fft_len = next power of two >= 2*cols-1
 *                     (reference: next_power_of_two, include/sparse_fft_internal.cuh:153-157,
 *                      used by sparse_fft_csc_bluestein and its _smem / _cufft wrappers,
 *                      the streaming, graph and binary-LUT methods) */
enum { GBSP_LEN_POW2 = 2, GBSP_LEN_3SMOOTH = 3, GBSP_LEN_7SMOOTH = 7 };

/* How a plan picks its radices, row block and pass-1 shape when the options
 * leave them open.
 *   GBSP_PLANNER_MODEL:   analytic cost model (default)
 *   GBSP_PLANNER_LEARNED: the installed MLP cost model (gbsp_cost_model_set)
 *                         scores every tuning candidate and the cheapest
 *                         prediction is built.  The spectrum never depends
 *                         on the choice. */
enum { GBSP_PLANNER_MODEL = 0, GBSP_PLANNER_LEARNED = 1 };

/* Pass-1 shapes (gbsp_options.pass1_shape, 1-based):
 *   1: 256 rows x 32-column windows, full twiddle table
 *   2: 256 x 32, half table      3: 128 x 64, full    4: 256 x 16, full
 *   5: 256 x 16, half            6: 128 x 32, half
 *   7: 256 x 32, two-level       8: 128 x 32, two-level (tall matrices)
 * The automatic choice takes the first that fits of 1, 2, 7, 3, 4, 5, 6, 8
 * (measured on GB300); the tuner and the learned planner consider them all. */
#define GBSP_N_PASS1_SHAPES 8
/* Length of the cost-model feature vector (gbsp_plan_features). */
#define GBSP_N_FEATURES 36

/* gbsp_options.stream_tile_rows: reserve the streaming slabs for the tile
 * gbsp_execute_to_host picks when its tile_rows is 0. */
#define GBSP_STREAM_TILE_AUTO (-1)

typedef struct gbsp_plan_s* gbsp_plan_t;

/* Tuning knobs.  Zero-initialise and set what you need; 0 means "default".
 * None of them changes the computed spectrum beyond FP32 rounding. */
typedef struct {
    int length_policy;     /* GBSP_LEN_3SMOOTH (default), GBSP_LEN_7SMOOTH or GBSP_LEN_POW2 */
    int u_tile;            /* Bluestein rows per tile (each yields output rows u and
                              rows-u); the --csc-tile analogue. 0 = all rows in one tile */
    int kahan_min_degree;  /* columns with >= this many nonzeros accumulate with Kahan
                              compensation; 0 = default 64; negative = never (plain FP32) */
    int index_bytes;       /* 0 = auto (2 when rows,cols <= 65536, else 4), or 2 / 4      */
    int max_channel_len;   /* largest per-CTA FFT length held in shared memory;
                              0 = as long as shared memory allows (about 28k points);
                              longer convolutions split into channels (a thread-block
                              cluster, or one CTA running them in turn)                   */
    int rows_threads;      /* row-kernel block size: 0 = auto, else a multiple of 32
                              in [64, 1024] (at most 512 when a radix exceeds 16)         */
    int row_table_mode;    /* pass-1 twiddle table: 0 = auto, 1 = full circle,
                              2 = half circle, 3 = two-level (W^p = hi[p/256]*lo[p%256],
                              any row count)                                              */
    int radix[8];          /* channel FFT radix per stage, first to last, 0-terminated;
                              all zero = auto.  Allowed: 2 3 4 5 7 8 9 12 15 16 20 21
                              24 25 28 32 35 40; product = channel length                 */
    int pass1_shape;       /* 0 = auto, else 1..GBSP_N_PASS1_SHAPES (must fit)          */
    int planner;           /* GBSP_PLANNER_MODEL (0) or GBSP_PLANNER_LEARNED            */
    int channel_mode;      /* convolutions split into channels: 1 = one CTA per channel
                              in a thread-block cluster, 2 = one CTA runs the channels in
                              turn (results parked in an L2-resident scratch); 0 = auto
                              (2 with 512-thread row blocks, else 1)                      */
    int stream_tile_rows;  /* > 0: reserve the two streaming slabs for tiles of this many
                              Bluestein rows in the plan's own allocation
                              (gbsp_execute_to_host then allocates nothing);
                              GBSP_STREAM_TILE_AUTO: reserve them for the automatic tile */
    int exact_phases;      /* pass-1 twiddles: 0 = default, the entry of the FP64-built table
                              at the exact integer phase (u*r) mod rows every 4th row and
                              three-term-recurrence steps (two FMAs) between; 1 = the table
                              entry at the exact phase for every row (no float products
                              beyond the table's rounding; slower)                        */
    int force_bluestein;   /* 0 = default: when cols itself is smooth for the length
                              policy (3-smooth, 7-smooth or a power of two) and fits one
                              CTA, each row is one forward FFT of length cols (the same
                              DFT, a quarter of the work, fft_len = cols); 1 = always the
                              Bluestein convolution, as the reference computes it        */
} gbsp_options;

typedef struct {
    int rows, cols, nnz, n_active;
    int fft_len;           /* Bluestein convolution length L                              */
    int channels;          /* K: L = K * channel_len, one CTA per channel                 */
    int channel_len;       /* per-CTA FFT length held in shared memory                    */
    int n_stages;          /* radix stages of the channel FFT                             */
    int radix[16];         /* radix of each stage, first to last                          */
    int output_cols;       /* cols/2 + 1                                                  */
    int output_pitch;      /* row pitch (complex elements) the reference returns:
                              (cols/2+1) rounded up to a multiple of 4                    */
    int half_rows;         /* rows/2 + 1 Bluestein rows (Hermitian pairing)              */
    int u_tile;            /* effective Bluestein rows per tile                           */
    int index_bytes;       /* 2 or 4                                                      */
    int row_table_mode;    /* pass-1 table in shared memory: 0 full, 1 half, 2 two-level  */
    int rows_threads;      /* row-kernel block size in use                                */
    size_t device_bytes;   /* device memory held by the plan                              */
    int pass1_shape;       /* pass-1 shape in use (1-based)                               */
    int planner;           /* planner that chose the configuration (GBSP_PLANNER_MODEL
                              when a learned request fell outside the model's domain)     */
    int channel_mode;      /* 0 single channel, 1 clusters, 2 sequential channels         */
    int exact_phases;      /* 1: every pass-1 twiddle an exact table lookup               */
    int direct;            /* 1: one FFT of length cols per row instead of Bluestein       */
} gbsp_plan_info;

int         gbsp_version(void);
const char* gbsp_status_string(int status);
/* Copies the calling thread's last error message into buf (NUL-terminated). */
int         gbsp_last_error(char* buf, size_t buflen);

/* ---- host-side input path ------------------------------------------------
 * Binarizing Matrix Market reader.  Replaces read_mtx
 * (reference src/mtx_reader.cu:7-77, declared include/mtx_reader.h:18):
 * coordinate header, "symmetric" substring => mirror off-diagonal entries,
 * values ignored, 1-based -> 0-based, (row,col) pairs sorted and
 * de-duplicated.  *row_idx / *col_idx are allocated by the library and
 * released with gbsp_free(). */
int gbsp_read_mtx(const char* path, int* rows, int* cols, int* nnz,
                  int** row_idx, int** col_idx);
void gbsp_free(void* p);

/* Compact CSC over the active (non-empty) columns.  Replaces
 * make_compact_csc (reference include/sparse_fft_internal.cuh:193-222):
 * sparse_cols = sorted unique columns, col_ptr over active columns
 * (n_active+1 entries), row_idx a stable counting sort of the COO order.
 * Capacities: sparse_cols >= cols, col_ptr >= cols+1, row_idx_out >= nnz. */
int gbsp_build_compact_csc(int rows, int cols, int nnz,
                           const int* coo_row, const int* coo_col,
                           int* n_active, int* sparse_cols, int* col_ptr,
                           int* row_idx_out);

/* Length policy helpers (same results as the reference's next_3_smooth /
 * next_7_smooth, src/sparse_fft_bluestein.cu:1975-1994). */
int gbsp_next_smooth(int n, int policy);

/* ---- plans ---------------------------------------------------------------
 * Builds every device table once (row twiddles, chirp, filter spectrum, FFT
 * twiddles: FP64 on the GPU, rounded to FP32) and uploads the CSC.  Host
 * arrays in, device state out; this is the reference's untimed setup
 * (src/sparse_fft_bluestein.cu:2263-2321).  `stream` is a cudaStream_t
 * (NULL = legacy default stream).  Row indices are range-checked on the
 * device during the upload (GBSP_ERR_INVALID when one is outside [0, rows)).
 * The plan's device memory is one allocation from a stream-ordered pool
 * private to the library (see gbsp_set_memory_cache). */
int gbsp_plan_create(int rows, int cols, int n_active, int nnz,
                     const int* col_ptr, const int* row_idx, const int* sparse_cols,
                     const gbsp_options* opts, void* stream, gbsp_plan_t* plan);
int gbsp_plan_get_info(gbsp_plan_t plan, gbsp_plan_info* info);
/* Waits for the device (as cudaFree does) and returns the plan's memory to
 * the pool. */
int gbsp_plan_destroy(gbsp_plan_t plan);

/* Freed plan memory the library's pool keeps for later plans, per device
 * (default 1 GiB), on top of the memory of the plans alive: a cudaMalloc and
 * a cudaFree of a plan's allocation cost ~0.1 ms each, a pooled one a few
 * microseconds.  Free memory above the limit goes back to the CUDA driver
 * at the next synchronisation; 0 keeps nothing.  Takes effect at once (trims
 * the pools to the live plans plus the new limit). */
int gbsp_set_memory_cache(size_t bytes);

/* Runs the transform: the reference's timed tile loop
 * (src/sparse_fft_bluestein.cu:2327-2370).  d_out is device memory of at
 * least rows*out_pitch complex64, 16-byte aligned; out_pitch >= cols/2+1 and
 * even.  Columns [cols/2+1, out_pitch) are written as zeros.  Asynchronous
 * on `stream`. */
int gbsp_execute(gbsp_plan_t plan, void* d_out, size_t out_pitch, void* stream);

/* Same work as gbsp_execute, with CUDA events recorded around each phase on
 * `stream`; blocks until the transform is done and returns the device time
 * of each phase summed over tiles (milliseconds).  This is the reference's
 * CUSPFFT_BREAKDOWN per-phase timing (src/sparse_fft_bluestein.cu:1752-1760,
 * 1844-1950), exposed for every method. */
int gbsp_execute_profiled(gbsp_plan_t plan, void* d_out, size_t out_pitch, void* stream,
                          float* ms_pass1, float* ms_rows);

/* The pass-1 intermediate for inspection and tests: for rows
 * u in [u0, u0+n_rows) (u0+n_rows <= rows) writes
 *   S[u-u0][c] = sum over nonzero rows r of column c of exp(-2*pi*i*u*r/rows)
 * for every column c < cols (zero for empty columns) to d_s (complex64, row
 * pitch s_pitch >= cols rounded up to even; one extra zero column when cols
 * is odd).  This is the reference's csc_build_bluestein_input_*kernel
 * (src/sparse_fft_bluestein.cu:334-397) before its chirp multiply. */
int gbsp_column_sums(gbsp_plan_t plan, int u0, int n_rows, void* d_s, size_t s_pitch,
                     void* stream);

/* Allocation-free variant of gbsp_execute (this entry point has no
 * counterpart in the reference).  For callers that must not allocate device
 * memory while they run transforms -- device memory owned by a pool with a
 * hard budget, or latency-critical code that cannot afford cudaMalloc's
 * implicit synchronisation: it computes the same result as gbsp_execute, but
 * the pass-1 intermediate lives in a fixed 32 MiB array inside the library
 * (held by every GPU that loads the library until the process exits) and no
 * allocating routine is called.
 *   - The plan's device must be current.  The first call on each device looks
 *     up the array's device address and keeps it; make that first call before
 *     any stream capture.  The address belongs to the device's context:
 *     resetting the device (cudaDeviceReset) after that first call is not
 *     supported.
 *   - Rows of the intermediate are processed in tiles that fit the array; a
 *     plan whose single row would not fit is rejected with
 *     GBSP_ERR_UNSUPPORTED (cannot happen for plans gbsp_plan_create accepts
 *     today: a row is at most a few hundred KB).
 *   - All calls share the array and nothing in it has to start at zero (each
 *     tile is fully rewritten before it is read).  Calls that overlap on the
 *     GPU race on it: issue them on one stream, or order their streams with
 *     events -- calls made one after another on the host but on different
 *     streams still overlap on the GPU.
 * Asynchronous on `stream`, like gbsp_execute; read gbsp_plan_error_flags
 * once the work has finished. */
int gbsp_execute_noalloc(gbsp_plan_t plan, void* d_out, size_t out_pitch, void* stream);

/* Streams the transform to host memory: the reference's streaming methods
 * (sparse_fft_csc_stockham_streaming / _cufft_streaming,
 * src/sparse_fft_bluestein.cu:912-1145, 1150-1296), for outputs larger than
 * device memory.  Tiles of tile_rows Bluestein rows (at most the plan's
 * u_tile; 0 = automatic: about a ninth of the rows, rounded to a multiple of
 * the SM count, so the first tile's compute -- the part the copies cannot
 * hide -- stays short while every row-kernel wave is full) are computed into one of two device slabs holding the
 * tile's output rows u and rows-u while the other slab is copied to h_out on
 * a second stream.  h_out: rows * out_pitch complex64 (pinned memory lets
 * the copies overlap); columns [cols/2+1, out_pitch) are written as zeros.
 * Extra device memory: 2 slabs of 2 * tile * out_pitch complex64, kept with
 * the plan (with a copy stream) for later calls.  Blocks until the whole
 * spectrum is in h_out; serialise calls on one plan. */
int gbsp_execute_to_host(gbsp_plan_t plan, void* h_out, size_t out_pitch, int tile_rows, void* stream);

/* Reads and clears the plan's device error flags (synchronises the device).
 * Bit 0: a bounded wait inside a kernel gave up; bit 1: a stage radix the
 * row kernel was not compiled for (plan/kernel mismatch).  Either way the
 * result of that transform is not valid.  0 means no error was recorded.
 * The asynchronous entry points (gbsp_execute, gbsp_execute_noalloc,
 * gbsp_batch_execute, gbsp_batch_graph_launch) cannot see the word without
 * synchronising, so callers read it here once their work has finished; the
 * blocking ones (gbsp_execute_to_host, gbsp_execute_profiled) and the C++
 * API of include/sparse_fft.h check it themselves. */
int gbsp_plan_error_flags(gbsp_plan_t plan, int* flags);

/* Status of a device error word as gbsp_plan_error_flags returns it:
 * GBSP_OK for 0, else GBSP_ERR_CUDA with gbsp_last_error() naming the bits.
 * (The reference raises every CUDA failure as an exception,
 * include/sparse_fft_internal.cuh:16-22; its C++ API here throws on this
 * status.)  Host-only. */
int gbsp_device_flags_status(int flags);

/* ---- batches ---------------------------------------------------------------
 * Many matrices of uneven size and sparsity transformed by one persistent
 * launch per pass, with work handed out by device queues: the GPU form of
 * the reference's driver, which transforms one matrix per process
 * (src/main.cu:249-311).  The reference has no batch entry point.
 *
 * gbsp_batch_create builds one sub-plan per matrix (same tables as
 * gbsp_plan_create, with one pass-1 shape common to the batch; opts'
 * u_tile, rows_threads and radix are ignored: each matrix gets the
 * planner's automatic radices and row block).  Pass 1 of all matrices is one
 * launch; the Bluestein rows are one launch per class of matrices sharing a
 * block size and CTAs-per-SM count.  Matrices whose convolution needs
 * several channels (thread-block clusters) run after the batched launches
 * through their own sub-plan.  Outputs are bound once with
 * gbsp_batch_set_outputs (same rules as gbsp_execute's d_out / out_pitch);
 * gbsp_batch_execute then enqueues the whole batch on `stream`.
 * gbsp_batch_graph_launch does the same through a CUDA graph captured on
 * its first call (and again after gbsp_batch_set_outputs).  Each output is
 * identical to what gbsp_execute writes for the same matrix and options. */
typedef struct gbsp_batch_s* gbsp_batch_t;

typedef struct {
    int rows, cols, n_active, nnz;
    const int* col_ptr;      /* compact CSC as for gbsp_plan_create (host memory) */
    const int* row_idx;
    const int* sparse_cols;
} gbsp_matrix;

int gbsp_batch_create(int count, const gbsp_matrix* mats, const gbsp_options* opts, void* stream,
                      gbsp_batch_t* batch);
int gbsp_batch_set_outputs(gbsp_batch_t batch, void* const* d_outs, const size_t* out_pitches);
int gbsp_batch_execute(gbsp_batch_t batch, void* stream);
int gbsp_batch_graph_launch(gbsp_batch_t batch, void* stream);
/* Plan details of matrix i (0-based, creation order). */
int gbsp_batch_plan_info(gbsp_batch_t batch, int i, gbsp_plan_info* info);
/* Reads and clears the device error flags of the batch and its sub-plans. */
int gbsp_batch_error_flags(gbsp_batch_t batch, int* flags);
int gbsp_batch_destroy(gbsp_batch_t batch);

/* ---- tuning and the learned cost model ------------------------------------
 * The reference fixes its configuration (--csc-tile, radix 9/3/2 order,
 * src/sparse_fft_bluestein.cu:1996-2011); these entry points have no
 * counterpart there.
 *
 * Candidates of a matrix: the `max_rows_cands` cheapest (radix sequence, row
 * block) choices of the analytic model crossed with every pass-1 shape that
 * fits.  out[i * n_p1 + j] pairs row choice i with shape j; each is `base`
 * with radix, rows_threads and pass1_shape filled in.  Host-only (uses the
 * current device's shared-memory limit, GB300's without a device). */
int gbsp_plan_candidates(int rows, int cols, const gbsp_options* base, int max_rows_cands,
                         gbsp_options* out, int cap, int* n_rows_cands, int* n_p1_cands);

/* Cost-model features of (matrix, candidate): GBSP_N_FEATURES floats.
 * [0,18) describe the matrix (log2 sizes, density, largest prime factors,
 * fft_len, channels, column-degree histogram), [18,28) the row choice
 * (block, stages, radices, shared memory, CTAs/SM, analytic cost) and
 * [28,36) the pass-1 shape.  Host-only. */
int gbsp_plan_features(int rows, int cols, int n_active, int nnz, const int* col_ptr,
                       const gbsp_options* cand, float* out);

/* One measured candidate: device time of pass 1 under its pass-1 shape and
 * of the Bluestein rows under its radices and block (best of `reps`). */
typedef struct {
    gbsp_options opts;
    float ms_pass1;
    float ms_rows;
} gbsp_tune_entry;

/* Exhaustive autotuner: measures every candidate of the matrix on the
 * current device (plans built, executed and destroyed in turn; one output
 * buffer allocated for the duration).  Pass 1 depends only on the pass-1
 * shape and the rows only on the row choice, so max(n_rows, n_p1) plans
 * cover the whole cross product; entries[i * n_p1 + j] holds the composed
 * times.  *best receives the candidate with the least total, with u_tile
 * (the --csc-tile analogue) chosen last among {cap, cap/2, cap/4} where cap
 * is base->u_tile (0 = all rows; smaller tiles bound the scratch memory).
 * Blocking. */
int gbsp_autotune(int rows, int cols, int n_active, int nnz, const int* col_ptr, const int* row_idx,
                  const int* sparse_cols, const gbsp_options* base, int max_rows_cands, int reps,
                  void* stream, gbsp_options* best, gbsp_tune_entry* entries, int cap,
                  int* n_rows_cands, int* n_p1_cands);

/* MLP cost model: n_in -> 64 -> 64 -> 1, ReLU, FP32.  Parameters, packed:
 * W1[n_in][64], b1[64], W2[64][64], b2[64], w3[64], b3 (W[k][j] maps input
 * k to unit j).  The kernels are deterministic (fixed reduction order). */
#define GBSP_MLP_HIDDEN 64
size_t gbsp_mlp_param_count(int n_in);
/* y[i] = f(x[i]) for n rows of x (row-major n x n_in).  Device pointers. */
int gbsp_mlp_forward(const float* d_params, int n_in, const float* d_x, int n, float* d_y, void* stream);
/* Gradient of the loss mean_i (f(x_i) - t_i)^2 with respect to every
 * parameter into d_grad (param_count floats) and the loss into *d_loss.
 * d_work: scratch of gbsp_mlp_work_floats(n_in) floats. */
size_t gbsp_mlp_work_floats(int n_in);
int gbsp_mlp_backward(const float* d_params, int n_in, const float* d_x, const float* d_target, int n,
                      float* d_grad, float* d_loss, float* d_work, void* stream);
/* One Adam step (bias-corrected, step >= 1) on n_params parameters. */
int gbsp_mlp_adam(float* d_params, const float* d_grad, float* d_m, float* d_v, size_t n_params, float lr,
                  float beta1, float beta2, float eps, int step, void* stream);
/* Installs the model GBSP_PLANNER_LEARNED uses (host arrays, copied):
 * inputs are standardised as (x - feat_mean) / feat_scale before the
 * network; the output is log(predicted ms).  n_in must be GBSP_N_FEATURES. */
int gbsp_cost_model_set(const float* params, int n_in, const float* feat_mean, const float* feat_scale);
/* Optional, after gbsp_cost_model_set (which clears it): the range of each
 * feature over the model's training candidates.  A matrix with a candidate
 * feature outside [lo - m, hi + m], m = 10 % of hi - lo, is planned by the
 * analytic model instead (its info.planner reads GBSP_PLANNER_MODEL): the
 * network is not trusted where it never saw data.  NULL, NULL clears it. */
int gbsp_cost_model_set_domain(int n_in, const float* feat_lo, const float* feat_hi);

#ifdef __cplusplus
}
#endif
#endif /* GBSPFFT_H */
