/*
 * ref_gpu_port.c -- FP32 restatement, on the CPU, of the reference's two GPU
 * methods for this path.  TEST INFRASTRUCTURE ONLY: tests/ and bench.py's
 * accuracy leg load oracle/_build/libref_port.so as a checker; the library
 * never does.
 *
 * It follows the reference's algorithm and FP32 operation order:
 *   pass 1   src/sparse_fft_bluestein.cu:366-397 (csc_build_bluestein_input_packed_kernel):
 *            idx = (u*r) mod rows in 32-bit, angle = (-2pi * (float)idx) * (1/rows)
 *            in float, summed in FP32 over the column, times chirp[c] with fmaf.
 *   FFT      out-of-place Stockham stages (:184-215 radix 2, :2017-2080 radix 3;
 *            the radix-9 stage :2093-2209 is two radix-3 stages fused, run here
 *            as the two stages) with twiddle angles formed in float; the
 *            7-smooth method's cuFFT (:2605-2686) and the power-of-two
 *            methods' FFTs are replaced by the same
 *            Stockham engine with radix 5 and 7 stages (cuFFT is closed
 *            source; only its contract -- an FP32 C2C FFT -- is restated).
 *   filter   B = FFT(b), b from make_bluestein_b (include/sparse_fft_internal.cuh:179-191)
 *   multiply pointwise_mul_batched_kernel (:316-329), scale 1/L (:74-80),
 *   finalize bluestein_finalize_kernel (:469-486).
 * The reference evaluates sines and cosines with the __sincosf fast
 * intrinsic, whose exact values cannot be restated; this port calls the C
 * library's sinf/cosf on the same float angles instead.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct { float x, y; } cf;

static cf cmk(float x, float y) { cf r; r.x = x; r.y = y; return r; }

static int next_smooth(int n, int seven) {
    for (int m = n;; ++m) {
        int x = m;
        while (x % 2 == 0) x /= 2;
        while (x % 3 == 0) x /= 3;
        if (seven) {
            while (x % 5 == 0) x /= 5;
            while (x % 7 == 0) x /= 7;
        }
        if (x == 1) return m;
    }
}

/* radices first to last: 3-smooth -> 3s (the reference's 9s are two 3s) then 2s;
   7-smooth -> 7s, 5s, 3s, 2s */
static int radix_list(int n, int seven, int* rs) {
    int k = 0;
    if (seven) {
        while (n % 7 == 0) { rs[k++] = 7; n /= 7; }
        while (n % 5 == 0) { rs[k++] = 5; n /= 5; }
    }
    while (n % 3 == 0) { rs[k++] = 3; n /= 3; }
    while (n % 2 == 0) { rs[k++] = 2; n /= 2; }
    return n == 1 ? k : -1;
}

/* Per-stage constants: the R-point DFT matrix and the output twiddles
   exp(sign*2pi*i*q*k/(R*m)) with the angle formed in float as the reference
   does (ang1 = sign*2pi*k/(R*m), ang_q = ang1*q).  Built once per length. */
typedef struct {
    int R, m;
    float dft_c[2][64], dft_s[2][64];  /* [inverse][s*R + q] */
    float* tw_c[2];                    /* [inverse][(q-1)*m + k] */
    float* tw_s[2];
} stage_t;

static void stage_init(stage_t* st, int R, int m) {
    const float two_pi = 6.28318530717958647f;
    st->R = R;
    st->m = m;
    for (int inv = 0; inv < 2; inv++) {
        for (int s = 0; s < R; s++)
            for (int q = 0; q < R; q++) {
                const float a = (inv ? two_pi : -two_pi) * (float)((s * q) % R) / (float)R;
                st->dft_c[inv][s * R + q] = cosf(a);
                st->dft_s[inv][s * R + q] = sinf(a);
            }
        st->tw_c[inv] = (float*)malloc(sizeof(float) * (size_t)(R > 1 ? R - 1 : 1) * m);
        st->tw_s[inv] = (float*)malloc(sizeof(float) * (size_t)(R > 1 ? R - 1 : 1) * m);
        for (int k = 0; k < m; k++) {
            const float ang1 = (inv ? two_pi : -two_pi) * (float)k / (float)(R * m);
            for (int q = 1; q < R; q++) {
                const float a = ang1 * (float)q;
                st->tw_c[inv][(q - 1) * m + k] = cosf(a);
                st->tw_s[inv][(q - 1) * m + k] = sinf(a);
            }
        }
    }
}

static void stage_free(stage_t* st) {
    for (int inv = 0; inv < 2; inv++) { free(st->tw_c[inv]); free(st->tw_s[inv]); }
}

/* One Stockham stage: in[j*R*m + s*m + k] -> R-point DFT -> output q times
   the stage twiddle -> out[(q*l + j)*m + k], l = n/(R*m). */
static void stockham_stage(const cf* in, cf* out, int n, const stage_t* st, int inverse) {
    const int R = st->R, m = st->m, l = n / (R * m);
    const float* dc = st->dft_c[inverse];
    const float* ds = st->dft_s[inverse];
    const float* tc = st->tw_c[inverse];
    const float* ts = st->tw_s[inverse];
    cf x[8], y[8];
    for (int j = 0; j < l; j++)
        for (int k = 0; k < m; k++) {
            for (int s = 0; s < R; s++) x[s] = in[j * R * m + s * m + k];
            for (int q = 0; q < R; q++) {
                float ax = 0.f, ay = 0.f;
                for (int s = 0; s < R; s++) {
                    const float c = dc[s * R + q], sn = ds[s * R + q];
                    ax += x[s].x * c - x[s].y * sn;
                    ay += x[s].x * sn + x[s].y * c;
                }
                y[q] = cmk(ax, ay);
            }
            if (k != 0)
                for (int q = 1; q < R; q++) {
                    const float c = tc[(q - 1) * m + k], sn = ts[(q - 1) * m + k];
                    const cf t = y[q];
                    y[q] = cmk(fmaf(t.x, c, -t.y * sn), fmaf(t.x, sn, t.y * c));
                }
            for (int q = 0; q < R; q++) out[(q * l + j) * m + k] = y[q];
        }
}

/* FFT of one row (length n) via ping-pong buffers; returns the result buffer. */
static cf* fft_row(cf* a, cf* b, int n, const stage_t* st, int nr, int inverse) {
    cf* src = a;
    cf* dst = b;
    for (int i = 0; i < nr; i++) {
        stockham_stage(src, dst, n, &st[i], inverse);
        cf* t = src; src = dst; dst = t;
    }
    return src;
}

/*
 * Full transform.  csc arrays as make_compact_csc returns them; out is
 * rows x (cols/2+1) interleaved float pairs.  method: 3 = mixed-radix
 * (3-smooth), 7 = cufft-smooth (7-smooth), 2 = the power-of-two methods
 * (sparse_fft_csc_bluestein and the others at
 * fft_len = next_power_of_two(2*cols-1), include/sparse_fft_internal.cuh:153-157,
 * radix-2 stages).  Returns 0 on success.
 */
int port_sparse_fft(int rows, int cols, int n_active, const int* sparse_cols, const int* col_ptr,
                    const int* row_idx, int method, float* out) {
    const int seven = (method == 7);
    int L = 1;
    if (method == 2)
        while (L < 2 * cols - 1) L <<= 1;
    else
        L = next_smooth(2 * cols - 1, seven);
    int rs[64];
    const int nr = radix_list(L, seven, rs);
    if (nr < 0) return 1;
    stage_t st[64];
    {
        int l = 1;
        for (int i = 0; i < nr; i++) {
            stage_init(&st[i], rs[i], L / (l * rs[i]));
            l *= rs[i];
        }
    }
    const int oc = cols / 2 + 1;
    cf* chirp = (cf*)malloc(sizeof(cf) * cols);
    cf* bb = (cf*)calloc(L, sizeof(cf));
    cf* w1 = (cf*)malloc(sizeof(cf) * L);
    cf* w2 = (cf*)malloc(sizeof(cf) * L);
    if (!chirp || !bb || !w1 || !w2) return 2;
    const double pi = 3.1415926535897932384626433832795;
    for (int k = 0; k < cols; k++) {
        const double ang = -pi * ((double)k * (double)k) / (double)cols;
        chirp[k] = cmk((float)cos(ang), (float)sin(ang));
    }
    bb[0] = cmk(1.f, 0.f);
    for (int k = 1; k < cols; k++) {
        const double ang = pi * ((double)k * (double)k) / (double)cols;
        const cf z = cmk((float)cos(ang), (float)sin(ang));
        bb[k] = z;
        bb[L - k] = z;
    }
    memcpy(w1, bb, sizeof(cf) * L);
    cf* bf = fft_row(w1, w2, L, st, nr, 0);
    cf* B = (cf*)malloc(sizeof(cf) * L);
    memcpy(B, bf, sizeof(cf) * L);
    const float two_pi = 6.28318530717958647f;
    const float inv_rows = 1.f / (float)rows;
    const float inv_L = 1.f / (float)L;
    for (int u = 0; u < rows; u++) {
        memset(w1, 0, sizeof(cf) * L);
        for (int j = 0; j < n_active; j++) {
            float re = 0.f, im = 0.f;
            for (int p = col_ptr[j]; p < col_ptr[j + 1]; p++) {
                const uint32_t idx = ((uint32_t)u * (uint32_t)row_idx[p]) % (uint32_t)rows;
                const float a = -two_pi * (float)idx * inv_rows;
                re += cosf(a);
                im += sinf(a);
            }
            const cf q = chirp[sparse_cols[j]];
            w1[sparse_cols[j]] = cmk(fmaf(re, q.x, -im * q.y), fmaf(re, q.y, im * q.x));
        }
        cf* f = fft_row(w1, w2, L, st, nr, 0);
        for (int k = 0; k < L; k++) {
            const cf x = f[k], y = B[k];
            f[k] = cmk(fmaf(x.x, y.x, -x.y * y.y), fmaf(x.x, y.y, x.y * y.x));
        }
        cf* other = (f == w1) ? w2 : w1;
        cf* g = fft_row(f, other, L, st, nr, 1);
        for (int v = 0; v < oc; v++) {
            const cf y = cmk(g[v].x * inv_L, g[v].y * inv_L), q = chirp[v];
            out[2 * ((size_t)u * oc + v)] = fmaf(y.x, q.x, -y.y * q.y);
            out[2 * ((size_t)u * oc + v) + 1] = fmaf(y.x, q.y, y.y * q.x);
        }
    }
    free(chirp); free(bb); free(w1); free(w2); free(B);
    for (int i = 0; i < nr; i++) stage_free(&st[i]);
    return 0;
}

int port_next_smooth(int n, int seven) { return next_smooth(n, seven); }
