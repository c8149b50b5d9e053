// gbsp_fft.cuh -- register-level small DFTs and the in-place shared-memory
// mixed-radix (2/3/4/5/7/8) FFT used by the Bluestein row kernel.
//
// The forward transform is an in-place decimation-in-frequency (DIF) network:
// a stage of radix R with span m reads x[j*R*m + s*m + k] (s < R), applies an
// R-point DFT, multiplies output q by W_{R*m}^{q*k} and writes it back to
// x[j*R*m + q*m + k].  After all stages the spectrum sits in digit-reversed
// order.  The inverse is the same network run backwards as
// decimation-in-time (DIT): conjugate twiddle first, inverse R-point DFT,
// store.  A Bluestein convolution never needs natural-order spectra: the
// kernel multiplies by the filter spectrum stored in the same digit-reversed
// order, so no permutation pass exists anywhere.
//
// The reference instead runs out-of-place Stockham stages through global
// memory, one launch per stage (src/sparse_fft_bluestein.cu:184-215,
// 2017-2254); here all stages of one row run inside one CTA.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbsp {

template <typename T> struct vec2;
template <> struct vec2<float>  { using type = float2; };
template <> struct vec2<double> { using type = double2; };

template <typename V> __host__ __device__ __forceinline__ V mk(decltype(V::x) x, decltype(V::x) y) {
    V r; r.x = x; r.y = y; return r;
}
template <typename V> __device__ __forceinline__ V cadd(V a, V b) { return mk<V>(a.x + b.x, a.y + b.y); }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { return mk<V>(a.x - b.x, a.y - b.y); }
// a * b
template <typename V> __device__ __forceinline__ V cmul(V a, V b) {
    return mk<V>(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a * conj(b)
template <typename V> __device__ __forceinline__ V cmulc(V a, V b) {
    return mk<V>(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}
template <typename V> __device__ __forceinline__ V cconj(V a) { return mk<V>(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename V> __device__ __forceinline__ V mul_mi(V a) {
    return INV ? mk<V>(-a.y, a.x) : mk<V>(a.y, -a.x);
}

// cos / sin of 2*pi*k/R, the exact constants of the small DFTs.
struct C3 { static constexpr double c1 = -0.5, s1 = 0.8660254037844386467637; };
struct C5 {
    static constexpr double c1 = 0.3090169943749474241023, s1 = 0.9510565162951535721164;
    static constexpr double c2 = -0.8090169943749474241023, s2 = 0.5877852522924731291687;
};
struct C7 {
    static constexpr double c1 = 0.623489801858733530525, s1 = 0.7818314824680298087084;
    static constexpr double c2 = -0.2225209339563144042889, s2 = 0.9749279121818236070181;
    static constexpr double c3 = -0.9009688679024191262361, s3 = 0.4338837391175581204758;
};
static constexpr double RSQRT2 = 0.7071067811865475244008;

// In-register R-point DFT.  Forward uses W_R = exp(-2*pi*i/R), inverse
// exp(+2*pi*i/R); neither scales.
template <int R, bool INV, typename V> struct SmallDFT;

template <bool INV, typename V> struct SmallDFT<2, INV, V> {
    __device__ __forceinline__ static void run(V* a) {
        V t = a[0];
        a[0] = cadd(t, a[1]);
        a[1] = csub(t, a[1]);
    }
};

template <bool INV, typename V> struct SmallDFT<3, INV, V> {
    __device__ __forceinline__ static void run(V* a) {
        using T = decltype(V::x);
        const T c1 = (T)C3::c1, s1 = (T)C3::s1;
        V s = cadd(a[1], a[2]);
        V d = csub(a[1], a[2]);
        V y0 = cadd(a[0], s);
        V t  = mk<V>(fma(c1, s.x, a[0].x), fma(c1, s.y, a[0].y));
        V sd = mk<V>(s1 * d.x, s1 * d.y);
        V r  = mul_mi<INV>(sd);
        a[0] = y0;
        a[1] = cadd(t, r);
        a[2] = csub(t, r);
    }
};

template <bool INV, typename V> struct SmallDFT<4, INV, V> {
    __device__ __forceinline__ static void run(V* a) {
        V s02 = cadd(a[0], a[2]), d02 = csub(a[0], a[2]);
        V s13 = cadd(a[1], a[3]), d13 = mul_mi<INV>(csub(a[1], a[3]));
        a[0] = cadd(s02, s13);
        a[2] = csub(s02, s13);
        a[1] = cadd(d02, d13);
        a[3] = csub(d02, d13);
    }
};

// Odd prime p via symmetric pairs: s_k = a_k + a_{p-k}, d_k = a_k - a_{p-k};
// y_q = a_0 + sum_k cos(2pi qk/p) s_k  -/+ i * sum_k sin(2pi qk/p) d_k.
template <bool INV, typename V> struct SmallDFT<5, INV, V> {
    __device__ __forceinline__ static void run(V* a) {
        using T = decltype(V::x);
        const T c1 = (T)C5::c1, s1 = (T)C5::s1, c2 = (T)C5::c2, s2 = (T)C5::s2;
        V s1v = cadd(a[1], a[4]), d1v = csub(a[1], a[4]);
        V s2v = cadd(a[2], a[3]), d2v = csub(a[2], a[3]);
        V y0 = cadd(a[0], cadd(s1v, s2v));
        V A1 = mk<V>(a[0].x + c1 * s1v.x + c2 * s2v.x, a[0].y + c1 * s1v.y + c2 * s2v.y);
        V A2 = mk<V>(a[0].x + c2 * s1v.x + c1 * s2v.x, a[0].y + c2 * s1v.y + c1 * s2v.y);
        V B1 = mk<V>(s1 * d1v.x + s2 * d2v.x, s1 * d1v.y + s2 * d2v.y);
        V B2 = mk<V>(s2 * d1v.x - s1 * d2v.x, s2 * d1v.y - s1 * d2v.y);
        V r1 = mul_mi<INV>(B1), r2 = mul_mi<INV>(B2);
        a[0] = y0;
        a[1] = cadd(A1, r1); a[4] = csub(A1, r1);
        a[2] = cadd(A2, r2); a[3] = csub(A2, r2);
    }
};

template <bool INV, typename V> struct SmallDFT<7, INV, V> {
    __device__ __forceinline__ static void run(V* a) {
        using T = decltype(V::x);
        const T c1 = (T)C7::c1, s1 = (T)C7::s1, c2 = (T)C7::c2, s2 = (T)C7::s2;
        const T c3 = (T)C7::c3, s3 = (T)C7::s3;
        V p1 = cadd(a[1], a[6]), m1 = csub(a[1], a[6]);
        V p2 = cadd(a[2], a[5]), m2 = csub(a[2], a[5]);
        V p3 = cadd(a[3], a[4]), m3 = csub(a[3], a[4]);
        V y0 = cadd(a[0], cadd(p1, cadd(p2, p3)));
        // cos(2pi*q*k/7) for q,k in 1..3 : (qk mod 7) -> c1,c2,c3 with symmetry
        V A1 = mk<V>(a[0].x + c1 * p1.x + c2 * p2.x + c3 * p3.x, a[0].y + c1 * p1.y + c2 * p2.y + c3 * p3.y);
        V A2 = mk<V>(a[0].x + c2 * p1.x + c3 * p2.x + c1 * p3.x, a[0].y + c2 * p1.y + c3 * p2.y + c1 * p3.y);
        V A3 = mk<V>(a[0].x + c3 * p1.x + c1 * p2.x + c2 * p3.x, a[0].y + c3 * p1.y + c1 * p2.y + c2 * p3.y);
        // sin(2pi*q*k/7): q=1: s1,s2,s3; q=2: s2,-s3,-s1; q=3: s3,-s1,s2
        V B1 = mk<V>(s1 * m1.x + s2 * m2.x + s3 * m3.x, s1 * m1.y + s2 * m2.y + s3 * m3.y);
        V B2 = mk<V>(s2 * m1.x - s3 * m2.x - s1 * m3.x, s2 * m1.y - s3 * m2.y - s1 * m3.y);
        V B3 = mk<V>(s3 * m1.x - s1 * m2.x + s2 * m3.x, s3 * m1.y - s1 * m2.y + s2 * m3.y);
        V r1 = mul_mi<INV>(B1), r2 = mul_mi<INV>(B2), r3 = mul_mi<INV>(B3);
        a[0] = y0;
        a[1] = cadd(A1, r1); a[6] = csub(A1, r1);
        a[2] = cadd(A2, r2); a[5] = csub(A2, r2);
        a[3] = cadd(A3, r3); a[4] = csub(A3, r3);
    }
};

// 8 = 2 x 4: radix-2 split with W_8^n twiddles, then two 4-point DFTs
// (even outputs from the sums, odd outputs from the twiddled differences).
template <bool INV, typename V> struct SmallDFT<8, INV, V> {
    __device__ __forceinline__ static void run(V* a) {
        using T = decltype(V::x);
        const T h = (T)RSQRT2;
        V b[4], c[4];
#pragma unroll
        for (int n = 0; n < 4; n++) { b[n] = cadd(a[n], a[n + 4]); c[n] = csub(a[n], a[n + 4]); }
        // c[1] *= W8^1, c[2] *= W8^2 = -+i, c[3] *= W8^3
        {
            V t = c[1];
            // forward W8 = (1 - i)/sqrt2 ; inverse (1 + i)/sqrt2
            c[1] = INV ? mk<V>(h * (t.x - t.y), h * (t.x + t.y)) : mk<V>(h * (t.x + t.y), h * (t.y - t.x));
            c[2] = mul_mi<INV>(c[2]);
            t = c[3];
            // forward W8^3 = (-1 - i)/sqrt2 ; inverse (-1 + i)/sqrt2
            c[3] = INV ? mk<V>(-h * (t.x + t.y), h * (t.x - t.y)) : mk<V>(h * (t.y - t.x), -h * (t.x + t.y));
        }
        SmallDFT<4, INV, V>::run(b);
        SmallDFT<4, INV, V>::run(c);
#pragma unroll
        for (int k = 0; k < 4; k++) { a[2 * k] = b[k]; a[2 * k + 1] = c[k]; }
    }
};

// Shared-memory index with one pad slot per 16 complex values: strides that
// are multiples of 16 (power-of-two radices) no longer land on one bank.
__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int padded_len(int n) { return n + (n >> 4) + 1; }

// One stage of the FFT network on a shared-memory buffer (padded indices).
//   MODE 0: forward DIF stage
//   MODE 1: inverse DIT stage
//   MODE 2: last forward stage + pointwise filter multiply + first inverse
//           stage (their twiddles cancel, so neither is applied)
// Twiddles are stored q-major per stage, tw[(q-1)*m + k] = W_{R*m}^{q*k}, so a
// warp's loads for one q are contiguous.  The filter of the fused stage (the
// last stage, m = 1, base = t*R) is stored in the same thread order,
// filt[q*(Lp/R) + t].  `magic` = ceil(2^32/m) gives j = t/m exactly for
// t, m < 2^16.
template <int R, int MODE, typename V>
__device__ __forceinline__ void fft_stage(V* __restrict__ buf, int Lp, int m, uint32_t magic,
                                          const V* __restrict__ tw, const V* __restrict__ filt,
                                          int tid, int nthreads) {
    const int nb = Lp / R;
    for (int t = tid; t < nb; t += nthreads) {
        int j, k;
        if (m == 1) { j = t; k = 0; }
        else { j = (int)__umulhi((uint32_t)t, magic); k = t - j * m; }
        const int base = j * R * m + k;
        V a[R];
#pragma unroll
        for (int s = 0; s < R; s++) a[s] = buf[pad16(base + s * m)];
        if (MODE == 0) {
            SmallDFT<R, false, V>::run(a);
            if (k != 0) {
#pragma unroll
                for (int q = 1; q < R; q++) a[q] = cmul(a[q], tw[(q - 1) * m + k]);
            }
        } else if (MODE == 1) {
            if (k != 0) {
#pragma unroll
                for (int q = 1; q < R; q++) a[q] = cmulc(a[q], tw[(q - 1) * m + k]);
            }
            SmallDFT<R, true, V>::run(a);
        } else {
            SmallDFT<R, false, V>::run(a);
#pragma unroll
            for (int q = 0; q < R; q++) a[q] = cmul(a[q], filt[q * nb + t]);
            SmallDFT<R, true, V>::run(a);
        }
#pragma unroll
        for (int s = 0; s < R; s++) buf[pad16(base + s * m)] = a[s];
    }
}

template <int MODE, typename V>
__device__ __forceinline__ void fft_stage_dispatch(int R, V* buf, int Lp, int m, uint32_t magic,
                                                   const V* tw, const V* filt, int tid, int nthreads) {
    switch (R) {
        case 2: fft_stage<2, MODE>(buf, Lp, m, magic, tw, filt, tid, nthreads); break;
        case 3: fft_stage<3, MODE>(buf, Lp, m, magic, tw, filt, tid, nthreads); break;
        case 4: fft_stage<4, MODE>(buf, Lp, m, magic, tw, filt, tid, nthreads); break;
        case 5: fft_stage<5, MODE>(buf, Lp, m, magic, tw, filt, tid, nthreads); break;
        case 7: fft_stage<7, MODE>(buf, Lp, m, magic, tw, filt, tid, nthreads); break;
        case 8: fft_stage<8, MODE>(buf, Lp, m, magic, tw, filt, tid, nthreads); break;
        default: break;
    }
}

}  // namespace gbsp
