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

#include <type_traits>
#include <utility>

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

// ---------------------------------------------------------------------------
// Compile-time roots of unity for the composite radices: cos / sin of
// 2*pi*j/n with the angle folded into [0, pi/4] by exact integer symmetry,
// then a Taylor series in double (error far below float rounding).
// ---------------------------------------------------------------------------
struct Root { double c, s; };

__host__ __device__ constexpr double ct_sin(double x) {
    double t = x, acc = x;
    for (int k = 1; k < 14; k++) { t *= -x * x / ((2.0 * k) * (2.0 * k + 1.0)); acc += t; }
    return acc;
}
__host__ __device__ constexpr double ct_cos(double x) {
    double t = 1.0, acc = 1.0;
    for (int k = 1; k < 14; k++) { t *= -x * x / ((2.0 * k - 1.0) * (2.0 * k)); acc += t; }
    return acc;
}
// angle 2*pi*j/n
__host__ __device__ constexpr Root unit_root(long j, long n) {
    j %= n;
    if (j < 0) j += n;
    if (2 * j > n) {  // (pi, 2pi): mirror
        Root r = unit_root(n - j, n);
        return Root{r.c, -r.s};
    }
    if (4 * j > n) {  // (pi/2, pi]: cos(t) = -cos(pi - t), sin(t) = sin(pi - t)
        Root r = unit_root(n - 2 * j, 2 * n);
        return Root{-r.c, r.s};
    }
    if (8 * j > n) {  // (pi/4, pi/2]: swap with pi/2 - t
        Root r = unit_root(n - 4 * j, 4 * n);
        return Root{r.s, r.c};
    }
    const double x = 6.283185307179586476925286766559 * (double)j / (double)n;
    return Root{ct_cos(x), ct_sin(x)};
}

template <int N, typename F, int... I>
__device__ __forceinline__ void static_for_impl(F&& f, std::integer_sequence<int, I...>) {
    (f(std::integral_constant<int, I>{}), ...);
}
// f(integral_constant<int, i>) for i = 0..N-1, each index a compile-time constant
template <int N, typename F>
__device__ __forceinline__ void static_for(F&& f) {
    static_for_impl<N>(f, std::make_integer_sequence<int, N>{});
}

// x * W_P^{E} (forward, W_P = exp(-2*pi*i/P)) or x * W_P^{-E} (inverse)
template <int P, int E, bool INV, typename V>
__device__ __forceinline__ V mul_root(V x) {
    constexpr int e = E % P;
    if constexpr (e == 0) {
        return x;
    } else if constexpr (2 * e == P) {
        return mk<V>(-x.x, -x.y);
    } else if constexpr (4 * e == P) {
        return mul_mi<INV>(x);
    } else if constexpr (4 * e == 3 * P) {
        return mul_mi<!INV>(x);
    } else {
        using T = decltype(V::x);
        constexpr Root r = unit_root(e, P);
        const T c = (T)r.c, sn = INV ? (T)r.s : (T)-r.s;
        return mk<V>(fma(x.x, c, -x.y * sn), fma(x.x, sn, x.y * c));
    }
}

// ---------------------------------------------------------------------------
// Radix<P>: the P-point DFT of one butterfly held in registers.
//   fwd(a): a[] natural-order input -> outputs X[q] at register out_reg(q)
//   inv(a): inputs X[q] at register out_reg(q) -> natural-order a[] (unscaled)
// Prime-power radices 2..8 use SmallDFT (out_reg = identity).  A composite
// P = A*B splits n = B*n1 + n2, q = k1 + A*k2: A-point DFTs over n1, the
// twiddles W_P^{n2*k1}, then B-point DFTs over n2, leaving X[k1 + A*k2] in
// register B*k1 + k2 -- no register shuffles, the stage's loads and stores
// absorb the permutation.
// ---------------------------------------------------------------------------
template <int P> struct Split;  // composite radices: A * B
template <> struct Split<9>  { static constexpr int A = 3, B = 3; };
template <> struct Split<12> { static constexpr int A = 4, B = 3; };
template <> struct Split<15> { static constexpr int A = 5, B = 3; };
template <> struct Split<16> { static constexpr int A = 4, B = 4; };
template <> struct Split<20> { static constexpr int A = 5, B = 4; };
template <> struct Split<21> { static constexpr int A = 7, B = 3; };
template <> struct Split<24> { static constexpr int A = 8, B = 3; };
template <> struct Split<25> { static constexpr int A = 5, B = 5; };
template <> struct Split<28> { static constexpr int A = 7, B = 4; };
template <> struct Split<32> { static constexpr int A = 8, B = 4; };
template <> struct Split<35> { static constexpr int A = 7, B = 5; };
template <> struct Split<40> { static constexpr int A = 8, B = 5; };

template <int P> struct IsBase { static constexpr bool value = (P == 2 || P == 3 || P == 4 || P == 5 || P == 7 || P == 8); };

template <int P, bool BASE = IsBase<P>::value> struct Radix;

template <int P> struct Radix<P, true> {
    __host__ __device__ static constexpr int out_reg(int q) { return q; }
    template <typename V> __device__ __forceinline__ static void fwd(V* a) { SmallDFT<P, false, V>::run(a); }
    template <typename V> __device__ __forceinline__ static void inv(V* a) { SmallDFT<P, true, V>::run(a); }
};

template <int P> struct Radix<P, false> {
    static constexpr int A = Split<P>::A, B = Split<P>::B;
    __host__ __device__ static constexpr int out_reg(int q) { return B * (q % A) + q / A; }
    template <typename V> __device__ __forceinline__ static void fwd(V* a) {
        static_for<B>([&](auto n2c) {
            constexpr int n2 = decltype(n2c)::value;
            V x[A];
#pragma unroll
            for (int n1 = 0; n1 < A; n1++) x[n1] = a[B * n1 + n2];
            SmallDFT<A, false, V>::run(x);
            static_for<A>([&](auto k1c) {
                constexpr int k1 = decltype(k1c)::value;
                a[B * k1 + n2] = mul_root<P, n2 * k1, false>(x[k1]);
            });
        });
#pragma unroll
        for (int k1 = 0; k1 < A; k1++) SmallDFT<B, false, V>::run(a + B * k1);
    }
    template <typename V> __device__ __forceinline__ static void inv(V* a) {
#pragma unroll
        for (int k1 = 0; k1 < A; k1++) SmallDFT<B, true, V>::run(a + B * k1);
        static_for<B>([&](auto n2c) {
            constexpr int n2 = decltype(n2c)::value;
            V x[A];
            static_for<A>([&](auto k1c) {
                constexpr int k1 = decltype(k1c)::value;
                x[k1] = mul_root<P, n2 * k1, true>(a[B * k1 + n2]);
            });
            SmallDFT<A, true, V>::run(x);
#pragma unroll
            for (int n1 = 0; n1 < A; n1++) a[B * n1 + n2] = x[n1];
        });
    }
};

// One stage of the FFT network on a shared-memory buffer.
//   MODE 0: forward DIF stage
//   MODE 1: inverse DIT stage
//   MODE 2: last forward stage + pointwise filter multiply + first inverse
//           stage (their twiddles cancel, so neither is applied); the last
//           stage always has span 1, so butterfly t covers buf[t*R, t*R+R)
// Twiddles are stored q-major per stage, tw[(q-1)*m + k] = W_{R*m}^{q*k}, so a
// warp's loads for one q are contiguous.  TWG: the twiddles are read through
// the read-only global path (stage 0, whose table does not fit in shared
// memory beside the row), else from shared memory.  The entries at k = 0 are
// exactly 1, so every butterfly applies its twiddles without a branch (a
// complex product by (1, 0) is exact).  The filter of the fused stage is
// stored in the same thread order, filt[q*(Lp/R) + t], in global memory.
//
// Thread -> butterfly mapping: for spans m >= 16 consecutive threads take
// consecutive k (unit-stride shared-memory accesses); for shorter spans with
// R*m odd they take consecutive j, i.e. stride R*m, which hits distinct banks.
// `magic` = ceil(2^32/d) gives t/d exactly for t, d < 2^16 where d is m
// (k-fastest) or l = Lp/(R*m) (j-fastest).
__host__ __device__ constexpr bool stage_j_fastest(int R, int m, int l) {
    return m > 1 && m < 16 && l > 1 && ((R * m) & 1) == 1;
}

template <bool TWG, typename V>
__device__ __forceinline__ V tw_load(const V* __restrict__ p) {
    if constexpr (TWG) return __ldg(p);
    else return *p;
}

template <int R, int MODE, bool TWG, typename V>
__device__ __forceinline__ void fft_stage(V* __restrict__ buf, int Lp, int m, uint32_t magic,
                                          const V* __restrict__ tw, const V* __restrict__ filt,
                                          int tid, int nthreads) {
    using RX = Radix<R>;
    const int nb = Lp / R;
    if constexpr (MODE == 2) {
        for (int t = tid; t < nb; t += nthreads) {
            V* p = buf + t * R;
            V a[R];
#pragma unroll
            for (int s = 0; s < R; s++) a[s] = p[s];
            RX::fwd(a);
            const V* f = filt + t;
#pragma unroll
            for (int q = 0; q < R; q++) a[RX::out_reg(q)] = cmul(a[RX::out_reg(q)], __ldg(f + q * nb));
            RX::inv(a);
#pragma unroll
            for (int s = 0; s < R; s++) p[s] = a[s];
        }
        return;
    }
    const int l = nb / m;
    const bool jfast = stage_j_fastest(R, m, l);
    for (int t = tid; t < nb; t += nthreads) {
        int j, k;
        if (m == 1) { j = t; k = 0; }
        else if (!jfast) { j = (int)__umulhi((uint32_t)t, magic); k = t - j * m; }
        else { k = (int)__umulhi((uint32_t)t, magic); j = t - k * l; }
        const int base = j * R * m + k;
        const V* twk = tw + k;
        V a[R];
        if (MODE == 1) {
            // inputs q sit in register out_reg(q)
#pragma unroll
            for (int q = 0; q < R; q++) a[RX::out_reg(q)] = buf[base + q * m];
#pragma unroll
            for (int q = 1; q < R; q++)
                a[RX::out_reg(q)] = cmulc(a[RX::out_reg(q)], tw_load<TWG>(twk + (q - 1) * m));
            RX::inv(a);
#pragma unroll
            for (int s = 0; s < R; s++) buf[base + s * m] = a[s];
        } else {
#pragma unroll
            for (int s = 0; s < R; s++) a[s] = buf[base + s * m];
            RX::fwd(a);
#pragma unroll
            for (int q = 1; q < R; q++)
                a[RX::out_reg(q)] = cmul(a[RX::out_reg(q)], tw_load<TWG>(twk + (q - 1) * m));
#pragma unroll
            for (int q = 0; q < R; q++) buf[base + q * m] = a[RX::out_reg(q)];
        }
    }
}

// The first forward stage reading its inputs straight from global memory
// (the sequential-channel rows: no bulk copy into shared memory, no separate
// pre-twiddle pass): x[n] = src[n] * pre[n] (PRE) or src[n] for n < cols,
// zero beyond.  Stage 0 has span m = Lp / R and one block, so butterfly k
// reads x[k + s*m]; results go to buf in the stage's usual places.
template <int R, bool PRE, typename V>
__device__ __forceinline__ void fft_stage0_global(V* __restrict__ buf, const V* __restrict__ src,
                                                  const V* __restrict__ pre, int cols, int m,
                                                  const V* __restrict__ tw, int tid, int nthreads) {
    using RX = Radix<R>;
    for (int k = tid; k < m; k += nthreads) {
        V a[R];
#pragma unroll
        for (int s = 0; s < R; s++) {
            const int idx = k + s * m;
            V x = mk<V>(0.f, 0.f);
            if (idx < cols) {
                x = __ldcg(src + idx);
                if (PRE) x = cmul(x, __ldg(pre + idx));
            }
            a[s] = x;
        }
        RX::fwd(a);
#pragma unroll
        for (int q = 1; q < R; q++) a[RX::out_reg(q)] = cmul(a[RX::out_reg(q)], __ldg(tw + k + (q - 1) * m));
#pragma unroll
        for (int q = 0; q < R; q++) buf[k + q * m] = a[RX::out_reg(q)];
    }
}

// Radices the row kernel supports; the plan only emits these.  A kernel
// compiled for blocks of up to 1024 threads (64 registers a thread) holds
// radices up to 16; the 512-thread variant (128 registers) all of them.
#define GBSP_RADIX_LIST(X) \
    X(2) X(3) X(4) X(5) X(7) X(8) X(9) X(12) X(15) X(16) X(20) X(21) X(24) X(25) X(28) X(32) X(35) X(40)

__host__ __device__ constexpr bool radix_supported(int r) {
    return r == 2 || r == 3 || r == 4 || r == 5 || r == 7 || r == 8 || r == 9 || r == 12 || r == 15 ||
           r == 16 || r == 20 || r == 21 || r == 24 || r == 25 || r == 28 || r == 32 || r == 35 || r == 40;
}
constexpr int MAX_RADIX_NT1024 = 16;
constexpr int MAX_RADIX_NT512 = 40;

// Runs one stage of radix R; returns false (and touches nothing) when this
// kernel was not compiled for R, so a plan/kernel mismatch is reported
// instead of silently skipping the stage.
template <int MODE, int MAXR, bool TWG, typename V>
__device__ __forceinline__ bool fft_stage_dispatch(int R, V* buf, int Lp, int m, uint32_t magic,
                                                   const V* tw, const V* filt, int tid, int nthreads) {
    switch (R) {
#define GBSP_STAGE_CASE(r)                                                                   \
        case r:                                                                              \
            if constexpr (r <= MAXR) {                                                       \
                fft_stage<r, MODE, TWG>(buf, Lp, m, magic, tw, filt, tid, nthreads);         \
                return true;                                                                 \
            }                                                                                \
            return false;
        GBSP_RADIX_LIST(GBSP_STAGE_CASE)
#undef GBSP_STAGE_CASE
        default: return false;
    }
}

template <int MAXR, bool PRE, typename V>
__device__ __forceinline__ bool fft_stage0_global_dispatch(int R, V* buf, const V* src, const V* pre, int cols,
                                                           int m, const V* tw, int tid, int nthreads) {
    switch (R) {
#define GBSP_STAGE0_CASE(r)                                                                  \
        case r:                                                                              \
            if constexpr (r <= MAXR) {                                                       \
                fft_stage0_global<r, PRE>(buf, src, pre, cols, m, tw, tid, nthreads);        \
                return true;                                                                 \
            }                                                                                \
            return false;
        GBSP_RADIX_LIST(GBSP_STAGE0_CASE)
#undef GBSP_STAGE0_CASE
        default: return false;
    }
}

}  // namespace gbsp
