// fft_device.cuh -- device building blocks of the GB300 FFT engine: complex
// helpers, register butterflies (radix 2/4/8/16 and odd primes 3..31), the
// shared-memory Stockham tile (tile_body) and the register-resident tile
// (tile_body_reg), and the element prologue/epilogue of fused Rader and
// Bluestein passes.  Included by the kernel translation units.
//
// The tiles replace the reference's recursive kf_work (kfft_work.c:1-59) and
// its butterflies kf_bfly2/3/4/5 and std_method_eval (kfft_bfly.c:1-152,
// kfft_generic.c:9-36); the prologue/epilogue wiring replaces
// rader_method_eval/kfft_part_convolution (kfft_rader.c).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cuda_fp16.h>

#include <cstring>
#include <type_traits>

#include "engine.cuh"

namespace kfft {

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
    return uint32_t((uint64_t(__umulhi(n, f.m)) + n) >> f.s);
}

#if defined(KFFT_HALF_SCALAR)
// FP32: Blackwell's paired FP32 instructions work on a float2 at once (one
// instruction for both parts, each rounded as the scalar operation would be)
__device__ __forceinline__ vec2_t cadd(vec2_t a, vec2_t b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ vec2_t csub(vec2_t a, vec2_t b) {
    return __ffma2_rn(b, make_float2(-1.f, -1.f), a);  // a - b, one rounding
}
__device__ __forceinline__ vec2_t cscale(vec2_t a, real_t s) { return __fmul2_rn(a, make_float2(s, s)); }
#else
__device__ __forceinline__ vec2_t cadd(vec2_t a, vec2_t b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ vec2_t csub(vec2_t a, vec2_t b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ vec2_t cscale(vec2_t a, real_t s) { return {a.x * s, a.y * s}; }
#endif
__device__ __forceinline__ vec2_t cmul(vec2_t a, vec2_t b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ vec2_t rot(vec2_t a) {
    return INV ? vec2_t{-a.y, a.x} : vec2_t{a.y, -a.x};
}

// one padding slot per 128 bytes of shared memory
#if defined(KFFT_HALF_SCALAR)
constexpr uint32_t kPadShift = 4;
#else
constexpr uint32_t kPadShift = 3;
#endif
__device__ __forceinline__ uint32_t pad(uint32_t i) { return i + (i >> kPadShift); }


// resident CTAs per SM the fused-I/O kernels are compiled for (register cap
// 65536 / (256 * blocks)): three for FP32, two for FP64 (more would spill)
#ifndef KFFT_REG_MINBLOCKS
#if defined(KFFT_HALF_SCALAR)
#define KFFT_REG_MINBLOCKS 3
#else
#define KFFT_REG_MINBLOCKS 2
#endif
#endif

// global loads each thread keeps in flight in the tile load phase
#if defined(KFFT_HALF_SCALAR)
constexpr int kLoadUnroll = 8;
#else
constexpr int kLoadUnroll = 4;
#endif

// ---------------------------------------------------------------------------
// compile-time trigonometry for the odd-prime butterflies: cos/sin(2 pi m / P)
// from an exact octant reduction and Taylor series on [0, pi/4].
// ---------------------------------------------------------------------------
constexpr double kPi = 3.14159265358979323846264338327950288;

constexpr double taylor_sin(double x) {
    double x2 = x * x, term = x, sum = x;
    for (int k = 1; k < 14; ++k) {
        term *= -x2 / double((2 * k) * (2 * k + 1));
        sum += term;
    }
    return sum;
}
constexpr double taylor_cos(double x) {
    double x2 = x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k < 14; ++k) {
        term *= -x2 / double((2 * k - 1) * (2 * k));
        sum += term;
    }
    return sum;
}
// returns cos (want_sin=false) or sin of 2*pi*m/P
constexpr double trig_ratio(long m, long P, bool want_sin) {
    m %= P;
    if (m < 0) m += P;
    long t = (8 * m) / P;          // octant 0..7
    long r = 8 * m - t * P;        // remainder: angle = (t + r/P) * pi/4
    double a = kPi / 4.0 * double(r) / double(P);
    // for odd octants use the complement to keep the argument in [0, pi/4]
    double s0 = 0, c0 = 0;
    if (t & 1) {
        double b = kPi / 4.0 * double(P - r) / double(P);
        s0 = taylor_sin(b);
        c0 = taylor_cos(b);
        // angle = (t+1)*pi/4 - b
        long q = (t + 1) / 2;  // multiples of pi/2
        double sv = 0, cv = 0;
        // sin(q*pi/2 - b), cos(q*pi/2 - b)
        switch (q & 3) {
            case 0: sv = -s0; cv = c0; break;
            case 1: sv = c0; cv = s0; break;
            case 2: sv = s0; cv = -c0; break;
            default: sv = -c0; cv = -s0; break;
        }
        return want_sin ? sv : cv;
    } else {
        s0 = taylor_sin(a);
        c0 = taylor_cos(a);
        long q = t / 2;
        double sv = 0, cv = 0;
        // sin(q*pi/2 + a), cos(q*pi/2 + a)
        switch (q & 3) {
            case 0: sv = s0; cv = c0; break;
            case 1: sv = c0; cv = -s0; break;
            case 2: sv = -s0; cv = -c0; break;
            default: sv = -c0; cv = s0; break;
        }
        return want_sin ? sv : cv;
    }
}


// ---------------------------------------------------------------------------
// butterflies (in registers)
// ---------------------------------------------------------------------------
template <bool INV>
__device__ __forceinline__ void dft2(vec2_t& a, vec2_t& b) {
    vec2_t t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(vec2_t& a0, vec2_t& a1, vec2_t& a2, vec2_t& a3) {
    vec2_t s0 = cadd(a0, a2), s1 = csub(a0, a2);
    vec2_t s2 = cadd(a1, a3), s3 = rot<INV>(csub(a1, a3));
    a0 = cadd(s0, s2);
    a2 = csub(s0, s2);
    a1 = cadd(s1, s3);
    a3 = csub(s1, s3);
}

constexpr double kR2 = 0.70710678118654752440084436210484903928;
constexpr double kC8 = 0.92387953251128675612818318939678828682;  // cos(pi/8)
constexpr double kS8 = 0.38268343236508977172845998403039886676;  // sin(pi/8)

// multiply by W_8^k (forward W = exp(-2 pi i/8))
template <bool INV, int K>
__device__ __forceinline__ vec2_t w8(vec2_t a) {
    const real_t r = real_t(kR2);
    if constexpr (K == 0) return a;
    else if constexpr (K == 2) return rot<INV>(a);
    else if constexpr (K == 1) {
        // (1 -+ i)/sqrt2 * a
        return INV ? vec2_t{(a.x - a.y) * r, (a.x + a.y) * r}
                   : vec2_t{(a.x + a.y) * r, (a.y - a.x) * r};
    } else {  // K == 3: (-1 -+ i)/sqrt2
        return INV ? vec2_t{-(a.x + a.y) * r, (a.x - a.y) * r}
                   : vec2_t{(a.y - a.x) * r, -(a.x + a.y) * r};
    }
}

template <bool INV>
__device__ __forceinline__ void dft8(vec2_t* v) {
    // radix-2 first (stride 4), twiddle, then two radix-4
    for (int i = 0; i < 4; ++i) dft2<INV>(v[i], v[i + 4]);
    v[5] = w8<INV, 1>(v[5]);
    v[6] = w8<INV, 2>(v[6]);
    v[7] = w8<INV, 3>(v[7]);
    dft4<INV>(v[0], v[1], v[2], v[3]);
    dft4<INV>(v[4], v[5], v[6], v[7]);
    // outputs: v[i] -> X[2i], v[4+i] -> X[2i+1]
    vec2_t t[8];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        t[2 * i] = v[i];
        t[2 * i + 1] = v[4 + i];
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = t[i];
}

// multiply by W_16^k, k in 0..9
template <bool INV>
__device__ __forceinline__ vec2_t w16(vec2_t a, int k) {
    const real_t c8 = real_t(kC8), s8 = real_t(kS8), r = real_t(kR2);
    real_t wr, wi;
    switch (k) {
        case 1: wr = c8; wi = -s8; break;
        case 2: wr = r; wi = -r; break;
        case 3: wr = s8; wi = -c8; break;
        case 4: return rot<INV>(a);
        case 6: wr = -r; wi = -r; break;
        case 9: wr = -c8; wi = s8; break;
        default: return a;
    }
    if (INV) wi = -wi;
    return {a.x * wr - a.y * wi, a.x * wi + a.y * wr};
}

template <bool INV>
__device__ __forceinline__ void dft16(vec2_t* v) {
    // 4 radix-4 over stride 4, twiddle W16^(n1*k2), 4 radix-4, transpose
#pragma unroll
    for (int i = 0; i < 4; ++i) dft4<INV>(v[i], v[i + 4], v[i + 8], v[i + 12]);
#pragma unroll
    for (int i = 1; i < 4; ++i)
#pragma unroll
        for (int k = 1; k < 4; ++k) v[i + 4 * k] = w16<INV>(v[i + 4 * k], i * k);
#pragma unroll
    for (int k = 0; k < 4; ++k) dft4<INV>(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    vec2_t t[16];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int i = 0; i < 4; ++i) t[k + 4 * i] = v[4 * k + i];
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = t[i];
}

// odd prime P: symmetric-pair DFT, (P-1)^2 real multiply-adds.  The cosines
// and sines are template-level constant expressions, so they become
// instruction immediates rather than a table in memory.
template <int P, int K, int N, int H>
struct OddAcc {
    __device__ static __forceinline__ void run(const vec2_t* s, const vec2_t* d, vec2_t& a,
                                               vec2_t& b) {
        constexpr real_t cc = real_t(trig_ratio(long(N) * K, P, false));
        constexpr real_t ss = real_t(trig_ratio(long(N) * K, P, true));
        a.x += s[N - 1].x * cc;
        a.y += s[N - 1].y * cc;
        b.x += d[N - 1].x * ss;
        b.y += d[N - 1].y * ss;
        if constexpr (N < H) OddAcc<P, K, N + 1, H>::run(s, d, a, b);
    }
};

template <int P, bool INV, int K, int H>
struct OddOut {
    __device__ static __forceinline__ void run(vec2_t x0, const vec2_t* s, const vec2_t* d,
                                               vec2_t* v) {
        vec2_t a = x0, b = {real_t(0), real_t(0)};
        OddAcc<P, K, 1, H>::run(s, d, a, b);
        // forward: X_k = a - i b, X_{P-k} = a + i b; inverse swaps
        const vec2_t ib = {-b.y, b.x};
        if (INV) {
            v[K] = cadd(a, ib);
            v[P - K] = csub(a, ib);
        } else {
            v[K] = csub(a, ib);
            v[P - K] = cadd(a, ib);
        }
        if constexpr (K < H) OddOut<P, INV, K + 1, H>::run(x0, s, d, v);
    }
};

template <int P, bool INV>
__device__ __forceinline__ void dft_odd(vec2_t* v) {
    constexpr int H = (P - 1) / 2;
    vec2_t s[H], d[H];
    const vec2_t x0 = v[0];
    vec2_t sum = v[0];
#pragma unroll
    for (int n = 1; n <= H; ++n) {
        s[n - 1] = cadd(v[n], v[P - n]);
        d[n - 1] = csub(v[n], v[P - n]);
        sum = cadd(sum, s[n - 1]);
    }
    OddOut<P, INV, 1, H>::run(x0, s, d, v);
    v[0] = sum;
}

template <int P, bool INV>
__device__ __forceinline__ void dft(vec2_t* v);

// ---------------------------------------------------------------------------
// composite radices 6, 9, 10, 12, 14, 15: a P = A*B point DFT in registers
// from A-point and B-point butterflies, so a mixed-radix tile runs fewer
// inner stages (each stage is a shared-memory round trip and a barrier).
// Coprime A, B use the Good-Thomas map (input n = (B n1 + A n2) mod P,
// output k = (B (B^-1 mod A) k1 + A (A^-1 mod B) k2) mod P, no twiddles);
// 9 = 3*3 uses Cooley-Tukey (n = 3 n1 + n2, k = k1 + 3 k2) with the
// twiddles W_9^(n2 k1) as instruction immediates.  Every index is a
// template constant, so the values stay in registers.
// ---------------------------------------------------------------------------
template <int I, int N, class F>
__device__ __forceinline__ void static_for(F&& f) {
    if constexpr (I < N) {
        f(std::integral_constant<int, I>{});
        static_for<I + 1, N>(f);
    }
}

constexpr int cgcd(int a, int b) { return b == 0 ? a : cgcd(b, a % b); }
// inverse of a modulo m (gcd(a, m) = 1)
constexpr int cinv(int a, int m) {
    for (int x = 1; x < m; ++x)
        if ((a * x) % m == 1) return x;
    return 1 % m;
}

// a * W_P^E (forward W = exp(-2 pi i / P)), E taken modulo P; quarter turns
// are exact rotations
template <int P, int E, bool INV>
__device__ __forceinline__ vec2_t wmul_const(vec2_t a) {
    constexpr int e = ((E % P) + P) % P;
    if constexpr (e == 0) {
        return a;
    } else if constexpr ((4 * e) % P == 0) {
        constexpr int q = (4 * e) / P;  // quarter turns, 1..3
        if constexpr (q == 2) return vec2_t{-a.x, -a.y};
        else if constexpr (q == 1) return rot<INV>(a);
        else return rot<!INV>(a);
    } else {
        constexpr real_t c = real_t(trig_ratio(e, P, false));
        constexpr real_t s = real_t(trig_ratio(e, P, true));
        constexpr real_t wi = INV ? s : -s;  // W^e = cos - i sin (forward)
        return {a.x * c - a.y * wi, a.x * wi + a.y * c};
    }
}

template <int A, int B, bool INV>
__device__ __forceinline__ void dft_composite(vec2_t* v) {
    constexpr int P = A * B;
    constexpr bool kPfa = cgcd(A, B) == 1;
    vec2_t t[P];  // t[n2 * A + k1]
    static_for<0, B>([&](auto n2c) {
        constexpr int n2 = decltype(n2c)::value;
        vec2_t a[A];
        static_for<0, A>([&](auto n1c) {
            constexpr int n1 = decltype(n1c)::value;
            constexpr int n = kPfa ? (B * n1 + A * n2) % P : B * n1 + n2;
            a[n1] = v[n];
        });
        dft<A, INV>(a);
        static_for<0, A>([&](auto k1c) {
            constexpr int k1 = decltype(k1c)::value;
            if constexpr (kPfa) t[n2 * A + k1] = a[k1];
            else t[n2 * A + k1] = wmul_const<P, n2 * k1, INV>(a[k1]);
        });
    });
    static_for<0, A>([&](auto k1c) {
        constexpr int k1 = decltype(k1c)::value;
        vec2_t b[B];
        static_for<0, B>([&](auto n2c) {
            constexpr int n2 = decltype(n2c)::value;
            b[n2] = t[n2 * A + k1];
        });
        dft<B, INV>(b);
        static_for<0, B>([&](auto k2c) {
            constexpr int k2 = decltype(k2c)::value;
            constexpr int k = kPfa ? (B * cinv(B % A, A) * k1 + A * cinv(A % B, B) * k2) % P
                                   : k1 + A * k2;
            v[k] = b[k2];
        });
    });
}

template <int P, bool INV>
__device__ __forceinline__ void dft(vec2_t* v) {
    if constexpr (P == 2) dft2<INV>(v[0], v[1]);
    else if constexpr (P == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
    else if constexpr (P == 8) dft8<INV>(v);
    else if constexpr (P == 16) dft16<INV>(v);
    else if constexpr (P == 6) dft_composite<2, 3, INV>(v);
    else if constexpr (P == 9) dft_composite<3, 3, INV>(v);
    else if constexpr (P == 10) dft_composite<2, 5, INV>(v);
    else if constexpr (P == 12) dft_composite<4, 3, INV>(v);
    else if constexpr (P == 14) dft_composite<2, 7, INV>(v);
    else if constexpr (P == 15) dft_composite<3, 5, INV>(v);
    else dft_odd<P, INV>(v);
}

// ---------------------------------------------------------------------------
// the pass kernel
// ---------------------------------------------------------------------------
struct InnerStep {
    FastDiv div_m, div_ns;
    uint32_t m, ns, twstride;
};

template <int P, bool INV>
__device__ __forceinline__ void inner_pass(const vec2_t* __restrict__ src, vec2_t* __restrict__ dst,
                                           uint32_t R, uint32_t C, const InnerStep& st,
                                           const vec2_t* __restrict__ tw) {
    const uint32_t items = C * st.m;
    for (uint32_t it = threadIdx.x; it < items; it += blockDim.x) {
        const uint32_t c = fdiv(it, st.div_m);
        const uint32_t jj = it - c * st.m;
        const uint32_t blk = fdiv(jj, st.div_ns);
        const uint32_t kk = jj - blk * st.ns;
        const uint32_t base = c * R;
        vec2_t v[P];
#pragma unroll
        for (int q = 0; q < P; ++q) v[q] = src[pad(base + jj + q * st.m)];
        if (st.ns > 1) {
            const uint32_t step = kk * st.twstride;
#pragma unroll
            for (int q = 1; q < P; ++q) v[q] = cmul(v[q], __ldg(&tw[q * step]));
        }
        dft<P, INV>(v);
        const uint32_t ob = base + blk * st.ns * P + kk;
#pragma unroll
        for (int q = 0; q < P; ++q) dst[pad(ob + q * st.ns)] = v[q];
    }
}

template <bool INV, bool BIG>
__device__ __forceinline__ void run_inner(int P, const vec2_t* src, vec2_t* dst, uint32_t R,
                                          uint32_t C, const InnerStep& st, const vec2_t* tw) {
    if constexpr (BIG) {
        switch (P) {
            case 17: inner_pass<17, INV>(src, dst, R, C, st, tw); return;
            case 19: inner_pass<19, INV>(src, dst, R, C, st, tw); return;
            case 23: inner_pass<23, INV>(src, dst, R, C, st, tw); return;
            case 29: inner_pass<29, INV>(src, dst, R, C, st, tw); return;
            case 31: inner_pass<31, INV>(src, dst, R, C, st, tw); return;
            default: break;
        }
    }
    switch (P) {
        case 2: inner_pass<2, INV>(src, dst, R, C, st, tw); break;
        case 3: inner_pass<3, INV>(src, dst, R, C, st, tw); break;
        case 4: inner_pass<4, INV>(src, dst, R, C, st, tw); break;
        case 5: inner_pass<5, INV>(src, dst, R, C, st, tw); break;
        case 7: inner_pass<7, INV>(src, dst, R, C, st, tw); break;
        case 6: inner_pass<6, INV>(src, dst, R, C, st, tw); break;
        case 8: inner_pass<8, INV>(src, dst, R, C, st, tw); break;
        case 9: inner_pass<9, INV>(src, dst, R, C, st, tw); break;
        case 10: inner_pass<10, INV>(src, dst, R, C, st, tw); break;
        case 11: inner_pass<11, INV>(src, dst, R, C, st, tw); break;
        case 12: inner_pass<12, INV>(src, dst, R, C, st, tw); break;
        case 13: inner_pass<13, INV>(src, dst, R, C, st, tw); break;
        case 14: inner_pass<14, INV>(src, dst, R, C, st, tw); break;
        case 15: inner_pass<15, INV>(src, dst, R, C, st, tw); break;
        case 16: inner_pass<16, INV>(src, dst, R, C, st, tw); break;
        default: break;
    }
}

__device__ __forceinline__ vec2_t load_elem(const PassDesc& d, uint32_t b, uint32_t n) {
    switch (d.pro_op) {
        case PRO_CHIRP:
            if (n < d.pro_bound)
                return cmul(__ldcg(&d.in[b * d.in_bs + uint64_t(n) * d.in_es]), __ldg(&d.pro_tab[n]));
            return {real_t(0), real_t(0)};
        case PRO_GATHER:
            return __ldcg(&d.in[b * d.in_bs + uint64_t(__ldg(&d.pro_perm[n])) * d.in_es]);
        default:
            return __ldcg(&d.in[b * d.in_bs + uint64_t(n) * d.in_es]);
    }
}

__device__ __forceinline__ void store_elem(const PassDesc& d, uint32_t b, uint32_t k, vec2_t v) {
    switch (d.epi_op) {
        case EPI_MUL:
            d.out[b * d.out_bs + uint64_t(k) * d.out_es] = cmul(v, __ldg(&d.epi_tab[k]));
            break;
        case EPI_CHIRP:
            if (k < d.epi_bound)
                d.out[b * d.out_bs + uint64_t(k) * d.out_es] =
                    cscale(cmul(v, __ldg(&d.epi_tab[k])), d.scale);
            break;
        case EPI_RADER_FWD:
            // spectrum of the gathered sequence times the kernel spectrum; bin 0
            // is sum_{n>=1} x_n, so X_0 = x_0 + v is saved with x_0 per sequence
            d.out[b * d.out_bs + uint64_t(k) * d.out_es] = cmul(v, __ldg(&d.epi_tab[k]));
            if (k == 0) {
                const vec2_t x0 = __ldcg(&d.aux_in[b * d.aux_in_bs]);
                d.aux_out[2 * uint64_t(b)] = x0;
                d.aux_out[2 * uint64_t(b) + 1] = cadd(x0, v);
            }
            break;
        case EPI_MUL_OUT: {
            const uint64_t i = b * d.out_bs + uint64_t(k) * d.out_es;
            d.out[i] = cscale(cmul(v, __ldcg(&d.epi_tab[i])), d.scale);
            break;
        }
        case EPI_RADER_INV: {
            // X[g^-k] = x_0 + c_k, and X_0 from the saved pair; never reads the input,
            // so the transform may run in place
            const vec2_t x0 = __ldcg(&d.aux_in[2 * uint64_t(b)]);
            const uint32_t idx = __ldg(&d.epi_perm[k]);
            vec2_t* o = d.aux_out + b * d.aux_out_bs;
            o[uint64_t(idx) * d.aux_out_es] = cscale(cadd(v, x0), d.scale);
            if (k == 0) o[0] = cscale(__ldcg(&d.aux_in[2 * uint64_t(b) + 1]), d.scale);
            break;
        }
        default:
            d.out[b * d.out_bs + uint64_t(k) * d.out_es] = cscale(v, d.scale);
            break;
    }
}

struct PassExtra {
    InnerStep step[kMaxInnerRadices];
};

PassExtra make_extra(const PassDesc& d);

// The outer twiddle W_N^e of a pass (e < N): the product of the two-level
// table's entries W_N^(e >> tw_shift << tw_shift) and W_N^(e mod 2^tw_shift).
__device__ __forceinline__ vec2_t outer_w(const PassDesc& d, uint32_t e) {
    const uint32_t mask = (1u << d.tw_shift) - 1u;
    return cmul(__ldg(&d.tw_hi[e >> d.tw_shift]), __ldg(&d.tw_lo[e & mask]));
}

// One tile of one pass: C lanes of the length-R sub-FFT, shared-memory staged.
template <bool INV, bool BIG>
__device__ __forceinline__ void tile_body(const PassDesc& d, const PassExtra& x, uint32_t tile,
                                          vec2_t* bufA) {
    const uint32_t tile_elems = d.C * d.R;
    vec2_t* bufB = bufA + pad(tile_elems) + 1;
    const uint32_t total_lanes = d.batch * d.lanes_j;
    const uint32_t lane0 = tile * d.C;

    // ---- load: kLoadUnroll independent loads per thread in flight ---------
    for (uint32_t base = threadIdx.x; base < tile_elems; base += kLoadUnroll * blockDim.x) {
        vec2_t v[kLoadUnroll];
        uint32_t slot[kLoadUnroll];
        uint32_t twe[kLoadUnroll];
#pragma unroll
        for (int u = 0; u < kLoadUnroll; ++u) {
            const uint32_t idx = base + u * blockDim.x;
            v[u] = {real_t(0), real_t(0)};
            slot[u] = 0xffffffffu;
            twe[u] = 0;
            if (idx >= tile_elems) continue;
            uint32_t c, r;
            if (d.load_mode == MODE_LANE) {
                r = fdiv(idx, d.div_C);
                c = idx - r * d.C;
            } else {
                c = fdiv(idx, d.div_R);
                r = idx - c * d.R;
            }
            slot[u] = pad(c * d.R + r);
            const uint32_t g = lane0 + c;
            if (g < total_lanes) {
                uint32_t b, j;
                if (d.order == ORDER_J) {
                    b = fdiv(g, d.div_lanes_j);
                    j = g - b * d.lanes_j;
                } else {
                    j = fdiv(g, d.div_batch);
                    b = g - j * d.batch;
                }
                v[u] = load_elem(d, b, j + r * d.lanes_j);
                if (d.Ns > 1) {
                    const uint32_t kq = fdiv(j, d.div_Ns);
                    const uint32_t k = j - kq * d.Ns;
                    twe[u] = uint32_t(uint64_t(r) * k * d.tw_mul);
                }
            }
        }
        if (d.Ns > 1) {
#pragma unroll
            for (int u = 0; u < kLoadUnroll; ++u) v[u] = cmul(v[u], outer_w(d, twe[u]));
        }
#pragma unroll
        for (int u = 0; u < kLoadUnroll; ++u)
            if (slot[u] != 0xffffffffu) bufA[slot[u]] = v[u];
    }
    __syncthreads();

    // ---- inner sub-FFT of length R ------------------------------------
    vec2_t* src = bufA;
    vec2_t* dst = bufB;
    for (int p = 0; p < d.nrad; ++p) {
        run_inner<INV, BIG>(d.rad[p], src, dst, d.R, d.C, x.step[p], d.tw_inner);
        __syncthreads();
        vec2_t* t = src;
        src = dst;
        dst = t;
    }

    // ---- store ----------------------------------------------------------
    for (uint32_t idx = threadIdx.x; idx < tile_elems; idx += blockDim.x) {
        uint32_t c, r;
        if (d.store_mode == MODE_LANE) {
            r = fdiv(idx, d.div_C);
            c = idx - r * d.C;
        } else {
            c = fdiv(idx, d.div_R);
            r = idx - c * d.R;
        }
        const uint32_t g = lane0 + c;
        if (g >= total_lanes) continue;
        uint32_t b, j;
        if (d.order == ORDER_J) {
            b = fdiv(g, d.div_lanes_j);
            j = g - b * d.lanes_j;
        } else {
            j = fdiv(g, d.div_batch);
            b = g - j * d.batch;
        }
        const uint32_t blk = fdiv(j, d.div_Ns);
        const uint32_t k = j - blk * d.Ns;
        const uint32_t outk = blk * d.Ns * d.R + k + r * d.Ns;
        store_elem(d, b, outk, src[pad(c * d.R + r)]);
    }
}

// ---------------------------------------------------------------------------
// register-resident tile: each inner pass moves its butterflies' values
// through registers; the first pass reads global memory directly (with the
// prologue and the outer twiddle), the last writes global memory directly
// (with the epilogue), and only the exchanges between inner passes go through
// one shared-memory buffer (read all, barrier, write all, barrier).
// ---------------------------------------------------------------------------
enum : int { IO_SMEM = 0, IO_GLOBAL = 1 };

// v[q] *= W^(q*step) for q = 1..P-1, W^i = tw[i].  FP64 loads every factor
// (the FP64 pipe, not the loads, bounds it).  FP32 loads the four anchors
// W^(step), W^(2 step), W^(4 step), W^(8 step) and forms the others as
// products of at most four anchors: a quarter of the table loads, which were
// the L1 bottleneck, for a few ulp of extra rounding.
template <int P>
__device__ __forceinline__ void apply_inner_twiddles(vec2_t* v, const vec2_t* __restrict__ tw,
                                                     uint32_t step) {
#if defined(KFFT_HALF_SCALAR)
    if constexpr (P >= 4) {
        vec2_t a[4];
#pragma unroll
        for (int b = 0; b < 4; ++b)
            if ((1 << b) < P) a[b] = __ldg(&tw[(1u << b) * step]);
#pragma unroll
        for (int q = 1; q < P; ++q) {
            vec2_t w = {real_t(1), real_t(0)};
            bool first = true;
#pragma unroll
            for (int b = 0; b < 4; ++b)
                if (q & (1 << b)) {
                    w = first ? a[b] : cmul(w, a[b]);
                    first = false;
                }
            v[q] = cmul(v[q], w);
        }
        return;
    }
#endif
#pragma unroll
    for (int q = 1; q < P; ++q) v[q] = cmul(v[q], __ldg(&tw[q * step]));
}

// The P inputs of one butterfly of the first inner pass, straight from global
// memory, through the prologue (chirp product or gather, if any).
template <int P>
__device__ __forceinline__ void prologue_load(const PassDesc& d, uint32_t bs, uint32_t j,
                                              uint32_t jj, uint32_t m, vec2_t* v) {
    const uint64_t base = uint64_t(bs) * d.in_bs;
    const uint64_t step = uint64_t(m) * d.lanes_j * d.in_es;
    const uint64_t first = uint64_t(j + jj * d.lanes_j) * d.in_es;
    switch (d.pro_op) {
        case PRO_CHIRP:
#pragma unroll
            for (int q = 0; q < P; ++q) {
                const uint32_t n = j + (jj + q * m) * d.lanes_j;
                v[q] = (n < d.pro_bound) ? cmul(__ldcg(&d.in[base + first + q * step]), __ldg(&d.pro_tab[n]))
                                         : vec2_t{real_t(0), real_t(0)};
            }
            break;
        case PRO_GATHER:
#pragma unroll
            for (int q = 0; q < P; ++q) {
                const uint32_t n = j + (jj + q * m) * d.lanes_j;
                v[q] = __ldcg(&d.in[base + uint64_t(__ldg(&d.pro_perm[n])) * d.in_es]);
            }
            break;
        default:
#pragma unroll
            for (int q = 0; q < P; ++q) v[q] = __ldcg(&d.in[base + first + q * step]);
            break;
    }
}

// The outer twiddle W_{Ns*R}^{r*k} of the first inner pass (applied in groups
// of four in FP64 to bound the registers held by table loads).
template <int P>
__device__ __forceinline__ void outer_twiddle(const PassDesc& d, uint32_t j, uint32_t jj,
                                              uint32_t m, vec2_t* v) {
    if (d.Ns > 1) {
        const uint32_t kq = fdiv(j, d.div_Ns);
        const uint32_t k = j - kq * d.Ns;
        const uint32_t e0 = uint32_t(uint64_t(jj) * k * d.tw_mul);
        const uint32_t es = uint32_t(uint64_t(m) * k * d.tw_mul);
#if defined(KFFT_HALF_SCALAR)
        if constexpr (P >= 4) {
            // FP32: W^(e0 + q es) from the base W^(e0) and the anchors W^(2^b es):
            // ten table loads per butterfly instead of 2P (the L1 bottleneck)
            auto tw2 = [&](uint32_t e) { return outer_w(d, e); };
            const vec2_t w0 = tw2(e0);
            vec2_t a[4];
#pragma unroll
            for (int b = 0; b < 4; ++b)
                if ((1 << b) < P) a[b] = tw2((1u << b) * es);
            v[0] = cmul(v[0], w0);
#pragma unroll
            for (int q = 1; q < P; ++q) {
                vec2_t w = w0;
#pragma unroll
                for (int b = 0; b < 4; ++b)
                    if (q & (1 << b)) w = cmul(w, a[b]);
                v[q] = cmul(v[q], w);
            }
            return;
        }
#endif
#pragma unroll
        for (int g = 0; g < P; g += 4) {
            vec2_t w[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (g + u < P) w[u] = outer_w(d, e0 + uint32_t(g + u) * es);  // < N, no wrap
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (g + u < P) v[g + u] = cmul(v[g + u], w[u]);
        }
    }
}

// Loads the P inputs of one butterfly of the first inner pass straight from
// global memory: prologue, then the outer twiddle.
template <int P>
__device__ __forceinline__ void fused_load(const PassDesc& d, uint32_t bs, uint32_t j, uint32_t jj,
                                           uint32_t m, vec2_t* v) {
    prologue_load<P>(d, bs, j, jj, m, v);
    outer_twiddle<P>(d, j, jj, m, v);
}

// Stores the P outputs of one butterfly of the last inner pass straight to
// global memory through the epilogue.
template <int P>
__device__ __forceinline__ void fused_store(const PassDesc& d, uint32_t bs, uint32_t j, uint32_t ob,
                                            uint32_t ns, const vec2_t* v) {
    const uint32_t blo = fdiv(j, d.div_Ns);
    const uint32_t ko = j - blo * d.Ns;
    const uint32_t base = blo * d.Ns * d.R + ko;
    if (d.epi_op == EPI_NONE) {
        vec2_t* o = d.out + uint64_t(bs) * d.out_bs;
        const uint64_t es = d.out_es;
#pragma unroll
        for (int q = 0; q < P; ++q) o[uint64_t(base + (ob + q * ns) * d.Ns) * es] = cscale(v[q], d.scale);
    } else {
#pragma unroll
        for (int q = 0; q < P; ++q) store_elem(d, bs, base + (ob + q * ns) * d.Ns, v[q]);
    }
}

// One inner Stockham pass of radix P over the tile: each thread takes one
// butterfly at a time from `src` (global memory on the first pass, else a
// shared buffer) and writes it to `dst` (global memory on the last pass, else
// the other shared buffer).
template <int P, bool INV>
__device__ __forceinline__ void fused_pass(const PassDesc& d, const InnerStep& st,
                                           const vec2_t* src, vec2_t* dst, uint32_t lane0,
                                           uint32_t total, int sio, int dio) {
    const uint32_t m = st.m;
    const uint32_t items = d.C * m;
    const bool cfast = (sio == IO_GLOBAL) ? (d.load_mode == MODE_LANE)
                                          : ((dio == IO_GLOBAL) ? (d.store_mode == MODE_LANE) : false);
    for (uint32_t it = threadIdx.x; it < items; it += blockDim.x) {
        uint32_t c, jj;
        if (cfast) {
            jj = fdiv(it, d.div_C);
            c = it - jj * d.C;
        } else {
            c = fdiv(it, st.div_m);
            jj = it - c * m;
        }
        const uint32_t g = lane0 + c;
        uint32_t bs = 0, j = 0;
        const bool live = g < total;
        if ((sio == IO_GLOBAL || dio == IO_GLOBAL) && live) {
            if (d.order == ORDER_J) {
                bs = fdiv(g, d.div_lanes_j);
                j = g - bs * d.lanes_j;
            } else {
                j = fdiv(g, d.div_batch);
                bs = g - j * d.batch;
            }
        }
        vec2_t v[P];
        if (sio == IO_GLOBAL) {
            if (live) {
                fused_load<P>(d, bs, j, jj, m, v);
            } else {
#pragma unroll
                for (int q = 0; q < P; ++q) v[q] = {real_t(0), real_t(0)};
            }
        } else {
#pragma unroll
            for (int q = 0; q < P; ++q) v[q] = src[c * d.lane_stride + pad(jj + q * m)];
        }
        const uint32_t blk = fdiv(jj, st.div_ns);
        const uint32_t kk = jj - blk * st.ns;
        if (st.ns > 1) apply_inner_twiddles<P>(v, d.tw_inner, kk * st.twstride);
        dft<P, INV>(v);
        const uint32_t ob = blk * st.ns * P + kk;
        if (dio == IO_SMEM) {
#pragma unroll
            for (int q = 0; q < P; ++q) dst[c * d.lane_stride + pad(ob + q * st.ns)] = v[q];
        } else if (live) {
            fused_store<P>(d, bs, j, ob, st.ns, v);
        }
    }
}

#if defined(KFFT_HALF_SCALAR)
// ---------------------------------------------------------------------------
// Tensor-core radix-16 (FP32 build): the 16-point DFT of 8 butterflies at a
// time as a real 16x16 by 16x8 matrix product per real/imaginary part on
// mma.sync.m16n8k16 (FP16 operands, FP32 accumulation).  Operands are split
// into FP16 hi + lo parts and three products are summed (Fh*Xh + Fh*Xl +
// Fl*Xh); each butterfly's inputs are scaled by a power of two so that their
// largest component lies in [0.5, 1), which keeps the lo parts normal.
// Fragment layout (PTX ISA, m16n8k16): lane = 4*g + t; A row-major 16x16:
// a{0,1} = (g, 2t+{0,1}), a{2,3} = (g+8, 2t+{0,1}), a{4,5} = (g, 2t+8+{0,1}),
// a{6,7} = (g+8, 2t+8+{0,1}); B col-major 16x8: b{0,1} = (2t+{0,1}, g),
// b{2,3} = (2t+8+{0,1}, g); C 16x8: c{0,1} = (g, 2t+{0,1}), c{2,3} = (g+8, 2t+{0,1}).
// ---------------------------------------------------------------------------
struct TcFrag {
    uint32_t hi[4], lo[4];
};

__device__ __forceinline__ uint32_t pack_half2(float a, float b) {
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

__device__ __forceinline__ void split_pair(float a, float b, uint32_t& hi, uint32_t& lo) {
    const __half ha = __float2half_rn(a), hb = __float2half_rn(b);
    const float ra = a - __half2float(ha), rb = b - __half2float(hb);
    __half2 h2 = __halves2half2(ha, hb);
    hi = *reinterpret_cast<uint32_t*>(&h2);
    lo = pack_half2(ra, rb);
}

// A fragment of cos (part 0), s*sin (part 1) or -s*sin (part 2) of 2*pi*m*k/16,
// s = -1 forward, +1 inverse
template <bool INV>
__device__ __forceinline__ TcFrag dft16_frag(int part) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int rows[4] = {g, g + 8, g, g + 8};
    const int cols[4] = {2 * t, 2 * t, 2 * t + 8, 2 * t + 8};
    TcFrag f;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float v[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int mk = (rows[r] * (cols[r] + e)) & 15;
            float s, c;
            sincospif(float(mk) / 8.0f, &s, &c);
            const float sgn = INV ? 1.0f : -1.0f;
            v[e] = part == 0 ? c : (part == 1 ? sgn * s : -sgn * s);
        }
        split_pair(v[0], v[1], f.hi[r], f.lo[r]);
    }
    return f;
}

__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// acc += F * X with F = Fh + Fl and X = Xh + Xl (three products), the small
// cross terms first so that they are summed before the large one: 2^24 FP32
// at 6.3e-7 against the FP64 oracle instead of 1.05e-6 with Fh Xh first (a
// fourth product, Fl Xl, changed nothing measurable)
__device__ __forceinline__ void mma_split(float* acc, const TcFrag& F, const uint32_t* xh,
                                          const uint32_t* xl) {
    mma16816(acc, F.lo, xh);
    mma16816(acc, F.hi, xl);
    mma16816(acc, F.hi, xh);
}

// One radix-16 inner pass on tensor cores.  Each warp takes butterflies in
// groups of 8: lane 4g+t loads inputs k = 2t, 2t+1, 2t+8, 2t+9 of butterfly g
// and, after the products, holds outputs g and g+8 of butterflies 2t, 2t+1.
template <bool INV>
__device__ __forceinline__ void tc_pass16(const PassDesc& d, const InnerStep& st,
                                          const vec2_t* src, vec2_t* dst, uint32_t lane0,
                                          uint32_t total, int sio, int dio, const TcFrag& Fr,
                                          const TcFrag& Fi, const TcFrag& Gm) {
    const uint32_t m = st.m;
    const uint32_t items = d.C * m;
    const int lane = threadIdx.x & 31, gq = lane >> 2, tq = lane & 3;
    const uint32_t warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const bool cfast = (sio == IO_GLOBAL) ? (d.load_mode == MODE_LANE)
                                          : ((dio == IO_GLOBAL) ? (d.store_mode == MODE_LANE) : false);
    const int ks[4] = {2 * tq, 2 * tq + 1, 2 * tq + 8, 2 * tq + 9};
    for (uint32_t grp = warp; grp * 8 < items; grp += nwarps) {
        // ---- inputs of butterfly gq --------------------------------------------
        const uint32_t it = grp * 8 + gq;
        vec2_t x[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
        if (it < items) {
            uint32_t c, jj;
            if (cfast) {
                jj = fdiv(it, d.div_C);
                c = it - jj * d.C;
            } else {
                c = fdiv(it, st.div_m);
                jj = it - c * m;
            }
            const uint32_t g = lane0 + c;
            if (sio == IO_GLOBAL) {
                if (g < total) {
                    uint32_t bs, j;
                    if (d.order == ORDER_J) {
                        bs = fdiv(g, d.div_lanes_j);
                        j = g - bs * d.lanes_j;
                    } else {
                        j = fdiv(g, d.div_batch);
                        bs = g - j * d.batch;
                    }
                    const uint32_t kq = fdiv(j, d.div_Ns);
                    const uint32_t kk = j - kq * d.Ns;
                    const uint32_t mask = (1u << d.tw_shift) - 1u;
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const uint32_t r = jj + uint32_t(ks[u]) * m;
                        x[u] = load_elem(d, bs, j + r * d.lanes_j);
                        if (d.Ns > 1) {
                            const uint32_t e = uint32_t(uint64_t(r) * kk * d.tw_mul);
                            x[u] = cmul(x[u], cmul(__ldg(&d.tw_hi[e >> d.tw_shift]),
                                                   __ldg(&d.tw_lo[e & mask])));
                        }
                    }
                }
            } else {
#pragma unroll
                for (int u = 0; u < 4; ++u) x[u] = src[c * d.lane_stride + pad(jj + uint32_t(ks[u]) * m)];
            }
            if (st.ns > 1) {
                const uint32_t blk = fdiv(jj, st.div_ns);
                const uint32_t kk = jj - blk * st.ns;
                const uint32_t step = kk * st.twstride;
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (ks[u]) x[u] = cmul(x[u], __ldg(&d.tw_inner[uint32_t(ks[u]) * step]));
            }
        }
        // ---- per-butterfly power-of-two scale ---------------------------------
        float mx = 0.f;
#pragma unroll
        for (int u = 0; u < 4; ++u) mx = fmaxf(mx, fmaxf(fabsf(x[u].x), fabsf(x[u].y)));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
        int ex = 0;
        if (mx > 0.f) frexpf(mx, &ex);
        const float sc = ldexpf(1.0f, -ex), inv_sc = ldexpf(1.0f, ex);
        uint32_t xrh[2], xrl[2], xih[2], xil[2];
        split_pair(x[0].x * sc, x[1].x * sc, xrh[0], xrl[0]);
        split_pair(x[2].x * sc, x[3].x * sc, xrh[1], xrl[1]);
        split_pair(x[0].y * sc, x[1].y * sc, xih[0], xil[0]);
        split_pair(x[2].y * sc, x[3].y * sc, xih[1], xil[1]);
        // ---- Yr = Fr Xr - Fi Xi, Yi = Fi Xr + Fr Xi ------------------------------
        float yr[4] = {0.f, 0.f, 0.f, 0.f}, yi[4] = {0.f, 0.f, 0.f, 0.f};
        mma_split(yr, Fr, xrh, xrl);
        mma_split(yr, Gm, xih, xil);
        mma_split(yi, Fi, xrh, xrl);
        mma_split(yi, Fr, xih, xil);
        // ---- outputs g and g+8 of butterflies 2t and 2t+1 -------------------------
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const uint32_t n = uint32_t(2 * tq + e);
            const float un = __shfl_sync(0xffffffffu, inv_sc, int(n) * 4);
            const uint32_t ito = grp * 8 + n;
            if (ito >= items) continue;
            uint32_t co, jo;
            if (cfast) {
                jo = fdiv(ito, d.div_C);
                co = ito - jo * d.C;
            } else {
                co = fdiv(ito, st.div_m);
                jo = ito - co * m;
            }
            const uint32_t blk = fdiv(jo, st.div_ns);
            const uint32_t kk = jo - blk * st.ns;
            const uint32_t ob = blk * st.ns * 16 + kk;
            const vec2_t o0 = {yr[e] * un, yi[e] * un};          // output gq
            const vec2_t o1 = {yr[2 + e] * un, yi[2 + e] * un};  // output gq + 8
            if (dio == IO_SMEM) {
                dst[co * d.lane_stride + pad(ob + uint32_t(gq) * st.ns)] = o0;
                dst[co * d.lane_stride + pad(ob + uint32_t(gq + 8) * st.ns)] = o1;
            } else {
                const uint32_t g = lane0 + co;
                if (g >= total) continue;
                uint32_t bs, j;
                if (d.order == ORDER_J) {
                    bs = fdiv(g, d.div_lanes_j);
                    j = g - bs * d.lanes_j;
                } else {
                    j = fdiv(g, d.div_batch);
                    bs = g - j * d.batch;
                }
                const uint32_t blo = fdiv(j, d.div_Ns);
                const uint32_t ko = j - blo * d.Ns;
                const uint32_t base = blo * d.Ns * d.R + ko;
                store_elem(d, bs, base + (ob + uint32_t(gq) * st.ns) * d.Ns, o0);
                store_elem(d, bs, base + (ob + uint32_t(gq + 8) * st.ns) * d.Ns, o1);
            }
        }
    }
}
#endif

// ---------------------------------------------------------------------------
// compile-time tile bodies for power-of-two pass lengths R = 16..4096 (inner
// radices 16,...,16 then 8, 4 or 2).  The same stages as fused_pass, with
// every per-stage constant (butterflies per lane M = R/P, the stride NS of
// the previous radices, the inner twiddle stride) known to the compiler: the
// lane/butterfly split is a shift and a mask, and where padding keeps the P
// shared-memory addresses of a butterfly equally spaced (a stride that is a
// multiple of the pad period, or a unit stride inside one period) they are
// one base plus immediate offsets.
// ---------------------------------------------------------------------------
template <int P, uint32_t R, uint32_t NS, int SIO, int DIO, bool INV>
__device__ __forceinline__ void spec_stage(const PassDesc& d, const vec2_t* __restrict__ src,
                                           vec2_t* __restrict__ dst, uint32_t lane0,
                                           uint32_t total) {
    constexpr uint32_t M = R / P;
    constexpr uint32_t TWS = R / (NS * P);
    constexpr uint32_t kPad = 1u << kPadShift;
    constexpr bool kLinLd = (M % kPad) == 0;
    constexpr bool kLinSt = (NS % kPad) == 0 || (NS == 1 && (kPad % P) == 0 && (R % kPad) == 0);
    constexpr uint32_t kLdStride = M + (M >> kPadShift);
    constexpr uint32_t kStStride = NS + (NS >> kPadShift);
    const uint32_t lstride = d.lane_stride;
    const uint32_t items = d.C * M;
    const bool cfast = (SIO == IO_GLOBAL) ? (d.load_mode == MODE_LANE)
                                          : ((DIO == IO_GLOBAL) ? (d.store_mode == MODE_LANE) : false);
    for (uint32_t it = threadIdx.x; it < items; it += blockDim.x) {
        uint32_t c, jj;
        if (cfast) {
            jj = fdiv(it, d.div_C);
            c = it - jj * d.C;
        } else {
            c = it / M;
            jj = it % M;
        }
        const uint32_t g = lane0 + c;
        uint32_t bs = 0, j = 0;
        const bool live = g < total;
        if ((SIO == IO_GLOBAL || DIO == IO_GLOBAL) && live) {
            if (d.order == ORDER_J) {
                bs = fdiv(g, d.div_lanes_j);
                j = g - bs * d.lanes_j;
            } else {
                j = fdiv(g, d.div_batch);
                bs = g - j * d.batch;
            }
        }
        vec2_t v[P];
        if constexpr (SIO == IO_GLOBAL) {
            if (live) {
                fused_load<P>(d, bs, j, jj, M, v);
            } else {
#pragma unroll
                for (int q = 0; q < P; ++q) v[q] = {real_t(0), real_t(0)};
            }
        } else if constexpr (kLinLd) {
            const vec2_t* p0 = src + c * lstride + pad(jj);
#pragma unroll
            for (int q = 0; q < P; ++q) v[q] = p0[q * kLdStride];
        } else {
            const vec2_t* l0 = src + c * lstride;
#pragma unroll
            for (int q = 0; q < P; ++q) v[q] = l0[pad(jj + q * M)];
        }
        const uint32_t blk = jj / NS;
        const uint32_t kk = jj % NS;
        if constexpr (NS > 1) apply_inner_twiddles<P>(v, d.tw_inner, kk * TWS);
        dft<P, INV>(v);
        const uint32_t ob = blk * NS * P + kk;
        if constexpr (DIO == IO_SMEM) {
            if constexpr (kLinSt) {
                vec2_t* p0 = dst + c * lstride + pad(ob);
#pragma unroll
                for (int q = 0; q < P; ++q) p0[q * kStStride] = v[q];
            } else {
                vec2_t* l0 = dst + c * lstride;
#pragma unroll
                for (int q = 0; q < P; ++q) l0[pad(ob + q * NS)] = v[q];
            }
        } else if (live) {
            fused_store<P>(d, bs, j, ob, NS, v);
        }
    }
}

constexpr uint32_t ilog2(uint32_t v) { return v <= 1 ? 0 : 1 + ilog2(v >> 1); }

// R = 16^K16 * T (T in 1, 2, 4, 8): stages of radix 16, then T; the same
// ping-pong buffers as the generic body (A after stage 0, B after stage 1)
template <uint32_t R, bool INV>
__device__ __forceinline__ void tile_body_spec(const PassDesc& d, uint32_t lane0, uint32_t total,
                                               vec2_t* bufA, vec2_t* bufB) {
    constexpr uint32_t L = ilog2(R);
    static_assert((1u << L) == R && L >= 4 && L <= 12, "power-of-two tile from 16 to 4096");
    constexpr uint32_t K16 = L / 4;
    constexpr int T = 1 << (L % 4);
    constexpr int NP = int(K16) + (T > 1 ? 1 : 0);
    constexpr int PL = T > 1 ? T : 16;  // radix of the last stage
    if constexpr (NP == 1) {
        spec_stage<16, R, 1, IO_GLOBAL, IO_GLOBAL, INV>(d, nullptr, nullptr, lane0, total);
    } else if constexpr (NP == 2) {
        spec_stage<16, R, 1, IO_GLOBAL, IO_SMEM, INV>(d, nullptr, bufA, lane0, total);
        __syncthreads();
        spec_stage<PL, R, 16, IO_SMEM, IO_GLOBAL, INV>(d, bufA, nullptr, lane0, total);
    } else {
        static_assert(NP == 3, "at most three inner stages");
        spec_stage<16, R, 1, IO_GLOBAL, IO_SMEM, INV>(d, nullptr, bufA, lane0, total);
        __syncthreads();
        spec_stage<16, R, 16, IO_SMEM, IO_SMEM, INV>(d, bufA, bufB, lane0, total);
        __syncthreads();
        spec_stage<PL, R, 256, IO_SMEM, IO_GLOBAL, INV>(d, bufB, nullptr, lane0, total);
    }
}

// A CTA that runs many tiles of one power-of-two pass in turn, with the
// global loads of its next tile's first stage issued before the current
// tile's arithmetic, so the HBM latency of one tile hides behind the work of
// the previous one.  Needs a plain prologue (no chirp or gather): the loads
// are raw and the outer twiddle is applied when the tile's turn comes.
// Every tile's first stage has at most one radix-16 butterfly per thread
// (C * R <= 4096 points, 256 threads).
template <uint32_t R, bool INV>
__device__ __forceinline__ void tile_loop_pipelined(const PassDesc& d, vec2_t* sm) {
    constexpr uint32_t L = ilog2(R);
    constexpr uint32_t K16 = L / 4;
    constexpr int T = 1 << (L % 4);
    constexpr int NP = int(K16) + (T > 1 ? 1 : 0);
    constexpr int PL = T > 1 ? T : 16;
    constexpr uint32_t M0 = R / 16;
    const uint32_t total = d.batch * d.lanes_j;
    const uint32_t lstride = d.lane_stride;
    vec2_t* bufA = sm;
    vec2_t* bufB = sm + d.C * lstride + 1;
    const uint32_t it = threadIdx.x;
    const bool act = it < d.C * M0;
    uint32_t c0, jj0;
    if (d.load_mode == MODE_LANE) {
        jj0 = fdiv(it, d.div_C);
        c0 = it - jj0 * d.C;
    } else {
        c0 = it / M0;
        jj0 = it % M0;
    }
    auto locate = [&](uint32_t tile, uint32_t& bs, uint32_t& j) -> bool {
        const uint32_t g = tile * d.C + c0;
        if (!act || g >= total) return false;
        if (d.order == ORDER_J) {
            bs = fdiv(g, d.div_lanes_j);
            j = g - bs * d.lanes_j;
        } else {
            j = fdiv(g, d.div_batch);
            bs = g - j * d.batch;
        }
        return true;
    };
    vec2_t nxt[16];
    uint32_t bs_n = 0, j_n = 0;
    bool live_n = false;
    uint32_t tile = blockIdx.x;
    if (tile < d.tiles) {
        live_n = locate(tile, bs_n, j_n);
        if (live_n) prologue_load<16>(d, bs_n, j_n, jj0, M0, nxt);
    }
    for (; tile < d.tiles; tile += gridDim.x) {
        vec2_t v[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) v[q] = nxt[q];
        const uint32_t bs = bs_n, j = j_n;
        const bool live = live_n;
        const uint32_t nt = tile + gridDim.x;
        if (nt < d.tiles) {
            live_n = locate(nt, bs_n, j_n);
            if (live_n) prologue_load<16>(d, bs_n, j_n, jj0, M0, nxt);
        }
        const uint32_t lane0 = tile * d.C;
        // first stage (radix 16, NS = 1): outer twiddle, butterfly, store
        if (act) {
            if (live) {
                outer_twiddle<16>(d, j, jj0, M0, v);
            } else {
#pragma unroll
                for (int q = 0; q < 16; ++q) v[q] = {real_t(0), real_t(0)};
            }
            dft<16, INV>(v);
            const uint32_t ob = jj0 * 16;
            if constexpr (NP == 1) {
                if (live) fused_store<16>(d, bs, j, ob, 1, v);
            } else {
                if constexpr (kPadShift >= 4) {
                    vec2_t* p0 = bufA + c0 * lstride + pad(ob);  // 16 slots inside one pad period
#pragma unroll
                    for (int q = 0; q < 16; ++q) p0[q] = v[q];
                } else {
                    vec2_t* l0 = bufA + c0 * lstride;
#pragma unroll
                    for (int q = 0; q < 16; ++q) l0[pad(ob + q)] = v[q];
                }
            }
        }
        if constexpr (NP == 2) {
            __syncthreads();
            spec_stage<PL, R, 16, IO_SMEM, IO_GLOBAL, INV>(d, bufA, nullptr, lane0, total);
        } else if constexpr (NP == 3) {
            __syncthreads();
            spec_stage<16, R, 16, IO_SMEM, IO_SMEM, INV>(d, bufA, bufB, lane0, total);
            __syncthreads();
            spec_stage<PL, R, 256, IO_SMEM, IO_GLOBAL, INV>(d, bufB, nullptr, lane0, total);
        }
        __syncthreads();  // the next tile's first stage overwrites bufA
    }
}

#if defined(KFFT_HALF_SCALAR)
// ---------------------------------------------------------------------------
// single-pass power-of-two tiles fed by one-dimensional bulk copies: the C
// sequences of a tile are C*R contiguous points, so one untiled bulk copy
// (cp.async.bulk global -> shared, no tensor map; completion counted on an
// mbarrier) moves the next tile into shared memory while the current one's
// later stages run.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return uint32_t(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

// one bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global to shared memory, its completion counted on `bar`
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

// Bounded wait for phase `parity` of `bar`; false when `max_polls` polls ran
// out.  The first poll is a non-blocking test_wait (the copy has usually
// landed long before its tile's turn), the others are try_wait, which may
// suspend the thread for a hardware-defined time.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t max_polls) {
    for (uint32_t it = 0; it < max_polls; ++it) {
        uint32_t done;
        if (it == 0) {
            asm volatile(
                "{\n .reg .pred p;\n"
                " mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                " selp.u32 %0, 1, 0, p;\n}"
                : "=r"(done) : "r"(smem_addr(bar)), "r"(parity) : "memory");
        } else {
            asm volatile(
                "{\n .reg .pred p;\n"
                " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                " selp.u32 %0, 1, 0, p;\n}"
                : "=r"(done) : "r"(smem_addr(bar)), "r"(parity) : "memory");
        }
        if (done) return true;
    }
    return false;
}

// Shared memory: [mbarrier | pad to 128 B | raw tile C*R | bufA | bufB].
// A wait that runs out after `max_polls` polls (only a failed or very slow
// copy can cause it) sets *fail; the CTA then waits once more, with the
// default limit, for the copy in flight to land and ends without finishing
// its tiles, so the caller must treat the output as invalid.
template <uint32_t R, bool INV>
__device__ __forceinline__ void tile_loop_bulk(const PassDesc& d, unsigned char* smem,
                                               uint32_t* fail, uint32_t max_polls) {
    constexpr uint32_t L = ilog2(R);
    constexpr uint32_t K16 = L / 4;
    constexpr int T = 1 << (L % 4);
    constexpr int NP = int(K16) + (T > 1 ? 1 : 0);
    constexpr int PL = T > 1 ? T : 16;
    constexpr uint32_t M0 = R / 16;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    vec2_t* raw = reinterpret_cast<vec2_t*>(smem + 128);
    const uint32_t lstride = d.lane_stride;
    vec2_t* bufA = raw + d.C * R;
    vec2_t* bufB = bufA + d.C * lstride + 1;
    const uint32_t total = d.batch;  // one lane per sequence (lanes_j == 1)
    const uint32_t it = threadIdx.x;
    const bool act = it < d.C * M0;
    const uint32_t c0 = it / M0, jj0 = it % M0;
    auto issue = [&](uint32_t tile) {
        const uint32_t s0 = tile * d.C;
        const uint32_t n = min(d.C, total - s0);
        bulk_load(raw, d.in + uint64_t(s0) * d.in_bs, n * R * uint32_t(sizeof(vec2_t)), bar);
    };
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    uint32_t tile = blockIdx.x;
    if (threadIdx.x == 0 && tile < d.tiles) issue(tile);
    uint32_t parity = 0;
    for (; tile < d.tiles; tile += gridDim.x) {
        // every thread waits (the mbarrier's completion makes the copied data
        // visible to it); the CTA leaves together if any wait ran out, after
        // a second bounded wait that lets the copy in flight land first
        const bool ok = mbar_wait(bar, parity, max_polls);
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) atomicExch(fail, 1u);
            mbar_wait(bar, parity, kBulkMaxPolls);
            return;
        }
        parity ^= 1u;
        const uint32_t lane0 = tile * d.C;
        const uint32_t g = lane0 + c0;
        const bool live = act && g < total;
        vec2_t v[16];
        if (live) {
            const vec2_t* p0 = raw + c0 * R + jj0;
#pragma unroll
            for (int q = 0; q < 16; ++q) v[q] = p0[q * M0];
        }
        __syncthreads();  // every read of raw is done: the next copy may land there
        const uint32_t nt = tile + gridDim.x;
        if (threadIdx.x == 0 && nt < d.tiles) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(nt);
        }
        if (act) {
            if (!live) {
#pragma unroll
                for (int q = 0; q < 16; ++q) v[q] = {0.f, 0.f};
            }
            dft<16, INV>(v);
            const uint32_t ob = jj0 * 16;
            if constexpr (NP == 1) {
                if (live) fused_store<16>(d, g, 0, ob, 1, v);
            } else {
                vec2_t* p0 = bufA + c0 * lstride + pad(ob);  // 16 slots inside one pad period
#pragma unroll
                for (int q = 0; q < 16; ++q) p0[q] = v[q];
            }
        }
        if constexpr (NP == 2) {
            __syncthreads();
            spec_stage<PL, R, 16, IO_SMEM, IO_GLOBAL, INV>(d, bufA, nullptr, lane0, total);
        } else if constexpr (NP == 3) {
            __syncthreads();
            spec_stage<16, R, 16, IO_SMEM, IO_SMEM, INV>(d, bufA, bufB, lane0, total);
            __syncthreads();
            spec_stage<PL, R, 256, IO_SMEM, IO_GLOBAL, INV>(d, bufB, nullptr, lane0, total);
        }
        __syncthreads();  // the next tile's first stage overwrites bufA
    }
}
#endif

template <bool INV>
__device__ __forceinline__ void fused_dispatch(int P, const PassDesc& d, const InnerStep& st,
                                               const vec2_t* src, vec2_t* dst, uint32_t lane0,
                                               uint32_t total, int sio, int dio) {
    switch (P) {
        case 2: fused_pass<2, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 3: fused_pass<3, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 4: fused_pass<4, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 5: fused_pass<5, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 7: fused_pass<7, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 6: fused_pass<6, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 8: fused_pass<8, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 9: fused_pass<9, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 10: fused_pass<10, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 11: fused_pass<11, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 12: fused_pass<12, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 13: fused_pass<13, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 14: fused_pass<14, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 15: fused_pass<15, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        case 16: fused_pass<16, INV>(d, st, src, dst, lane0, total, sio, dio); break;
        default: break;
    }
}

// A tile whose first inner pass reads global memory and whose last writes it:
// two shared-memory round trips fewer than tile_body.  Shared memory holds two
// buffers of C*lane_stride+1 elements, lane c at c*lane_stride (only when the
// sub-FFT has 3+ inner passes; one buffer for 2 passes; none for 1).
// SPEC: dispatch power-of-two passes (d.spec) to their compile-time bodies;
// the pass kernel launches those as kernels of their own and leaves it off.
// TC: keep the tensor-core radix-16 stage; the queue kernel leaves it off
// (its planner clears d.tc) to keep its instruction footprint small.
template <bool INV, bool SPEC = true, bool TC = true>
__device__ __forceinline__ void tile_body_reg(const PassDesc& d, const PassExtra& x, uint32_t tile,
                                              vec2_t* sm) {
    const uint32_t total = d.batch * d.lanes_j;
    const uint32_t lane0 = tile * d.C;
    const int np = d.nrad;
    if (np == 0) {  // length-1 sub-FFT: the pass is a scaled copy (with its fused ops)
        for (uint32_t c = threadIdx.x; c < d.C; c += blockDim.x) {
            const uint32_t g = lane0 + c;
            if (g >= total) continue;
            uint32_t bs, j;
            if (d.order == ORDER_J) {
                bs = fdiv(g, d.div_lanes_j);
                j = g - bs * d.lanes_j;
            } else {
                j = fdiv(g, d.div_batch);
                bs = g - j * d.batch;
            }
            store_elem(d, bs, j, load_elem(d, bs, j));
        }
        return;
    }
    vec2_t* bufA = sm;
    vec2_t* bufB = sm + d.C * d.lane_stride + 1;
#if defined(KFFT_HALF_SCALAR)
    if constexpr (SPEC) switch (d.spec) {
        case 4: tile_body_spec<16, INV>(d, lane0, total, bufA, bufB); return;
        case 5: tile_body_spec<32, INV>(d, lane0, total, bufA, bufB); return;
        case 6: tile_body_spec<64, INV>(d, lane0, total, bufA, bufB); return;
        case 7: tile_body_spec<128, INV>(d, lane0, total, bufA, bufB); return;
        case 8: tile_body_spec<256, INV>(d, lane0, total, bufA, bufB); return;
        case 9: tile_body_spec<512, INV>(d, lane0, total, bufA, bufB); return;
        case 10: tile_body_spec<1024, INV>(d, lane0, total, bufA, bufB); return;
        case 11: tile_body_spec<2048, INV>(d, lane0, total, bufA, bufB); return;
        case 12: tile_body_spec<4096, INV>(d, lane0, total, bufA, bufB); return;
        default: break;
    }
#endif
    const vec2_t* src = nullptr;
#if defined(KFFT_HALF_SCALAR)
    TcFrag Fr, Fi, Gm;
    if (TC && d.tc) {
        Fr = dft16_frag<INV>(0);
        Fi = dft16_frag<INV>(1);
        Gm = dft16_frag<INV>(2);
    }
#endif
    for (int p = 0; p < np; ++p) {
        const bool last = (p + 1 == np);
        vec2_t* dst = last ? nullptr : ((p % 2 == 0) ? bufA : bufB);
        const int sio = p == 0 ? IO_GLOBAL : IO_SMEM, dio = last ? IO_GLOBAL : IO_SMEM;
#if defined(KFFT_HALF_SCALAR)
        if (TC && d.tc && d.rad[p] == 16)
            tc_pass16<INV>(d, x.step[p], src, dst, lane0, total, sio, dio, Fr, Fi, Gm);
        else
#endif
            fused_dispatch<INV>(d.rad[p], d, x.step[p], src, dst, lane0, total, sio, dio);
        if (!last) __syncthreads();
        src = dst;
    }
}

// ---- persistent-queue helpers --------------------------------------------
// One queue item: tile `tile` of pass `desc`, which may start once
// done[dep] reaches `need` (the tiles of the pass it reads; dep < 0: none).
struct QueueItem {
    uint32_t desc;
    uint32_t tile;
    int32_t dep;
    uint32_t need;
};

__device__ __forceinline__ uint32_t load_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Waits for all tiles of pass `dep` to finish; a bounded spin that reports
// failure instead of hanging.
__device__ __forceinline__ bool wait_for(const uint32_t* done, uint32_t need, uint32_t max_polls) {
    for (uint32_t it = 0; it < max_polls; ++it) {
        if (load_acquire(done) >= need) return true;
        __nanosleep(200);
    }
    return false;
}

PassExtra make_extra(const PassDesc& d);

}  // namespace kfft
