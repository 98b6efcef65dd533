// kernels.cu -- sm_103a kernels of the GB300 FFT engine.
//
// k_pass: one Stockham pass of radix R over a tile of C lanes (see engine.cuh).
//   load   : global -> shared, fused prologue (chirp / gather) and the outer
//            twiddle W_{Ns*R}^{r*k} from a two-level FP64-generated table;
//   inner  : the length-R sub-FFT as shared-memory Stockham passes of radix
//            2, 4, 8, 16 and odd primes 3..31 (register butterflies);
//   store  : shared -> global, fused epilogue (scale, spectrum product, chirp,
//            Rader scatter).
// It replaces the reference's recursive kf_work (kfft_work.c:1-59) and its
// butterflies kf_bfly2/3/4/5 and std_method_eval (kfft_bfly.c:1-152,
// kfft_generic.c:9-36); the Rader and Bluestein wiring of the prologue and
// epilogue replaces rader_method_eval/kfft_part_convolution (kfft_rader.c).
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>

#include "engine.cuh"

namespace kfft {

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
void FastDiv::init(uint32_t div) {
    d = div ? div : 1;
    uint32_t l = 0;
    while (l < 32 && (uint64_t(1) << l) < d) ++l;
    s = l;
    // m = floor(2^32 * (2^l - d) / d) + 1  (fits in 32 bits for d >= 1)
    m = uint32_t(((uint64_t(1) << 32) * ((uint64_t(1) << l) - d)) / d + 1);
}

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
    return uint32_t((uint64_t(__umulhi(n, f.m)) + n) >> f.s);
}

__device__ __forceinline__ vec2_t cadd(vec2_t a, vec2_t b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ vec2_t csub(vec2_t a, vec2_t b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ vec2_t cmul(vec2_t a, vec2_t b) {
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
__device__ __forceinline__ vec2_t cscale(vec2_t a, real_t s) { return {a.x * s, a.y * s}; }
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

template <int P>
struct OddTrig {
    static constexpr int H = (P - 1) / 2;
    real_t c[H * H];
    real_t s[H * H];
    constexpr OddTrig() : c(), s() {
        for (int k = 1; k <= H; ++k)
            for (int n = 1; n <= H; ++n) {
                c[(k - 1) * H + (n - 1)] = real_t(trig_ratio(long(n) * k, P, false));
                s[(k - 1) * H + (n - 1)] = real_t(trig_ratio(long(n) * k, P, true));
            }
    }
};

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

// odd prime P: symmetric-pair DFT, (P-1)^2 real multiply-adds
template <int P, bool INV>
__device__ __forceinline__ void dft_odd(vec2_t* v) {
    constexpr int H = (P - 1) / 2;
    constexpr OddTrig<P> T{};
    vec2_t s[H], d[H];
    vec2_t x0 = v[0], sum = v[0];
#pragma unroll
    for (int n = 1; n <= H; ++n) {
        s[n - 1] = cadd(v[n], v[P - n]);
        d[n - 1] = csub(v[n], v[P - n]);
        sum = cadd(sum, s[n - 1]);
    }
#pragma unroll
    for (int k = 1; k <= H; ++k) {
        vec2_t a = x0, b = {real_t(0), real_t(0)};
#pragma unroll
        for (int n = 1; n <= H; ++n) {
            const real_t cc = T.c[(k - 1) * H + (n - 1)];
            const real_t ss = T.s[(k - 1) * H + (n - 1)];
            a.x += s[n - 1].x * cc;
            a.y += s[n - 1].y * cc;
            b.x += d[n - 1].x * ss;
            b.y += d[n - 1].y * ss;
        }
        // forward: X_k = a - i b, X_{P-k} = a + i b; inverse swaps
        vec2_t ib = {-b.y, b.x};
        if (INV) {
            v[k] = cadd(a, ib);
            v[P - k] = csub(a, ib);
        } else {
            v[k] = csub(a, ib);
            v[P - k] = cadd(a, ib);
        }
    }
    v[0] = sum;
}

template <int P, bool INV>
__device__ __forceinline__ void dft(vec2_t* v) {
    if constexpr (P == 2) dft2<INV>(v[0], v[1]);
    else if constexpr (P == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
    else if constexpr (P == 8) dft8<INV>(v);
    else if constexpr (P == 16) dft16<INV>(v);
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
        case 8: inner_pass<8, INV>(src, dst, R, C, st, tw); break;
        case 11: inner_pass<11, INV>(src, dst, R, C, st, tw); break;
        case 13: inner_pass<13, INV>(src, dst, R, C, st, tw); break;
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
            const uint32_t mask = (1u << d.tw_shift) - 1u;
#pragma unroll
            for (int u = 0; u < kLoadUnroll; ++u) {
                const vec2_t w = cmul(__ldg(&d.tw_hi[twe[u] >> d.tw_shift]), __ldg(&d.tw_lo[twe[u] & mask]));
                v[u] = cmul(v[u], w);
            }
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

template <bool INV, bool BIG>
__global__ void __launch_bounds__(kPassThreads) k_pass(const __grid_constant__ PassDesc d,
                                                       const __grid_constant__ PassExtra x) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    tile_body<INV, BIG>(d, x, blockIdx.x, reinterpret_cast<vec2_t*>(smem_raw));
}

// ---------------------------------------------------------------------------
// persistent work-queue kernel: items (pass, tile) ordered by dependency level
// ---------------------------------------------------------------------------
struct QueueItem {
    uint32_t desc;
    uint32_t tile;
};

__device__ __forceinline__ uint32_t load_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Waits for all tiles of pass `dep` to finish; a bounded spin that reports
// failure instead of hanging.
__device__ __forceinline__ bool wait_for(const uint32_t* done, uint32_t need) {
    for (uint32_t it = 0; it < (1u << 24); ++it) {
        if (load_acquire(done) >= need) return true;
        __nanosleep(200);
    }
    return false;
}

__global__ void __launch_bounds__(kPassThreads) k_persistent(
    const PassDesc* __restrict__ descs, const PassExtra* __restrict__ extras,
    const int32_t* __restrict__ deps, const QueueItem* __restrict__ items, uint32_t nitems,
    uint32_t* head, uint32_t* done, uint32_t* error) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t s_item;
    __shared__ uint32_t s_ok;
    __shared__ __align__(16) PassDesc s_desc;
    __shared__ __align__(16) PassExtra s_extra;
    vec2_t* buf = reinterpret_cast<vec2_t*>(smem_raw);
    while (true) {
        if (threadIdx.x == 0) s_item = atomicAdd(head, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if (it >= nitems) return;
        const QueueItem q = items[it];
        if (threadIdx.x == 0) {
            bool ok = true;
            const int32_t dep = deps[q.desc];
            if (dep >= 0) ok = wait_for(&done[dep], descs[dep].tiles);
            if (!ok) atomicExch(error, 1u);
            s_ok = ok ? 1u : 0u;
        }
        // stage the descriptor in shared memory
        {
            const uint32_t* src = reinterpret_cast<const uint32_t*>(&descs[q.desc]);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&s_desc);
            for (uint32_t i = threadIdx.x; i < sizeof(PassDesc) / 4; i += blockDim.x) dst[i] = src[i];
            const uint32_t* xs = reinterpret_cast<const uint32_t*>(&extras[q.desc]);
            uint32_t* xd = reinterpret_cast<uint32_t*>(&s_extra);
            for (uint32_t i = threadIdx.x; i < sizeof(PassExtra) / 4; i += blockDim.x) xd[i] = xs[i];
        }
        __syncthreads();
        if (s_ok) {
            if (s_desc.inv) tile_body<true, false>(s_desc, s_extra, q.tile, buf);
            else tile_body<false, false>(s_desc, s_extra, q.tile, buf);
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) atomicAdd(&done[q.desc], 1u);
    }
}

static bool configure_pass_kernels() {
    static bool done = false;
    if (done) return true;
    const void* fns[4] = {(const void*)k_pass<false, false>, (const void*)k_pass<true, false>,
                          (const void*)k_pass<false, true>, (const void*)k_pass<true, true>};
    for (const void* f : fns) {
        cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             227 * 1024);
        if (e != cudaSuccess) {
            note_cuda_error(e);
            return false;
        }
    }
    done = true;
    return true;
}

void launch_pass(const PassDesc& d, cudaStream_t st) {
    if (!configure_pass_kernels()) return;
    const PassExtra x = make_extra(d);
    bool big = false;
    for (int p = 0; p < d.nrad; ++p) big = big || d.rad[p] > 16;
    if (d.inv) {
        if (big) k_pass<true, true><<<d.tiles, d.threads, d.smem_bytes, st>>>(d, x);
        else k_pass<true, false><<<d.tiles, d.threads, d.smem_bytes, st>>>(d, x);
    } else {
        if (big) k_pass<false, true><<<d.tiles, d.threads, d.smem_bytes, st>>>(d, x);
        else k_pass<false, false><<<d.tiles, d.threads, d.smem_bytes, st>>>(d, x);
    }
    note_cuda_error(cudaGetLastError());
    count_launch();
}

PassExtra make_extra(const PassDesc& d) {
    PassExtra x;
    memset(&x, 0, sizeof(x));
    uint32_t ns = 1;
    for (int p = 0; p < d.nrad; ++p) {
        const uint32_t P = d.rad[p];
        InnerStep& s = x.step[p];
        s.m = d.R / P;
        s.ns = ns;
        s.twstride = d.R / (ns * P);
        s.div_m.init(s.m);
        s.div_ns.init(ns);
        ns *= P;
    }
    return x;
}

size_t pass_extra_bytes() { return sizeof(PassExtra); }

void fill_extras(const PassDesc* d, void* extras, size_t n) {
    PassExtra* x = static_cast<PassExtra*>(extras);
    for (size_t i = 0; i < n; ++i) x[i] = make_extra(d[i]);
}

bool launch_persistent(const PassDesc* descs, const void* extras, const int32_t* deps,
                       const void* items, uint32_t nitems, uint32_t* head, uint32_t* done,
                       uint32_t* error, uint32_t smem_bytes, cudaStream_t st) {
    static int blocks_per_sm = -1;
    static uint32_t configured_smem = 0;
    static int sms = 0;
    if (configured_smem < smem_bytes) {
        cudaError_t e = cudaFuncSetAttribute(k_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             int(smem_bytes));
        if (e != cudaSuccess) {
            note_cuda_error(e);
            return false;
        }
        configured_smem = smem_bytes;
        blocks_per_sm = -1;
    }
    if (blocks_per_sm < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_persistent, kPassThreads,
                                                      smem_bytes);
        if (blocks_per_sm < 1) blocks_per_sm = 1;
    }
    uint32_t grid = uint32_t(sms * blocks_per_sm);
    if (grid > nitems) grid = nitems ? nitems : 1;
    k_persistent<<<grid, kPassThreads, smem_bytes, st>>>(
        descs, static_cast<const PassExtra*>(extras), deps, static_cast<const QueueItem*>(items),
        nitems, head, done, error);
    note_cuda_error(cudaGetLastError());
    count_launch();
    return true;
}

// ---------------------------------------------------------------------------
// FP64 table generation
// ---------------------------------------------------------------------------
__global__ void k_gen_twiddles(vec2_t* t, uint32_t count, uint64_t mult, uint32_t n, int sign) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += gridDim.x * blockDim.x) {
        uint64_t e = (uint64_t(i) * mult) % n;
        int64_t es = (2 * e > n) ? int64_t(e) - int64_t(n) : int64_t(e);
        double s, c;
        sincospi(2.0 * double(es) / double(n), &s, &c);
        t[i] = {real_t(c), real_t(sign * s)};
    }
}

void gen_twiddles(vec2_t* t, uint32_t count, uint64_t mult, uint32_t n, int sign,
                  cudaStream_t st) {
    if (!count) return;
    uint32_t blocks = (count + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_gen_twiddles<<<blocks, 256, 0, st>>>(t, count, mult, n, sign);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_gen_chirp(vec2_t* c, uint32_t count, uint32_t n, int sign) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count;
         k += gridDim.x * blockDim.x) {
        const uint64_t two_n = 2 * uint64_t(n);
        uint64_t kk = k % two_n;
        uint64_t e = (kk * kk) % two_n;  // k^2 mod 2n, exact in integers
        int64_t es = (e > n) ? int64_t(e) - int64_t(two_n) : int64_t(e);
        double s, co;
        sincospi(double(es) / double(n), &s, &co);
        c[k] = {real_t(co), real_t(sign * s)};
    }
}

void gen_chirp(vec2_t* c, uint32_t count, uint32_t n, int sign, cudaStream_t st) {
    uint32_t blocks = (count + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_gen_chirp<<<blocks, 256, 0, st>>>(c, count, n, sign);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_bluestein_filter(vec2_t* b, const vec2_t* chirp, uint32_t n, uint32_t m_len) {
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < m_len;
         m += gridDim.x * blockDim.x) {
        vec2_t v = {real_t(0), real_t(0)};
        if (m < n) v = chirp[m];
        else if (m > m_len - n) v = chirp[m_len - m];
        b[m] = {v.x, -v.y};
    }
}

void gen_bluestein_filter(vec2_t* b, const vec2_t* chirp, uint32_t n, uint32_t m_len,
                          cudaStream_t st) {
    uint32_t blocks = (m_len + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_bluestein_filter<<<blocks, 256, 0, st>>>(b, chirp, n, m_len);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_gen_rader(vec2_t* s, const uint32_t* pidx, uint32_t p, int sign) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j + 1 < p;
         j += gridDim.x * blockDim.x) {
        uint32_t e = pidx[j];
        int64_t es = (2 * uint64_t(e) > p) ? int64_t(e) - int64_t(p) : int64_t(e);
        double sn, c;
        sincospi(2.0 * double(es) / double(p), &sn, &c);
        s[j] = {real_t(c), real_t(sign * sn)};
    }
}

void gen_rader_kernel(vec2_t* s, const uint32_t* pidx, uint32_t p, int sign, cudaStream_t st) {
    uint32_t blocks = (p + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_gen_rader<<<blocks, 256, 0, st>>>(s, pidx, p, sign);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_super_twiddles(vec2_t* t, uint32_t h, int sign) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < h; k += gridDim.x * blockDim.x) {
        // phase = sign * pi * ((k+1)/h + 1/2) = sign * pi * (2(k+1) + h) / (2h)
        uint64_t num = (2 * uint64_t(k + 1) + h) % (4 * uint64_t(h));
        int64_t ns = (num > 2 * uint64_t(h)) ? int64_t(num) - int64_t(4 * uint64_t(h)) : int64_t(num);
        double s, c;
        sincospi(double(ns) / (2.0 * double(h)), &s, &c);
        t[k] = {real_t(c), real_t(sign * s)};
    }
}

void gen_super_twiddles(vec2_t* t, uint32_t h, int sign, cudaStream_t st) {
    if (!h) return;
    uint32_t blocks = (h + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_super_twiddles<<<blocks, 256, 0, st>>>(t, h, sign);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_scale_table(vec2_t* t, uint32_t count, double s) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += gridDim.x * blockDim.x)
        t[i] = {real_t(t[i].x * s), real_t(t[i].y * s)};
}

void scale_table(vec2_t* t, uint32_t count, double s, cudaStream_t st) {
    uint32_t blocks = (count + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_scale_table<<<blocks, 256, 0, st>>>(t, count, s);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

// ---------------------------------------------------------------------------
// real transform post/pre processing (kfft_scalar.c:174-242)
// ---------------------------------------------------------------------------
__global__ void k_real_post(const vec2_t* __restrict__ z, vec2_t* __restrict__ out,
                            const vec2_t* __restrict__ stt, uint32_t h, uint32_t batch,
                            uint64_t out_bs, int expand) {
    const uint32_t half = h / 2;  // k = 1..half
    const uint64_t per = uint64_t(half) + 1;
    const uint64_t total = per * batch;
    for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < total;
         t += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t b = uint32_t(t / per);
        const uint32_t k = uint32_t(t - uint64_t(b) * per);
        const vec2_t* Z = z + uint64_t(b) * h;
        vec2_t* O = out + uint64_t(b) * out_bs;
        const uint32_t n = 2 * h;
        if (k == 0) {
            vec2_t z0 = Z[0];
            O[0] = {z0.x + z0.y, real_t(0)};
            O[h] = {z0.x - z0.y, real_t(0)};
            if (expand && h > 0) { /* mirror of bin h is itself */ }
            continue;
        }
        vec2_t fpk = Z[k];
        vec2_t zn = Z[h - k];
        vec2_t fpnk = {zn.x, -zn.y};
        vec2_t f1k = cadd(fpk, fpnk), f2k = csub(fpk, fpnk);
        vec2_t tw = cmul(f2k, stt[k - 1]);
        vec2_t a = {real_t(0.5) * (f1k.x + tw.x), real_t(0.5) * (f1k.y + tw.y)};
        vec2_t bb = {real_t(0.5) * (f1k.x - tw.x), real_t(0.5) * (tw.y - f1k.y)};
        if (2 * k == h) {
            O[k] = bb;  // both writes land on the same bin; the later one wins
            if (expand) O[n - k] = {bb.x, -bb.y};
        } else {
            O[k] = a;
            O[h - k] = bb;
            if (expand) {
                O[n - k] = {a.x, -a.y};
                O[n - (h - k)] = {bb.x, -bb.y};
            }
        }
    }
}

void launch_real_post(const vec2_t* z, vec2_t* out, const vec2_t* st_tab, uint32_t h,
                      uint32_t batch, uint64_t out_bs, int expand, cudaStream_t st) {
    uint64_t total = (uint64_t(h / 2) + 1) * batch;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    k_real_post<<<uint32_t(blocks), 256, 0, st>>>(z, out, st_tab, h, batch, out_bs, expand);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_real_pre(const vec2_t* __restrict__ in, vec2_t* __restrict__ z,
                           const vec2_t* __restrict__ stt, uint32_t h, uint32_t batch,
                           uint64_t in_bs) {
    const uint32_t half = h / 2;
    const uint64_t per = uint64_t(half) + 1;
    const uint64_t total = per * batch;
    for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < total;
         t += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t b = uint32_t(t / per);
        const uint32_t k = uint32_t(t - uint64_t(b) * per);
        const vec2_t* I = in + uint64_t(b) * in_bs;
        vec2_t* Z = z + uint64_t(b) * h;
        if (k == 0) {
            Z[0] = {I[0].x + I[h].x, I[0].x - I[h].x};
            continue;
        }
        vec2_t fk = I[k];
        vec2_t fn = I[h - k];
        vec2_t fnkc = {fn.x, -fn.y};
        vec2_t fek = cadd(fk, fnkc), tmp = csub(fk, fnkc);
        vec2_t fok = cmul(tmp, stt[k - 1]);
        vec2_t lo = cadd(fek, fok);
        vec2_t hi = csub(fek, fok);
        hi.y = -hi.y;
        if (2 * k == h) {
            Z[k] = hi;
        } else {
            Z[k] = lo;
            Z[h - k] = hi;
        }
    }
}

void launch_real_pre(const vec2_t* in, vec2_t* z, const vec2_t* st_tab, uint32_t h,
                     uint32_t batch, uint64_t in_bs, cudaStream_t st) {
    uint64_t total = (uint64_t(h / 2) + 1) * batch;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    k_real_pre<<<uint32_t(blocks), 256, 0, st>>>(in, z, st_tab, h, batch, in_bs);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_widen(const real_t* __restrict__ in, vec2_t* __restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
         i += uint64_t(gridDim.x) * blockDim.x)
        out[i] = {in[i], real_t(0)};
}
void launch_widen(const real_t* in, vec2_t* out, uint64_t n, cudaStream_t st) {
    uint64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (!blocks) return;
    k_widen<<<uint32_t(blocks), 256, 0, st>>>(in, out, n);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_narrow(const vec2_t* __restrict__ in, real_t* __restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
         i += uint64_t(gridDim.x) * blockDim.x)
        out[i] = in[i].x;
}
void launch_narrow(const vec2_t* in, real_t* out, uint64_t n, cudaStream_t st) {
    uint64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (!blocks) return;
    k_narrow<<<uint32_t(blocks), 256, 0, st>>>(in, out, n);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

// 32x32 tiled transpose: out[b][c][r] = in[b][r][c]
template <typename E>
__global__ void k_transpose(const E* __restrict__ in, E* __restrict__ out, uint32_t rows,
                            uint32_t cols) {
    __shared__ E tile[32][33];
    const uint64_t boff = uint64_t(blockIdx.z) * rows * cols;
    const uint32_t c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (uint32_t i = threadIdx.y; i < 32; i += blockDim.y) {
        uint32_t r = r0 + i, c = c0 + threadIdx.x;
        if (r < rows && c < cols) tile[i][threadIdx.x] = in[boff + uint64_t(r) * cols + c];
    }
    __syncthreads();
    for (uint32_t i = threadIdx.y; i < 32; i += blockDim.y) {
        uint32_t c = c0 + i, r = r0 + threadIdx.x;
        if (r < rows && c < cols) out[boff + uint64_t(c) * rows + r] = tile[threadIdx.x][i];
    }
}

void launch_transpose(const vec2_t* in, vec2_t* out, uint32_t rows, uint32_t cols,
                      uint32_t batch, cudaStream_t st) {
    dim3 grid((cols + 31) / 32, (rows + 31) / 32, batch);
    k_transpose<vec2_t><<<grid, dim3(32, 8), 0, st>>>(in, out, rows, cols);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

void launch_transpose_real(const real_t* in, real_t* out, uint32_t rows, uint32_t cols,
                           cudaStream_t st) {
    dim3 grid((cols + 31) / 32, (rows + 31) / 32, 1);
    k_transpose<real_t><<<grid, dim3(32, 8), 0, st>>>(in, out, rows, cols);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_hadamard(vec2_t* __restrict__ b, const vec2_t* __restrict__ a, uint64_t n) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
         i += uint64_t(gridDim.x) * blockDim.x)
        b[i] = cmul(b[i], a[i]);
}

void launch_hadamard(vec2_t* b, const vec2_t* a, uint64_t n, cudaStream_t st) {
    uint64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (!blocks) return;
    k_hadamard<<<uint32_t(blocks), 256, 0, st>>>(b, a, n);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

__global__ void k_copy_rows(const vec2_t* __restrict__ in, vec2_t* __restrict__ out, uint32_t len,
                            uint64_t ss, uint64_t ds, uint32_t rows) {
    const uint64_t total = uint64_t(len) * rows;
    for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < total;
         t += uint64_t(gridDim.x) * blockDim.x) {
        uint64_t r = t / len, c = t - r * len;
        out[r * ds + c] = in[r * ss + c];
    }
}

void launch_copy_rows(const vec2_t* in, vec2_t* out, uint32_t len, uint64_t src_stride,
                      uint64_t dst_stride, uint32_t rows, cudaStream_t st) {
    uint64_t total = uint64_t(len) * rows;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    if (!blocks) return;
    k_copy_rows<<<uint32_t(blocks), 256, 0, st>>>(in, out, len, src_stride, dst_stride, rows);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

}  // namespace kfft
