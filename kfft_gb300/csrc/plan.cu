// plan.cu -- device planner and pass executor of the GB300 FFT engine.
//
// Replaces the reference planner (kf_factor / kfft_kinit / kfft_calculate,
// kfft_cpx.c:103-318): instead of a recursive radix schedule with an N-entry
// host twiddle table, a length N becomes
//   DIRECT     N = R_0 * R_1 * ... (every prime factor <= 31): one Stockham
//              pass per R_i, each R_i <= the shared-memory tile, FP64-generated
//              device tables (W_R per pass, two-level W_N for the outer twiddles);
//   RADER      N prime, N-1 DIRECT: (N-1)-point cyclic convolution with the
//              generator gather fused into the first forward pass and the
//              scatter into the last inverse pass (kfft_rader.c:17-63);
//   BLUESTEIN  any other N: chirp-z convolution of length M >= 2N-1, M 7-smooth,
//              with the chirps and the filter product fused into the passes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <sstream>

#include "engine.cuh"
#include "plan_host.h"

namespace kfft {

// ---------------------------------------------------------------------------
// sizing rules
// ---------------------------------------------------------------------------
constexpr size_t kSmemBudget = 200 * 1024;  // bytes of dynamic shared memory per CTA
#if defined(KFFT_HALF_SCALAR)
constexpr uint32_t kPadShiftHost = 4;
constexpr uint32_t kMultiLanes = 8;   // 64-byte row segments
#else
constexpr uint32_t kPadShiftHost = 3;
constexpr uint32_t kMultiLanes = 4;   // 64-byte row segments
#endif

// Multi-lane tiles of passes of 256 points or more hold half a full tile in
// the FP64 build (measured faster there); FP32 tiles are full (with lanes
// skewed in shared memory, a full tile of a 256-point pass measured 18-23%
// faster than half of one).
static uint32_t lane_share(uint32_t R) {
#if defined(KFFT_HALF_SCALAR)
    (void)R;
    return 1;
#else
    return R >= 256 ? 2u : 1u;
#endif
}

static uint32_t pad_host(uint32_t i) { return i + (i >> kPadShiftHost); }

static uint32_t tile_capacity() {
    // two ping-pong buffers of pad(C*R)+1 elements
    double per = 2.0 * sizeof(vec2_t) * (1.0 + 1.0 / double(1u << kPadShiftHost));
    return uint32_t(double(kSmemBudget - 64) / per);
}

bool columns_coalesce(const FftPlan& P) {
    if (P.method != METHOD_DIRECT) return false;
    // a column pass's tile takes min(16, capacity / R) columns: four or more
    // keep its row segments at 32 bytes or longer
    for (const PassSpec& s : P.passes)
        if (uint64_t(s.R) * 4 > tile_capacity()) return false;
    return true;
}

static uint32_t smem_for(uint32_t elems) {
    return 2u * (pad_host(elems) + 1u) * uint32_t(sizeof(vec2_t));
}

// ---------------------------------------------------------------------------
// shared-memory lane stride of the register-tile bodies (lane_stride_search
// in plan_host.h), cached per (R, C, lane modes, threads)
// ---------------------------------------------------------------------------
uint32_t spec_lane_stride(uint32_t R, uint32_t C, bool load_lane, bool store_lane,
                          uint32_t threads) {
    static std::mutex mu;
    static std::map<std::pair<uint64_t, uint32_t>, uint32_t> cache;
    const auto key = std::make_pair((uint64_t(R) << 32) | C,
                                    uint32_t(load_lane) | (uint32_t(store_lane) << 1) | (threads << 2));
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    const uint32_t best = lane_stride_search(R, C, load_lane, store_lane, threads);
    cache[key] = best;
    return best;
}

// ---------------------------------------------------------------------------
// arithmetic helpers
// ---------------------------------------------------------------------------
bool is_direct_length(uint32_t n, uint32_t max_prime) {
    if (n == 0) return false;
    for (uint32_t p : prime_factors(n))
        if (p > max_prime) return false;
    return true;
}

static bool is_prime(uint32_t n) {
    if (n < 2) return false;
    for (uint32_t p = 2; uint64_t(p) * p <= n; ++p)
        if (n % p == 0) return false;
    return true;
}

static uint32_t modpow(uint64_t x, uint64_t y, uint64_t m) {
    uint64_t r = 1 % m;
    x %= m;
    while (y) {
        if (y & 1) r = r * x % m;
        x = x * x % m;
        y >>= 1;
    }
    return uint32_t(r);
}

// smallest primitive root of prime p (same choice as kfft_math.c:5-33)
static uint32_t primitive_root(uint32_t p) {
    std::vector<uint32_t> f = prime_factors(p - 1);
    f.erase(std::unique(f.begin(), f.end()), f.end());
    for (uint32_t g = 2; g < p; ++g) {
        bool ok = true;
        for (uint32_t q : f)
            if (modpow(g, (p - 1) / q, p) == 1) {
                ok = false;
                break;
            }
        if (ok) return g;
    }
    return p == 2 ? 1 : 0;
}

// lanes of a multi-pass register-resident tile
constexpr uint32_t kRegLanes = 4;

// true when a tile of C lanes of length R fits the fused-I/O kernel: every
// inner radix <= 16 and at most kRegTile points per tile
static bool reg_tile_fits(uint32_t R, uint32_t C, uint32_t cap = kRegTile) {
    if (C < 1 || uint64_t(C) * R > std::min(cap, kRegTile)) return false;
    if (R == 1) return true;  // a length-1 pass is a copy
    std::vector<uint8_t> rad = inner_radices(R);
    if (rad.empty() || rad.size() > size_t(kMaxInnerRadices)) return false;
    for (uint8_t r : rad)
        if (r > 16) return false;
    return true;
}

// ---------------------------------------------------------------------------
// device arena
// ---------------------------------------------------------------------------
void* DeviceArena::alloc(size_t n) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, n ? n : 16);
    if (e != cudaSuccess) {
        note_cuda_error(e);
        return nullptr;
    }
    blocks.push_back(p);
    bytes += n;
    account_device_bytes(int64_t(n));
    return p;
}

DeviceArena::~DeviceArena() {
    for (void* p : blocks) cudaFree(p);
    account_device_bytes(-int64_t(bytes));
}

vec2_t* Workspace::take(size_t elems) {
    size_t bytes = (elems * sizeof(vec2_t) + 255) & ~size_t(255);
    if (used + bytes > size) return nullptr;
    vec2_t* p = reinterpret_cast<vec2_t*>(base + used);
    used += bytes;
    return p;
}

FftPlan::~FftPlan() {
    delete sub_fwd;
    delete sub_inv;
}

// ---------------------------------------------------------------------------
// plan construction
// ---------------------------------------------------------------------------
static bool build_direct(FftPlan* P, DeviceArena& arena, cudaStream_t st) {
    const uint32_t N = P->N;
    std::vector<uint32_t> Rs;
    // lengths whose radices are all <= 16 run in register-resident tiles (one
    // pass when the whole sequence fits, else the largest balanced split whose
    // tiles of kRegLanes lanes fit); others use the shared-memory ping-pong tile
    bool small_radices = true;
    for (uint32_t f : prime_factors(N)) small_radices = small_radices && f <= 13;
    const PlanVariant& V = P->var;
    if (V.no_fused) small_radices = false;
    if (small_radices && N <= V.single_cap && reg_tile_fits(N, 1, V.tile_cap)) {
        Rs.push_back(N);
    } else if (small_radices) {
#if defined(KFFT_HALF_SCALAR)
        const bool pow2 = (N & (N - 1)) == 0;
#else
        const bool pow2 = false;
#endif
        if (pow2) Rs = pow2_split(N, V.rmax);
        for (uint32_t rmax : {1024u, 768u, 512u, 384u, 256u, 128u, 64u, 32u, 16u}) {
            if (!Rs.empty()) break;
            if (rmax > V.rmax) continue;
            std::vector<uint32_t> cand = split_passes(N, rmax);
            bool ok = !cand.empty();
            for (uint32_t R : cand) ok = ok && reg_tile_fits(R, std::min(kRegLanes, N / R), V.tile_cap);
            if (ok) Rs = cand;
        }
    }
    if (Rs.empty()) {
        if (N <= tile_capacity() && N <= std::max(V.single_cap, kRegTile)) Rs.push_back(N);
        else Rs = split_passes(N, std::min(kMultiRmax, V.rmax));
    }
    if (Rs.empty()) return false;
    if (V.reverse) std::reverse(Rs.begin(), Rs.end());
    std::map<uint32_t, const vec2_t*> inner;
    uint32_t Ns = 1;
    for (uint32_t R : Rs) {
        PassSpec s;
        s.R = R;
        s.Ns = Ns;
        s.radices = inner_radices(R);
        if (s.radices.size() > size_t(kMaxInnerRadices)) return false;
        auto it = inner.find(R);
        if (it == inner.end()) {
            vec2_t* t = static_cast<vec2_t*>(arena.alloc(sizeof(vec2_t) * R));
            if (!t) return false;
            gen_twiddles(t, R, 1, R, P->sign, st);
            it = inner.emplace(R, t).first;
        }
        s.tw_inner = it->second;
        P->passes.push_back(s);
        Ns *= R;
    }
    if (P->passes.size() > 1) {
        uint32_t bits = 0;
        while ((uint64_t(1) << bits) < N) ++bits;
        uint32_t shift = (bits + 1) / 2;
        uint32_t nlo = 1u << shift;
        uint32_t nhi = (N >> shift) + 2;
        vec2_t* lo = static_cast<vec2_t*>(arena.alloc(sizeof(vec2_t) * nlo));
        vec2_t* hi = static_cast<vec2_t*>(arena.alloc(sizeof(vec2_t) * nhi));
        if (!lo || !hi) return false;
        gen_twiddles(lo, nlo, 1, N, P->sign, st);
        gen_twiddles(hi, nhi, uint64_t(nlo), N, P->sign, st);
        P->tw_lo = lo;
        P->tw_hi = hi;
        P->tw_shift = shift;
    }
    return true;
}

// runs `plan` once on device data to precompute a spectrum (contiguous, batch 1)
static bool transform_once(const FftPlan& plan, const vec2_t* in, vec2_t* out, cudaStream_t st) {
    size_t ws_bytes = workspace_bytes(plan, 1);
    void* ws_mem = nullptr;
    if (ws_bytes) {
        cudaError_t e = cudaMalloc(&ws_mem, ws_bytes);
        if (e != cudaSuccess) {
            note_cuda_error(e);
            return false;
        }
    }
    Workspace ws;
    ws.base = static_cast<char*>(ws_mem);
    ws.size = ws_bytes;
    Layout l;
    l.batch = 1;
    l.bs = plan.N;
    std::vector<PassDesc> descs;
    bool ok = build_passes(plan, in, l, out, l, real_t(1), ws, descs);
    if (ok) run_passes(descs, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        note_cuda_error(e);
        ok = false;
    }
    if (ws_mem) cudaFree(ws_mem);
    return ok;
}

// The tuner's search space: each variant changes one planning decision of
// the default rule (variant 0); all compute the same transform.
PlanVariant plan_variant(uint32_t index) {
    PlanVariant v;
    switch (index) {
        case 1: v.rmax = 512; break;                  // shorter passes, more of them
        case 2: v.rmax = 256; v.lanes = 16; break;     // short passes, wide tiles
        case 3: v.no_fused = true; break;              // shared-memory tiles
        case 4: v.single_cap = 1024; break;            // split lengths above 1024
        case 5: v.reverse = true; break;               // pass order reversed
        case 6: v.lanes_mul = 2; break;                // twice the lanes per multi-pass tile
        case 7: v.single_div = 2; break;               // half the lanes per single-pass tile
        case 8: v.no_rader = true; break;              // Bluestein instead of Rader
        case 9: v.tc = true; break;                    // tensor-core radix-16 stages
        default: break;
    }
    return v;
}

// 1: a Bluestein plan sizes its convolution for the pass limits of its own
// variant (the uneven batch's 2048-point tiles and 512-point passes)
#ifndef KFFT_BLUESTEIN_PLAN_AWARE
#define KFFT_BLUESTEIN_PLAN_AWARE 1
#endif

FftPlan* make_plan(uint32_t N, int sign, DeviceArena& arena, cudaStream_t st,
                   uint32_t max_prime, const PlanVariant& var) {
    FftPlan* P = new FftPlan();
    P->N = N;
    P->var = var;
#if defined(KFFT_HALF_SCALAR)
    P->tc = var.tc;
#endif
    P->sign = sign;
    if (N == 0) return P;
    if (is_direct_length(N, max_prime)) {
        P->method = METHOD_DIRECT;
        if (!build_direct(P, arena, st)) {
            delete P;
            return nullptr;
        }
        return P;
    }
    if (is_prime(N) && is_direct_length(N - 1, max_prime) && !var.no_rader) {
        // ---- Rader: X[g^-q] = x0 + sum_j x[g^j] W^(g^(j-q)) ------------------
        P->method = METHOD_RADER;
        const uint32_t L = N - 1;
        P->L = L;
        P->generator = primitive_root(N);
        const uint32_t g = P->generator;
        const uint32_t ginv = modpow(g, N - 2, N);
        std::vector<uint32_t> gp(L), ip(L);
        uint64_t a = 1, b = 1;
        for (uint32_t j = 0; j < L; ++j) {
            gp[j] = uint32_t(a);
            ip[j] = uint32_t(b);
            a = a * g % N;
            b = b * ginv % N;
        }
        uint32_t* dgp = static_cast<uint32_t*>(arena.alloc(sizeof(uint32_t) * L));
        uint32_t* dip = static_cast<uint32_t*>(arena.alloc(sizeof(uint32_t) * L));
        vec2_t* kern = static_cast<vec2_t*>(arena.alloc(sizeof(vec2_t) * L));
        vec2_t* spec = static_cast<vec2_t*>(arena.alloc(sizeof(vec2_t) * L));
        if (!dgp || !dip || !kern || !spec) {
            delete P;
            return nullptr;
        }
        cudaMemcpyAsync(dgp, gp.data(), sizeof(uint32_t) * L, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(dip, ip.data(), sizeof(uint32_t) * L, cudaMemcpyHostToDevice, st);
        P->gperm = dgp;
        P->iperm = dip;
        P->sub_fwd = make_plan(L, -1, arena, st, max_prime, var);
        P->sub_inv = make_plan(L, +1, arena, st, max_prime, var);
        if (!P->sub_fwd || !P->sub_inv) {
            delete P;
            return nullptr;
        }
        // kernel s[j] = W_N^(g^-j) in the direction of the plan, spectrum / L
        gen_rader_kernel(kern, dip, N, sign, st);
        if (!transform_once(*P->sub_fwd, kern, spec, st)) {
            delete P;
            return nullptr;
        }
        scale_table(spec, L, 1.0 / double(L), st);
        P->spectrum = spec;
        return P;
    }
    // ---- Bluestein: X_k = c_k sum_n (x_n c_n) conj(c_{k-n}) --------------------
    P->method = METHOD_BLUESTEIN;
#if KFFT_BLUESTEIN_PLAN_AWARE
    const uint32_t b_rmax = std::min(var.rmax, kMultiRmax);
    const uint32_t b_single = std::min(std::min(var.tile_cap, var.single_cap), kRegTile);
    uint64_t M = bluestein_length(2 * uint64_t(N) - 1, b_rmax, b_single);
#else
    uint64_t M = bluestein_length(2 * uint64_t(N) - 1);
#endif
    if (M > 0xFFFFFFFFull) {
        delete P;
        return nullptr;
    }
    P->L = uint32_t(M);
    vec2_t* chirp = static_cast<vec2_t*>(arena.alloc(sizeof(vec2_t) * N));
    vec2_t* filt = static_cast<vec2_t*>(arena.alloc(sizeof(vec2_t) * M));
    vec2_t* spec = static_cast<vec2_t*>(arena.alloc(sizeof(vec2_t) * M));
    if (!chirp || !filt || !spec) {
        delete P;
        return nullptr;
    }
    gen_chirp(chirp, N, N, sign, st);
    gen_bluestein_filter(filt, chirp, N, uint32_t(M), st);
    P->sub_fwd = make_plan(uint32_t(M), -1, arena, st, max_prime, var);
    P->sub_inv = make_plan(uint32_t(M), +1, arena, st, max_prime, var);
    if (!P->sub_fwd || !P->sub_inv) {
        delete P;
        return nullptr;
    }
    if (!transform_once(*P->sub_fwd, filt, spec, st)) {
        delete P;
        return nullptr;
    }
    scale_table(spec, uint32_t(M), 1.0 / double(M), st);
    P->chirp = chirp;
    P->spectrum = spec;
    return P;
}

void set_tensor_cores(FftPlan* p, bool on) {
    if (!p) return;
    p->tc = on;
    set_tensor_cores(p->sub_fwd, on);
    set_tensor_cores(p->sub_inv, on);
}

std::string describe(const FftPlan& p) {
    std::ostringstream o;
    const char* m[] = {"direct", "rader", "bluestein"};
    o << "N=" << p.N << " " << m[p.method];
    if (p.method != METHOD_DIRECT) {
        o << " L=" << p.L << " [" << describe(*p.sub_fwd) << "]";
        return o.str();
    }
    bool has16 = false;
    for (const PassSpec& s : p.passes) {
        o << " | R=" << s.R << " Ns=" << s.Ns << " radices=";
        for (size_t i = 0; i < s.radices.size(); ++i) {
            o << (i ? "," : "") << int(s.radices[i]);
            has16 = has16 || s.radices[i] == 16;
        }
    }
    // variant knobs that change the kernels but not the pass split
    if (p.var.lanes && p.passes.size() > 1) o << " | lanes=" << p.var.lanes;
    if (p.var.lanes_mul > 1 && p.passes.size() > 1) o << " | lanes x" << p.var.lanes_mul;
    if (p.var.single_div > 1 && p.passes.size() == 1) o << " | tiles /" << p.var.single_div;
    if (p.var.no_fused) o << " | smem";
    if (p.tc && has16) o << " | tc";
    return o.str();
}

// ---------------------------------------------------------------------------
// workspace and pass descriptors
// ---------------------------------------------------------------------------
static size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

size_t workspace_bytes(const FftPlan& p, uint32_t batch) {
    if (p.N == 0) return 0;
    if (p.method == METHOD_DIRECT) {
        size_t per = round256(sizeof(vec2_t) * size_t(p.N) * batch);
        if (p.passes.size() >= 3) return 2 * per;
        if (p.passes.size() == 2) return per;
        return 0;
    }
    size_t a = round256(sizeof(vec2_t) * size_t(p.L) * batch);
    size_t extra = (p.method == METHOD_RADER) ? round256(sizeof(vec2_t) * 2 * size_t(batch)) : 0;
    return a + extra + std::max(workspace_bytes(*p.sub_fwd, batch), workspace_bytes(*p.sub_inv, batch));
}

struct Fuse {
    uint8_t pro_op = PRO_NONE, epi_op = EPI_NONE;
    const vec2_t* pro_tab = nullptr;
    const uint32_t* pro_perm = nullptr;
    uint32_t pro_bound = 0;
    const vec2_t* epi_tab = nullptr;
    const uint32_t* epi_perm = nullptr;
    uint32_t epi_bound = 0;
    const vec2_t* aux_in = nullptr;
    vec2_t* aux_out = nullptr;
    uint64_t aux_in_bs = 0, aux_out_bs = 0;
    uint32_t aux_out_es = 1;
};

static PassDesc make_desc(const FftPlan& P, size_t pi, const vec2_t* in, const Layout& lin,
                          vec2_t* out, const Layout& lout, real_t scale) {
    const PassSpec& s = P.passes[pi];
    PassDesc d;
    memset(&d, 0, sizeof(d));
    d.in = in;
    d.out = out;
    d.in_bs = lin.bs;
    d.out_bs = lout.bs;
    d.in_es = lin.es;
    d.out_es = lout.es;
    d.batch = lin.batch;
    d.N = P.N;
    d.R = s.R;
    d.Ns = s.Ns;
    d.lanes_j = P.N / s.R;
    d.order = lin.order;
    d.inv = P.sign > 0 ? 1 : 0;
#if defined(KFFT_HALF_SCALAR)
    d.tc = P.tc ? 1 : 0;
#endif
    d.nrad = uint8_t(s.radices.size());
    for (size_t i = 0; i < s.radices.size(); ++i) d.rad[i] = s.radices[i];
    const uint32_t cap = tile_capacity();
    uint32_t C;
    if (d.order == ORDER_B) {
        // consecutive lanes are consecutive sequences (columns of a 2D
        // array): at least 16 (128-byte segments), and, as for row lanes
        // below, enough that every thread has a butterfly in every inner stage
        uint32_t want = 16;
        const uint32_t share = lane_share(s.R);
        for (uint8_t r : s.radices)
            want = std::max<uint32_t>(want, (kPassThreads * r + share * s.R - 1) / (share * s.R));
        C = std::min<uint32_t>(want, std::max<uint32_t>(1, cap / s.R));
        C = std::min(C, d.batch);
        d.load_mode = MODE_LANE;
        d.store_mode = MODE_LANE;
    } else if (d.lanes_j == 1) {
        const uint32_t target = ((sizeof(vec2_t) == 8) ? 4096 : 2048) / std::max<uint32_t>(1, P.var.single_div);
        C = std::max<uint32_t>(1, std::min(target / std::max<uint32_t>(s.R, 1), cap / std::max<uint32_t>(s.R, 1)));
        C = std::min(C, d.batch);
        d.load_mode = MODE_ELEM;
        d.store_mode = MODE_ELEM;
    } else {
        // enough lanes that every thread (or half of them, lane_share) has a
        // butterfly in every inner stage (C * R / radix >= threads), and at
        // least kMultiLanes for row segments
        uint32_t want = kMultiLanes;
        const uint32_t share = lane_share(s.R);
        for (uint8_t r : s.radices)
            want = std::max<uint32_t>(want, (kPassThreads * r + share * s.R - 1) / (share * s.R));
        C = std::min(P.var.lanes ? P.var.lanes : want * std::max<uint32_t>(1, P.var.lanes_mul), d.lanes_j);
        d.load_mode = MODE_LANE;
        d.store_mode = (s.Ns == 1) ? MODE_ELEM : MODE_LANE;
    }
    if (C < 1) C = 1;
    // register-resident tile when every inner radix is <= 16 and each thread's
    // share of every inner pass fits its register budget (lower C if needed)
    {
        bool radix_ok = (!s.radices.empty() || s.R == 1) && !P.var.no_fused;
        for (uint8_t r : s.radices) radix_ok = radix_ok && r <= 16;
        for (uint32_t c = C; radix_ok && c >= 1; --c) {
            const bool fits = reg_tile_fits(s.R, c, P.var.tile_cap);
            const bool coalesced_enough = (d.order == ORDER_J && d.lanes_j == 1) ||
                                          c >= std::min<uint32_t>(C, kRegLanes);
            if (fits && coalesced_enough) {
                C = c;
                d.regmode = 1;
                break;
            }
            if (!coalesced_enough) break;
        }
    }
    // a shared-memory tile must fit the per-CTA budget whatever the variant asked
    while (!d.regmode && C > 1 && smem_for(C * s.R) > kSmemBudget) --C;
    d.C = C;
    // power-of-two register tiles of 16..4096 points run a compile-time body
    // (FP32 only: in FP64 its fully unrolled stages spill and the FP64 pipe,
    // not index arithmetic, bounds the pass)
    d.spec = 0;
#if defined(KFFT_HALF_SCALAR)
    if (d.regmode && !d.tc && s.R >= 16 && s.R <= 4096 && (s.R & (s.R - 1)) == 0) {
        uint32_t l = 0;
        while ((1u << l) < s.R) ++l;
        d.spec = uint8_t(l);
    }
#endif
    const uint64_t lanes = uint64_t(d.batch) * d.lanes_j;
    d.tiles = uint32_t((lanes + C - 1) / C);
    uint32_t elems = C * s.R;
    if (d.regmode) {
        d.threads = kPassThreads;
        const uint32_t nbuf = s.radices.size() >= 3 ? 2u : (s.radices.size() == 2 ? 1u : 0u);
        d.lane_stride = spec_lane_stride(s.R, C, d.load_mode == MODE_LANE,
                                         d.store_mode == MODE_LANE, kPassThreads);
        d.smem_bytes = nbuf * (C * d.lane_stride + 1u) * uint32_t(sizeof(vec2_t));
    } else {
        uint32_t t = (elems + 7) / 8;
        t = (t + 31) / 32 * 32;
        d.threads = std::max<uint32_t>(64, std::min<uint32_t>(kPassThreads, t));
        d.smem_bytes = smem_for(elems);
    }
    d.div_R.init(s.R);
    d.div_lanes_j.init(d.lanes_j);
    d.div_batch.init(d.batch);
    d.div_Ns.init(s.Ns);
    d.div_C.init(C);
    d.tw_inner = s.tw_inner;
    d.tw_lo = P.tw_lo;
    d.tw_hi = P.tw_hi;
    d.tw_shift = P.tw_shift;
    d.tw_mul = d.lanes_j / s.Ns;
    d.scale = scale;
    return d;
}

PassDesc make_pass_desc(const FftPlan& P, size_t pass, const vec2_t* in, const Layout& lin,
                        vec2_t* out, const Layout& lout, real_t scale) {
    return make_desc(P, pass, in, lin, out, lout, scale);
}

static void apply_fuse(PassDesc& d, const Fuse& f, bool first, bool last) {
    if (first) {
        d.pro_op = f.pro_op;
        d.pro_tab = f.pro_tab;
        d.pro_perm = f.pro_perm;
        d.pro_bound = f.pro_bound;
    }
    if (last) {
        d.epi_op = f.epi_op;
        d.epi_tab = f.epi_tab;
        d.epi_perm = f.epi_perm;
        d.epi_bound = f.epi_bound;
        d.aux_in = f.aux_in;
        d.aux_out = f.aux_out;
        d.aux_in_bs = f.aux_in_bs;
        d.aux_out_bs = f.aux_out_bs;
        d.aux_out_es = f.aux_out_es;
    }
}

static bool build_direct_passes(const FftPlan& P, const vec2_t* in, const Layout& lin, vec2_t* out,
                                const Layout& lout, real_t scale, const Fuse& f, Workspace& ws,
                                std::vector<PassDesc>& descs) {
    const size_t m = P.passes.size();
    if (m == 0) return true;
    Layout mid;
    mid.batch = lin.batch;
    mid.order = lin.order;
    if (lin.order == ORDER_B) {
        mid.bs = 1;
        mid.es = lin.batch;
    } else {
        mid.bs = P.N;
        mid.es = 1;
    }
    vec2_t* s1 = nullptr;
    vec2_t* s2 = nullptr;
    if (m >= 2 && !(s1 = ws.take(size_t(P.N) * lin.batch))) return false;
    if (m >= 3 && !(s2 = ws.take(size_t(P.N) * lin.batch))) return false;
    const vec2_t* cur = in;
    Layout lcur = lin;
    for (size_t i = 0; i < m; ++i) {
        const bool last = (i + 1 == m);
        vec2_t* dst = last ? out : ((i % 2 == 0) ? s1 : s2);
        Layout ldst = last ? lout : mid;
        PassDesc d = make_desc(P, i, cur, lcur, dst, ldst, last ? scale : real_t(1));
        apply_fuse(d, f, i == 0, last);
        descs.push_back(d);
        cur = dst;
        lcur = ldst;
    }
    return true;
}

// The passes of one transform.  A Rader or Bluestein plan runs its forward
// sub-transform with the gather or pre-chirp in the first pass's loads and
// the spectrum product in the last pass's stores, then its inverse
// sub-transform with the output permutation or post-chirp in the last pass's
// stores.  Returns false when the layouts or the workspace do not allow it.
bool build_passes(const FftPlan& P, const vec2_t* in, const Layout& lin, vec2_t* out,
                  const Layout& lout, real_t scale, Workspace& ws, std::vector<PassDesc>& descs) {
    if (P.N == 0) return true;
    if (uint64_t(lin.batch) * P.N >= (uint64_t(1) << 32) && P.method == METHOD_DIRECT &&
        P.passes.size() > 1)
        return false;  // lane indices are 32-bit
    Fuse none;
    if (P.method == METHOD_DIRECT) return build_direct_passes(P, in, lin, out, lout, scale, none, ws, descs);
    if (lin.order != ORDER_J || lout.order != ORDER_J) return false;
    const uint32_t B = lin.batch;
    Layout la;
    la.batch = B;
    la.bs = P.L;
    la.es = 1;
    vec2_t* A = ws.take(size_t(P.L) * B);
    if (!A) return false;
    if (P.method == METHOD_BLUESTEIN) {
        Fuse ff;
        ff.pro_op = PRO_CHIRP;
        ff.pro_tab = P.chirp;
        ff.pro_bound = P.N;
        ff.epi_op = EPI_MUL;
        ff.epi_tab = P.spectrum;
        Layout lx = lin;  // the input seen as length-L sequences with the caller's strides
        const size_t mark = ws.used;
        if (!build_direct_passes(*P.sub_fwd, in, lx, A, la, real_t(1), ff, ws, descs)) return false;
        ws.used = mark;  // the inverse reuses the forward's scratch (stream ordered)
        Fuse fi;
        fi.epi_op = EPI_CHIRP;
        fi.epi_tab = P.chirp;
        fi.epi_bound = P.N;
        return build_direct_passes(*P.sub_inv, A, la, out, lout, scale, fi, ws, descs);
    }
    // Rader
    vec2_t* pairs = ws.take(size_t(2) * B);
    if (!pairs) return false;
    Fuse ff;
    ff.pro_op = PRO_GATHER;
    ff.pro_perm = P.gperm;
    ff.epi_op = EPI_RADER_FWD;
    ff.epi_tab = P.spectrum;
    ff.aux_in = in;
    ff.aux_in_bs = lin.bs;
    ff.aux_out = pairs;
    const size_t mark = ws.used;
    if (!build_direct_passes(*P.sub_fwd, in, lin, A, la, real_t(1), ff, ws, descs)) return false;
    ws.used = mark;  // the inverse reuses the forward's scratch (stream ordered)
    Fuse fi;
    fi.epi_op = EPI_RADER_INV;
    fi.epi_perm = P.iperm;
    fi.aux_in = pairs;
    fi.aux_out = out;
    fi.aux_out_bs = lout.bs;
    fi.aux_out_es = lout.es;
    return build_direct_passes(*P.sub_inv, A, la, A, la, scale, fi, ws, descs);
}

void run_passes(const std::vector<PassDesc>& descs, cudaStream_t st) {
    for (const PassDesc& d : descs) launch_pass(d, st);
}

}  // namespace kfft
