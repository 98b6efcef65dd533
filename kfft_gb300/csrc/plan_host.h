// plan_host.h -- host-only planning arithmetic shared by the planner and its
// CPU tests: prime factors, the inner radix schedule of a tile, the splits of
// a length into passes, the Bluestein convolution length, and the
// shared-memory bank model that picks the lane stride of a register tile.  No device code; builds with the
// host compiler.
#pragma once

#include <algorithm>
#include <cstdint>
#include <functional>
#include <vector>

#include "engine.cuh"

namespace kfft {

inline std::vector<uint32_t> prime_factors(uint32_t n) {
    std::vector<uint32_t> f;
    for (uint32_t p = 2; uint64_t(p) * p <= n; ++p)
        while (n % p == 0) {
            f.push_back(p);
            n /= p;
        }
    if (n > 1) f.push_back(n);
    return f;
}

// Estimated real flops per point of one inner stage of radix r: the
// butterfly (register DFT) plus the r-1 twiddle products of a later stage.
// Used only to break ties between schedules with equally many stages.
inline double radix_flops_per_point(uint32_t r) {
    double bfly;
    switch (r) {
        case 2: bfly = 4; break;
        case 3: bfly = 16; break;
        case 4: bfly = 16; break;
        case 5: bfly = 40; break;
        case 6: bfly = 44; break;    // Good-Thomas 2 x 3
        case 7: bfly = 72; break;
        case 8: bfly = 52; break;
        case 9: bfly = 120; break;   // Cooley-Tukey 3 x 3
        case 10: bfly = 100; break;  // Good-Thomas 2 x 5
        case 11: bfly = 140; break;
        case 12: bfly = 112; break;  // Good-Thomas 4 x 3
        case 13: bfly = 190; break;
        case 14: bfly = 172; break;  // Good-Thomas 2 x 7
        case 15: bfly = 200; break;  // Good-Thomas 3 x 5
        case 16: bfly = 144; break;
        default: bfly = 4.0 * r * r; break;  // odd primes 17..31
    }
    return (bfly + 6.0 * (r - 1)) / r;
}

// Inner radix schedule of a tile length R.  Powers of two: 16s, then 8, 4 or
// 2 (the compile-time tile bodies assume exactly this).  Other lengths: the
// fewest stages whose radices multiply to R, each radix one the register
// butterflies implement (2-16, including the composites 6, 9, 10, 12, 14,
// 15), ties broken by the least estimated arithmetic; prime factors 17-31
// (shared-memory tiles only) are stages of their own.  Every stage is a
// shared-memory round trip and a barrier, which is what bounds a mixed-radix
// tile: 729 = 3^6 runs as 9, 9, 9 instead of six radix-3 stages.  Radices are
// listed largest first.
inline std::vector<uint8_t> inner_radices(uint32_t R) {
    std::vector<uint8_t> r;
    if (R >= 2 && (R & (R - 1)) == 0) {
        uint32_t e2 = 0;
        while ((1u << e2) < R) ++e2;
        while (e2 >= 4) {
            r.push_back(16);
            e2 -= 4;
        }
        if (e2 == 3) r.push_back(8);
        if (e2 == 2) r.push_back(4);
        if (e2 == 1) r.push_back(2);
        return r;
    }
    std::vector<uint8_t> big;
    uint32_t rest = R;
    for (uint32_t p : prime_factors(R))
        if (p > 16) {
            big.push_back(uint8_t(p));
            rest /= p;
        }
    // best[d]: (stages, flops) of the best schedule of divisor d of `rest`
    static const uint32_t kSet[] = {16, 15, 14, 13, 12, 11, 10, 9, 8, 7, 6, 5, 4, 3, 2};
    std::vector<uint32_t> divs;
    for (uint32_t d = 1; uint64_t(d) * d <= rest; ++d)
        if (rest % d == 0) {
            divs.push_back(d);
            if (d != rest / d) divs.push_back(rest / d);
        }
    std::sort(divs.begin(), divs.end());
    std::vector<uint32_t> stages(divs.size(), 0), pick(divs.size(), 0);
    std::vector<double> flops(divs.size(), 0.0);
    auto index_of = [&](uint32_t d) {
        return size_t(std::lower_bound(divs.begin(), divs.end(), d) - divs.begin());
    };
    for (size_t i = 1; i < divs.size(); ++i) {
        const uint32_t d = divs[i];
        stages[i] = UINT32_MAX;
        for (uint32_t q : kSet) {
            if (d % q) continue;
            const size_t j = index_of(d / q);
            if (stages[j] == UINT32_MAX) continue;
            const uint32_t s = stages[j] + 1;
            const double f = flops[j] + radix_flops_per_point(q);
            if (s < stages[i] || (s == stages[i] && f < flops[i] - 1e-9)) {
                stages[i] = s;
                flops[i] = f;
                pick[i] = q;
            }
        }
    }
    for (uint32_t d = rest; d > 1;) {
        const uint32_t q = pick[index_of(d)];
        r.push_back(uint8_t(q));
        d /= q;
    }
    std::sort(r.rbegin(), r.rend());
    for (uint8_t p : big) r.push_back(p);
    return r;
}

// Largest pass length of a balanced multi-pass split.
constexpr uint32_t kMultiRmax = 1024;

// the least 7-smooth number >= n
inline uint64_t next_smooth(uint64_t n) {
    uint64_t best = UINT64_MAX;
    for (uint64_t a = 1; a < 2 * n + 2; a *= 2)
        for (uint64_t b = a; b < 2 * n + 2; b *= 3)
            for (uint64_t c = b; c < 2 * n + 2; c *= 5)
                for (uint64_t d = c; d < 2 * n + 2; d *= 7)
                    if (d >= n && d < best) best = d;
    return best;
}

// split a DIRECT length into pass lengths, balanced, each <= rmax
inline std::vector<uint32_t> split_passes(uint32_t N, uint32_t rmax) {
    std::vector<uint32_t> f = prime_factors(N);
    std::sort(f.rbegin(), f.rend());
    for (uint32_t m = 1; m <= 32; ++m) {
        std::vector<uint64_t> g(m, 1);
        bool ok = true;
        for (uint32_t p : f) {
            // place in the group with the smallest product that still fits
            int best = -1;
            for (uint32_t i = 0; i < m; ++i)
                if (g[i] * p <= rmax && (best < 0 || g[i] < g[best])) best = int(i);
            if (best < 0) {
                ok = false;
                break;
            }
            g[best] *= p;
        }
        if (ok) {
            std::vector<uint32_t> out;
            for (uint64_t v : g)
                if (v > 1) out.push_back(uint32_t(v));
            std::sort(out.rbegin(), out.rend());
            if (out.empty()) out.push_back(1);
            return out;
        }
    }
    return {};
}

// Length of the Bluestein convolution for a minimum of m: the 7-smooth M >= m
// (up to 2m) with the least estimated cost M * passes(M) * (1 + 0.15 * odd
// factors).  A pass is one HBM round trip, and radix-3/5/7 stages cost about
// 30% more per point than radix-2/4/8/16 ones on this kernel; the nearest
// 7-smooth length is often odd-heavy or one pass deeper than a power-of-two
// one slightly above it.  `rmax` and `single` are the plan's longest pass of
// a multi-pass split and longest one-pass length (the uneven batch's queue
// plans use 512 and 2048).
#ifndef KFFT_BLUESTEIN_ODD_COST
#define KFFT_BLUESTEIN_ODD_COST 0.15
#endif
inline uint64_t bluestein_length(uint64_t m, uint32_t rmax = kMultiRmax,
                                 uint32_t single = kRegTile) {
    uint64_t best = next_smooth(m);
    double best_cost = -1.0;
    for (uint64_t a = 1; a <= 2 * m; a *= 2)
        for (uint64_t b = a; b <= 2 * m; b *= 3)
            for (uint64_t c = b; c <= 2 * m; c *= 5)
                for (uint64_t d = c; d <= 2 * m; d *= 7) {
                    if (d < m || d > 0xFFFFFFFFull) continue;
                    uint64_t r = d;
                    int odd = 0;
                    for (uint64_t q : {3ull, 5ull, 7ull})
                        while (r % q == 0) {
                            r /= q;
                            ++odd;
                        }
                    const size_t passes = std::max<size_t>(1, split_passes(uint32_t(d), rmax).size());
                    const double cost = double(d) * double(d <= single ? 1 : passes) *
                                        (1.0 + KFFT_BLUESTEIN_ODD_COST * odd);
                    if (best_cost < 0 || cost < best_cost) {
                        best_cost = cost;
                        best = d;
                    }
                }
    return best;
}

// ---------------------------------------------------------------------------
// shared-memory lane stride of the register-tile bodies
// ---------------------------------------------------------------------------
// Elements per 128-byte shared-memory row (one request of a warp-wide access).
constexpr uint32_t kRowElems = 128 / sizeof(vec2_t);

// Shared-memory wavefronts of one warp-wide access to the element slots `idx`
// (-1: thread idle): every kRowElems threads form one request, which takes as
// many wavefronts as the most distinct elements that share a bank group
// (slot mod kRowElems).
inline uint32_t smem_wavefronts(const int64_t* idx) {
    uint32_t total = 0;
    for (uint32_t h = 0; h < 32; h += kRowElems) {
        int64_t seen[kRowElems];
        uint32_t n = 0;
        uint32_t per[kRowElems] = {0};
        for (uint32_t t = h; t < h + kRowElems; ++t) {
            if (idx[t] < 0) continue;
            bool dup = false;
            for (uint32_t i = 0; i < n; ++i) dup = dup || seen[i] == idx[t];
            if (dup) continue;
            seen[n++] = idx[t];
            ++per[idx[t] % kRowElems];
        }
        uint32_t worst = 0;
        for (uint32_t v : per) worst = std::max(worst, v);
        total += worst;
    }
    return total;
}

// Wavefronts of the shared-memory accesses of one tile iteration of a
// register-tile body (inner radices of R, C lanes `stride` slots apart, run
// by `threads` threads).  Stages with a global access in lane mode put
// consecutive threads on consecutive lanes; the others put them on
// consecutive butterflies of one lane.
inline uint64_t tile_smem_cost(uint32_t R, uint32_t C, uint32_t stride, bool load_lane,
                               bool store_lane, uint32_t threads) {
    auto padh = [](uint64_t i) { return i + i / kRowElems; };
    const std::vector<uint8_t> rad = inner_radices(R);
    const size_t np = rad.size();
    uint64_t cost = 0;
    uint32_t NS = 1;
    int64_t idx[32];
    for (size_t st = 0; st < np; ++st) {
        const uint32_t P = rad[st], M = R / P, items = C * M;
        const bool last = st + 1 == np;
        const bool cfast = (st == 0 && load_lane) || (last && store_lane);
        const uint32_t warps = std::min<uint32_t>(threads / 32, (items + 31) / 32);
        for (uint32_t w = 0; w < warps; ++w) {
            for (uint32_t q = 0; q < P; ++q) {
                for (int rw = 0; rw < 2; ++rw) {
                    if ((rw == 0 && st == 0) || (rw == 1 && last)) continue;
                    for (uint32_t t = 0; t < 32; ++t) {
                        const uint32_t it = w * 32 + t;
                        if (it >= items) {
                            idx[t] = -1;
                            continue;
                        }
                        uint32_t c, jj;
                        if (cfast) {
                            jj = it / C;
                            c = it % C;
                        } else {
                            c = it / M;
                            jj = it % M;
                        }
                        const uint64_t ob = uint64_t(jj / NS) * NS * P + jj % NS;
                        const uint64_t slot = rw == 0 ? padh(jj + uint64_t(q) * M) : padh(ob + uint64_t(q) * NS);
                        idx[t] = int64_t(uint64_t(c) * stride + slot);
                    }
                    cost += smem_wavefronts(idx);
                }
            }
        }
        NS *= P;
    }
    return cost;
}

// The padded lane length plus the skew (0 .. kRowElems-1 slots) with the
// fewest shared-memory wavefronts per tile: without a skew the lanes of a
// lane-major access can all fall in the same banks (a lane of 2^k >= 16
// points is a whole number of 128-byte rows).  Ties go to the smaller skew.
inline uint32_t lane_stride_search(uint32_t R, uint32_t C, bool load_lane, bool store_lane,
                                   uint32_t threads) {
    const uint32_t base = R + R / kRowElems;
    uint32_t best = base;
    uint64_t best_cost = ~uint64_t(0);
    if (C > 1 && inner_radices(R).size() > 1) {
        for (uint32_t skew = 0; skew < kRowElems; ++skew) {
            const uint64_t c = tile_smem_cost(R, C, base + skew, load_lane, store_lane, threads);
            if (c < best_cost) {
                best_cost = c;
                best = base + skew;
            }
        }
    }
    return best;
}

// FP32 powers of two (compile-time bodies): the pass lengths 16..rmax (at
// most 1024), longest first, with the least estimated time.  A pass costs its
// measured launch time relative to a 256-point pass on 2^24 points: up to 256
// points 1 (tiles of 16+ lanes, row segments of 128 bytes or more), 512
// points 1.44 and 1024 points 1.65 (8 and 4 lanes per 4096-point tile, 16 and
// 8 on the wide kernel).  Ties go to fewer passes, then to the more even
// split (lexicographically smaller lengths, longest first).  2^18 runs as 1024 x 256 (0.292 ms per forward + inverse
// step at 64 sequences, against 0.315 as 512 x 512), 2^20 as 128 x 128 x 64.
inline std::vector<uint32_t> pow2_split(uint32_t N, uint32_t rmax) {
    uint32_t L = 0;
    while ((1u << L) < N) ++L;
    uint32_t emax = 0;
    while (emax < 10 && (2u << emax) <= rmax) ++emax;
    auto cost = [](uint32_t e) { return e == 10 ? 1.65 : (e == 9 ? 1.44 : 1.0); };
    std::vector<uint32_t> best, cur;
    double best_cost = -1.0;
    // non-increasing exponents in [4, emax] summing to L
    std::function<void(uint32_t, uint32_t, double)> walk = [&](uint32_t left, uint32_t top, double c) {
        if (left == 0) {
            const bool better = best_cost < 0.0 || c < best_cost - 1e-9 ||
                                (c < best_cost + 1e-9 && (cur.size() < best.size() ||
                                                          (cur.size() == best.size() && cur < best)));
            if (better) {
                best_cost = c;
                best = cur;
            }
            return;
        }
        for (uint32_t e = std::min(top, left); e >= 4; --e) {
            cur.push_back(e);
            walk(left - e, e, c + cost(e));
            cur.pop_back();
        }
    };
    if (emax >= 4) walk(L, emax, 0.0);
    std::vector<uint32_t> Rs;
    for (uint32_t e : best) Rs.push_back(1u << e);
    return Rs;
}

}  // namespace kfft
