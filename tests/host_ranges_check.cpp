// Property check of the host-buffer pipeline's chunk and copy ranges
// (chunk_start, copy_range in kfft_gb300/csrc/engine.cuh), built with the
// host compiler by tests/test_host_ranges.py.  Exits non-zero on the first
// violated property, printing the case.
#include "engine.cuh"

#include <cstdio>
#include <random>
#include <vector>

using kfft::CopyRange;

static int fail(const char* what, size_t total, size_t k) {
    std::printf("FAIL %s (total %zu, chunks %zu)\n", what, total, k);
    return 1;
}

// chunks of `per` bytes per sequence over `batch` sequences, `k` chunks
static int check(size_t per, uint64_t batch, uint64_t k) {
    const size_t total = per * batch;
    std::vector<size_t> b(k + 1);
    for (uint64_t i = 0; i <= k; ++i) b[i] = per * kfft::chunk_start(i, k, batch);
    if (b[0] != 0 || b[k] != total) return fail("chunk starts span the batch", total, k);
    for (uint64_t i = 0; i < k; ++i)
        if (batch >= 2 * k && b[i + 1] <= b[i]) return fail("chunk starts increase", total, k);
    std::vector<CopyRange> r(k);
    for (uint64_t i = 0; i < k; ++i) r[i] = kfft::copy_range(b[i], b[i + 1], total, i == 0, i + 1 == k);
    for (uint64_t i = 0; i < k; ++i) {
        // copies in and copies out each tile [0, total) in order
        if (r[i].in0 != (i ? r[i - 1].in1 : 0) || r[i].out0 != (i ? r[i - 1].out1 : 0))
            return fail("copy ranges are contiguous", total, k);
        if (r[i].in1 < r[i].in0 || r[i].out1 < r[i].out0) return fail("copy ranges are ordered", total, k);
        // interior ends on 256-byte boundaries (or clamped to the end)
        auto aligned = [&](size_t x) { return x % 256 == 0 || x == total; };
        if (i + 1 < k && (!aligned(r[i].in1) || !aligned(r[i].out1))) return fail("256-byte ends", total, k);
        // chunk i's transform reads [b[i], b[i+1]): copied by copies in 0..i
        if (r[i].in1 < b[i + 1]) return fail("input copied before its transform", total, k);
        // copy out i reads only output of transforms 0..i
        if (r[i].out1 > b[i + 1]) return fail("only finished output copied out", total, k);
        // copy out i may run beside copies in i+1..: their ranges never meet
        // (in-place host buffers stay correct)
        for (uint64_t j = i + 1; j < k; ++j)
            if (r[i].out1 > r[j].in0 && r[j].in1 > r[i].out0 && r[j].in1 > r[j].in0 && r[i].out1 > r[i].out0)
                return fail("copy out i and later copies in are disjoint", total, k);
    }
    if (r[k - 1].in1 != total || r[k - 1].out1 != total) return fail("last ranges reach the end", total, k);
    return 0;
}

int main() {
    std::mt19937_64 rng(7);
    const size_t pers[] = {8, 16, 24000, 32768, 262152, 8 * 4095, 16 * 4096, 4 * 3000 + 8};
    for (size_t per : pers)
        for (uint64_t k : {2ull, 3ull, 4ull, 7ull, 16ull})
            for (uint64_t batch : {k, 2 * k, 3 * k + 1, 100 * k + 13})
                if (check(per, batch, k)) return 1;
    for (int t = 0; t < 20000; ++t) {
        const size_t per = 8 * (1 + rng() % 100000);
        const uint64_t k = 2 + rng() % 15;
        const uint64_t batch = k + rng() % 5000;
        if (check(per, batch, k)) return 1;
    }
    std::printf("ok\n");
    return 0;
}
