// Prints the host planning arithmetic of plan_host.h (FP32 build) for the
// CPU test tests/test_plan_host.py: power-of-two pass splits, the lane
// strides the shared-memory bank model picks with their wavefront costs,
// Bluestein convolution lengths and balanced multi-pass splits.
#include "plan_host.h"

#include <cstdio>

int main() {
    for (uint32_t L = 13; L <= 28; ++L)
        for (uint32_t rmax : {1024u, 512u, 256u}) {
            std::printf("split %u %u", L, rmax);
            for (uint32_t R : kfft::pow2_split(1u << L, rmax)) std::printf(" %u", R);
            std::printf("\n");
        }
    const uint32_t cases[][5] = {
        {512, 8, 1, 0, 256}, {512, 8, 1, 1, 256}, {1024, 4, 1, 1, 256}, {256, 16, 1, 1, 256},
        {256, 16, 1, 0, 256}, {128, 32, 1, 1, 256}, {64, 64, 1, 1, 256}, {64, 32, 0, 0, 256},
        {4096, 1, 0, 0, 256}, {2048, 2, 0, 0, 256}, {512, 16, 1, 1, 512}, {1024, 8, 1, 0, 512},
        {1000, 4, 1, 1, 256}, {768, 5, 1, 0, 256}, {390, 10, 1, 1, 256}, {616, 6, 1, 0, 256}};
    for (const auto& c : cases) {
        const uint32_t R = c[0], C = c[1], T = c[4];
        const bool ll = c[2] != 0, sl = c[3] != 0;
        const uint32_t s = kfft::lane_stride_search(R, C, ll, sl, T);
        const uint32_t base = R + R / kfft::kRowElems;
        std::printf("stride %u %u %u %u %u %u %llu %llu\n", R, C, c[2], c[3], T, s,
                    (unsigned long long)kfft::tile_smem_cost(R, C, s, ll, sl, T),
                    (unsigned long long)kfft::tile_smem_cost(R, C, base, ll, sl, T));
    }
    for (uint32_t n : {5u, 17u, 127u, 1009u, 4099u, 65521u, 104729u, 700523u, 999983u}) {
        std::printf("bluestein %u %llu\n", n, (unsigned long long)kfft::bluestein_length(2ull * n - 1));
        // the pass limits of the uneven batch's queue plans
        std::printf("bluestein_q %u %llu\n", n,
                    (unsigned long long)kfft::bluestein_length(2ull * n - 1, 512, 2048));
    }
    for (uint32_t n : {240240u, 1000000u, 729000u, 1081080u, 4096u * 243u})
        for (uint32_t rmax : {1024u, 512u, 256u}) {
            std::printf("balanced %u %u", n, rmax);
            for (uint32_t R : kfft::split_passes(n, rmax)) std::printf(" %u", R);
            std::printf("\n");
        }
    for (uint32_t R : {1u, 2u, 3u, 16u, 32u, 48u, 60u, 72u, 81u, 90u, 96u, 100u, 105u, 108u, 112u,
                       120u, 126u, 144u, 243u, 250u, 270u, 432u, 486u, 500u, 540u, 567u, 576u,
                       600u, 630u, 648u, 672u, 700u, 720u, 729u, 750u, 756u, 864u, 945u, 1000u,
                       1008u, 2048u, 2187u, 3125u, 3888u, 4096u, 4095u, 3003u, 496u, 17u * 27u})
    {
        std::printf("radices %u", R);
        for (uint8_t q : kfft::inner_radices(R)) std::printf(" %u", unsigned(q));
        std::printf("\n");
    }
    return 0;
}
