// pass_reg.cu -- the register-resident pass kernel k_pass_reg.
#include "fft_device.cuh"

#include <map>
#include <mutex>
#include <utility>

namespace kfft {

template <bool INV>
__global__ void __launch_bounds__(kPassThreads, KFFT_REG_MINBLOCKS) k_pass_reg(const __grid_constant__ PassDesc d,
                                                              const __grid_constant__ PassExtra x) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    tile_body_reg<INV>(d, x, blockIdx.x, reinterpret_cast<vec2_t*>(smem_raw));
}

#if defined(KFFT_HALF_SCALAR)
// FP32 power-of-two passes with a plain prologue and more tiles than fit the
// GPU at once: a grid of resident CTAs, each running many tiles with its next
// tile's loads in flight (tile_loop_pipelined).  The FP64 build does not use
// it: the FP64 pipe, not load latency, bounds that path, and the second tile's
// registers would spill.
template <bool INV>
__global__ void __launch_bounds__(kPassThreads, 2) k_pass_pipe(const __grid_constant__ PassDesc d) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    vec2_t* sm = reinterpret_cast<vec2_t*>(smem_raw);
    switch (d.spec) {
        case 4: tile_loop_pipelined<16, INV>(d, sm); break;
        case 5: tile_loop_pipelined<32, INV>(d, sm); break;
        case 6: tile_loop_pipelined<64, INV>(d, sm); break;
        case 7: tile_loop_pipelined<128, INV>(d, sm); break;
        case 8: tile_loop_pipelined<256, INV>(d, sm); break;
        case 9: tile_loop_pipelined<512, INV>(d, sm); break;
        case 10: tile_loop_pipelined<1024, INV>(d, sm); break;
        case 11: tile_loop_pipelined<2048, INV>(d, sm); break;
        case 12: tile_loop_pipelined<4096, INV>(d, sm); break;
        default: break;
    }
}

#endif

namespace {
#if defined(KFFT_HALF_SCALAR)
// resident CTAs per SM of k_pass_pipe for a dynamic shared-memory size
int pipe_blocks_per_sm(bool inv, uint32_t smem) {
    static std::mutex mu;
    static std::map<std::pair<bool, uint32_t>, int> cache;
    std::lock_guard<std::mutex> lk(mu);
    auto key = std::make_pair(inv, smem);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    int n = 0;
    const void* f = inv ? (const void*)k_pass_pipe<true> : (const void*)k_pass_pipe<false>;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, kPassThreads, smem) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    cache[key] = n;
    return n;
}

int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}
#endif
}  // namespace

void launch_pass_reg(const PassDesc& d, const PassExtra& x, cudaStream_t st) {
    static bool configured = false;
    if (!configured) {
        for (const void* f : {(const void*)k_pass_reg<false>, (const void*)k_pass_reg<true>}) {
            cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 227 * 1024);
            if (e != cudaSuccess) {
                note_cuda_error(e);
                return;
            }
        }
        configured = true;
    }
#if defined(KFFT_HALF_SCALAR)
    static bool pipe_configured = false;
    if (!pipe_configured) {
        for (const void* f : {(const void*)k_pass_pipe<false>, (const void*)k_pass_pipe<true>}) {
            cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 227 * 1024);
            if (e != cudaSuccess) {
                note_cuda_error(e);
                return;
            }
        }
        pipe_configured = true;
    }
    if (d.spec && d.pro_op == PRO_NONE && d.threads == kPassThreads) {
        const int per_sm = pipe_blocks_per_sm(d.inv != 0, d.smem_bytes);
        const uint32_t grid = uint32_t(per_sm) * uint32_t(sm_count());
        if (per_sm > 0 && d.tiles >= 2 * grid) {
            if (d.inv) k_pass_pipe<true><<<grid, kPassThreads, d.smem_bytes, st>>>(d);
            else k_pass_pipe<false><<<grid, kPassThreads, d.smem_bytes, st>>>(d);
            note_cuda_error(cudaGetLastError());
            count_launch();
            return;
        }
    }
#endif
    if (d.inv) k_pass_reg<true><<<d.tiles, d.threads, d.smem_bytes, st>>>(d, x);
    else k_pass_reg<false><<<d.tiles, d.threads, d.smem_bytes, st>>>(d, x);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

}  // namespace kfft
