// pass_reg.cu -- the register-resident pass kernel k_pass_reg.
#include "fft_device.cuh"

namespace kfft {

template <bool INV>
__global__ void __launch_bounds__(kPassThreads, KFFT_REG_MINBLOCKS) k_pass_reg(const __grid_constant__ PassDesc d,
                                                              const __grid_constant__ PassExtra x) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    tile_body_reg<INV>(d, x, blockIdx.x, reinterpret_cast<vec2_t*>(smem_raw));
}

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
    if (d.inv) k_pass_reg<true><<<d.tiles, d.threads, d.smem_bytes, st>>>(d, x);
    else k_pass_reg<false><<<d.tiles, d.threads, d.smem_bytes, st>>>(d, x);
    note_cuda_error(cudaGetLastError());
    count_launch();
}

}  // namespace kfft
