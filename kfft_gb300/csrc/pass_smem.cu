// pass_smem.cu -- per-pass launches: the shared-memory ping-pong tile kernel
// k_pass (any radix up to 31) and the dispatcher to the register-resident
// kernel, plus the per-pass inner-step tables.
#include "fft_device.cuh"

namespace kfft {

void launch_pass_reg(const PassDesc& d, const PassExtra& x, cudaStream_t st);

template <bool INV, bool BIG>
__global__ void __launch_bounds__(kPassThreads) k_pass(const __grid_constant__ PassDesc d,
                                                       const __grid_constant__ PassExtra x) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    tile_body<INV, BIG>(d, x, blockIdx.x, reinterpret_cast<vec2_t*>(smem_raw));
}

// One-time shared-memory limit of the shared-memory tile kernels; the
// initialisation of a function-local static is thread-safe, and a failure is
// reported on every call.
static bool configure_pass_kernels() {
    static const cudaError_t status = [] {
        const void* fns[4] = {(const void*)k_pass<false, false>, (const void*)k_pass<true, false>,
                              (const void*)k_pass<false, true>, (const void*)k_pass<true, true>};
        for (const void* f : fns) {
            cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 227 * 1024);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return e;
            }
        }
        return cudaSuccess;
    }();
    if (status != cudaSuccess) {
        note_cuda_error(status);
        return false;
    }
    return true;
}

void launch_pass(const PassDesc& d, cudaStream_t st) {
    if (!configure_pass_kernels()) return;
    const PassExtra x = make_extra(d);
    if (d.regmode) {
        launch_pass_reg(d, x, st);
        return;
    }
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

}  // namespace kfft
