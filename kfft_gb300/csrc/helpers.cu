// helpers.cu -- the reference's post-transform helpers on the GPU: fftshift
// (kfft_shift.c:4-61, ext/2d/kfft_cpx2.c:188-240, ext/2d/kfft_scalar2.c:248-300)
// and the kfft_math API (kfft_math.c:42-148): Hadamard products, transposes,
// magnitudes and the average.  Each entry point keeps the reference signature
// and accepts host or device buffers; host buffers are staged through a
// temporary device buffer for the call.
#include <cuda_runtime.h>

#include <cstring>

#include "engine.cuh"
#include "kfft.h"

using namespace kfft;

namespace {

bool dev_ptr(const void* p) {
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// A caller buffer seen from the device: the buffer itself when it is device
// memory, else a staged copy that is written back on release when `out`.
struct DevView {
    void* host = nullptr;
    void* dev = nullptr;
    size_t bytes = 0;
    bool staged = false, out = false;
    bool open(const void* p, size_t n, bool copy_in, bool write_back, cudaStream_t st) {
        bytes = n;
        out = write_back;
        if (dev_ptr(p)) {
            dev = const_cast<void*>(p);
            return true;
        }
        host = const_cast<void*>(p);
        staged = true;
        if (cudaMalloc(&dev, n ? n : 16) != cudaSuccess) {
            cudaGetLastError();
            dev = nullptr;
            return false;
        }
        if (copy_in) cudaMemcpyAsync(dev, p, n, cudaMemcpyHostToDevice, st);
        return true;
    }
    void close(cudaStream_t st) {
        if (staged && dev) {
            if (out) cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, st);
            cudaStreamSynchronize(st);
            cudaFree(dev);
        }
        dev = nullptr;
    }
};

uint32_t blocks_for(uint64_t n) {
    uint64_t b = (n + 255) / 256;
    if (b > 152 * 32) b = 152 * 32;
    return uint32_t(b ? b : 1);
}

// out[r][c] = in[(r + sy) mod y][(c + sx) mod x]  (a cyclic shift per axis)
template <typename E>
__global__ void k_cyclic_shift2(const E* __restrict__ in, E* __restrict__ out, uint32_t x,
                                uint32_t y, uint32_t sx, uint32_t sy) {
    const uint64_t n = uint64_t(x) * y;
    for (uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; t < n;
         t += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t r = uint32_t(t / x), c = uint32_t(t - uint64_t(r) * x);
        uint32_t rr = r + sy, cc = c + sx;
        if (rr >= y) rr -= y;
        if (cc >= x) cc -= x;
        out[t] = in[uint64_t(rr) * x + cc];
    }
}

// fftshift rotates by ceil(n/2), ifftshift by floor(n/2) (kfft_shift.c:4-61)
uint32_t shift_amount(uint32_t n, bool inverse) { return inverse ? n / 2 : n - n / 2; }

template <typename E>
void shift2(E* buf, uint32_t x, uint32_t y, bool inverse) {
    if (!ensure_device() || uint64_t(x) * y == 0) return;
    cudaStream_t st = cudaStreamPerThread;
    const size_t bytes = sizeof(E) * size_t(x) * y;
    DevView v;
    if (!v.open(buf, bytes, true, true, st)) return;
    void* tmp = nullptr;
    if (cudaMalloc(&tmp, bytes) != cudaSuccess) {
        cudaGetLastError();
        v.close(st);
        return;
    }
    k_cyclic_shift2<E><<<blocks_for(uint64_t(x) * y), 256, 0, st>>>(
        static_cast<const E*>(v.dev), static_cast<E*>(tmp), x, y, shift_amount(x, inverse),
        shift_amount(y, inverse));
    count_launch();
    cudaMemcpyAsync(v.dev, tmp, bytes, cudaMemcpyDeviceToDevice, st);
    note_cuda_error(cudaGetLastError());
    v.close(st);
    cudaStreamSynchronize(st);
    cudaFree(tmp);
}

__global__ void k_hadamard_real(real_t* __restrict__ b, const real_t* __restrict__ a, uint64_t n) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
         i += uint64_t(gridDim.x) * blockDim.x)
        b[i] *= a[i];
}

// |z| = sqrt(re^2 + im^2), the reference's kfft_math_mgnt (incs/kfft_math.h:148-151)
__global__ void k_magnitude(const vec2_t* __restrict__ in, real_t* __restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
         i += uint64_t(gridDim.x) * blockDim.x) {
        const vec2_t z = in[i];
        out[i] = sqrt(z.x * z.x + z.y * z.y);
    }
}

// per-block FP64 partial sums of a real array
__global__ void k_sum(const real_t* __restrict__ in, uint64_t n, double* __restrict__ partial) {
    __shared__ double s[256];
    double acc = 0.0;
    for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n;
         i += uint64_t(gridDim.x) * blockDim.x)
        acc += double(in[i]);
    s[threadIdx.x] = acc;
    __syncthreads();
    for (uint32_t w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

}  // namespace

extern "C" {

// ---- incs/kfft_shift.h:16-27 ----------------------------------------------
KFFT_API void kfft_shift_cpx(kfft_cpx* buf, const uint32_t size, const bool is_inverse,
                             kfft_pool_t* mmgr) {
    (void)mmgr;
    shift2<vec2_t>(reinterpret_cast<vec2_t*>(buf), size, 1, is_inverse);
}

KFFT_API void kfft_shift_scalar(kfft_scalar* buf, const uint32_t size, const bool is_inverse,
                                kfft_pool_t* mmgr) {
    (void)mmgr;
    shift2<real_t>(reinterpret_cast<real_t*>(buf), size, 1, is_inverse);
}

// ---- ext/2d/kfft_cpx2.h:19-21, ext/2d/kfft_scalar2.h:21-23 -----------------
KFFT_API void kfft_shift2_cpx(kfft_cpx* buf, kfft_cpx* ftmp, const uint32_t sz_x,
                              const uint32_t sz_y, const bool is_inverse, kfft_pool_t* mmgr) {
    (void)ftmp;
    (void)mmgr;
    shift2<vec2_t>(reinterpret_cast<vec2_t*>(buf), sz_x, sz_y, is_inverse);
}

KFFT_API void kfft_shift2_scalar(kfft_scalar* buf, kfft_scalar* ftmp, const uint32_t sz_x,
                                 const uint32_t sz_y, const bool is_inverse, kfft_pool_t* mmgr) {
    (void)ftmp;
    (void)mmgr;
    shift2<real_t>(reinterpret_cast<real_t*>(buf), sz_x, sz_y, is_inverse);
}

// ---- incs/kfft_math.h:251-350 ----------------------------------------------
KFFT_API void kfft_math_hadamard_cpx(kfft_cpx* Fout, const kfft_cpx* Fin, uint32_t size) {
    if (!ensure_device() || !size) return;
    cudaStream_t st = cudaStreamPerThread;
    DevView o, i;
    const size_t bytes = sizeof(vec2_t) * size_t(size);
    if (!o.open(Fout, bytes, true, true, st) || !i.open(Fin, bytes, true, false, st)) {
        o.close(st);
        return;
    }
    launch_hadamard(static_cast<vec2_t*>(o.dev), static_cast<const vec2_t*>(i.dev), size, st);
    i.close(st);
    o.close(st);
}

KFFT_API void kfft_math_hadamard_scalar(kfft_scalar* Fout, const kfft_scalar* Fin, uint32_t size) {
    if (!ensure_device() || !size) return;
    cudaStream_t st = cudaStreamPerThread;
    DevView o, i;
    const size_t bytes = sizeof(real_t) * size_t(size);
    if (!o.open(Fout, bytes, true, true, st) || !i.open(Fin, bytes, true, false, st)) {
        o.close(st);
        return;
    }
    k_hadamard_real<<<blocks_for(size), 256, 0, st>>>(static_cast<real_t*>(o.dev),
                                                       static_cast<const real_t*>(i.dev), size);
    count_launch();
    i.close(st);
    o.close(st);
}

// Fout (x rows of y) = transpose of Fin (y rows of x), kfft_math.c:60-78
KFFT_API void kfft_math_transpose_cpx(const kfft_cpx* Fin, kfft_cpx* Fout, const uint32_t x,
                                      const uint32_t y) {
    if (!ensure_device() || uint64_t(x) * y == 0) return;
    cudaStream_t st = cudaStreamPerThread;
    DevView o, i;
    const size_t bytes = sizeof(vec2_t) * size_t(x) * y;
    if (!i.open(Fin, bytes, true, false, st) || !o.open(Fout, bytes, false, true, st)) {
        i.close(st);
        return;
    }
    launch_transpose(static_cast<const vec2_t*>(i.dev), static_cast<vec2_t*>(o.dev), y, x, 1, st);
    i.close(st);
    o.close(st);
}

KFFT_API void kfft_math_transpose_scalar(const kfft_scalar* Fin, kfft_scalar* Fout, const uint32_t x,
                                         const uint32_t y) {
    if (!ensure_device() || uint64_t(x) * y == 0) return;
    cudaStream_t st = cudaStreamPerThread;
    DevView o, i;
    const size_t bytes = sizeof(real_t) * size_t(x) * y;
    if (!i.open(Fin, bytes, true, false, st) || !o.open(Fout, bytes, false, true, st)) {
        i.close(st);
        return;
    }
    launch_transpose_real(static_cast<const real_t*>(i.dev), static_cast<real_t*>(o.dev), y, x, st);
    i.close(st);
    o.close(st);
}

// in-place variants (kfft_math.c:80-121): same result as the out-of-place ones
KFFT_API void kfft_math_transpose_ip_cpx(kfft_cpx* Fin, const uint32_t x, const uint32_t y) {
    if (!ensure_device() || uint64_t(x) * y == 0) return;
    cudaStream_t st = cudaStreamPerThread;
    DevView v;
    const size_t bytes = sizeof(vec2_t) * size_t(x) * y;
    if (!v.open(Fin, bytes, true, true, st)) return;
    void* tmp = nullptr;
    if (cudaMalloc(&tmp, bytes) == cudaSuccess) {
        launch_transpose(static_cast<const vec2_t*>(v.dev), static_cast<vec2_t*>(tmp), y, x, 1, st);
        cudaMemcpyAsync(v.dev, tmp, bytes, cudaMemcpyDeviceToDevice, st);
        cudaStreamSynchronize(st);
        cudaFree(tmp);
    } else {
        cudaGetLastError();
    }
    v.close(st);
}

KFFT_API void kfft_math_transpose_ip_scalar(kfft_scalar* Fin, const uint32_t x, const uint32_t y) {
    if (!ensure_device() || uint64_t(x) * y == 0) return;
    cudaStream_t st = cudaStreamPerThread;
    DevView v;
    const size_t bytes = sizeof(real_t) * size_t(x) * y;
    if (!v.open(Fin, bytes, true, true, st)) return;
    void* tmp = nullptr;
    if (cudaMalloc(&tmp, bytes) == cudaSuccess) {
        launch_transpose_real(static_cast<const real_t*>(v.dev), static_cast<real_t*>(tmp), y, x, st);
        cudaMemcpyAsync(v.dev, tmp, bytes, cudaMemcpyDeviceToDevice, st);
        cudaStreamSynchronize(st);
        cudaFree(tmp);
    } else {
        cudaGetLastError();
    }
    v.close(st);
}

KFFT_API void kfft_math_magnitude(const kfft_cpx* Fin, kfft_scalar* Fout, uint32_t size) {
    if (!ensure_device() || !size) return;
    cudaStream_t st = cudaStreamPerThread;
    DevView i, o;
    if (!i.open(Fin, sizeof(vec2_t) * size_t(size), true, false, st) ||
        !o.open(Fout, sizeof(real_t) * size_t(size), false, true, st)) {
        i.close(st);
        return;
    }
    k_magnitude<<<blocks_for(size), 256, 0, st>>>(static_cast<const vec2_t*>(i.dev),
                                                   static_cast<real_t*>(o.dev), size);
    count_launch();
    i.close(st);
    o.close(st);
}

// the first `size` reals of the buffer become the magnitudes (kfft_math.c:131-137)
KFFT_API void kfft_math_magnitude_ip(kfft_cpx* Fin, uint32_t size) {
    if (!ensure_device() || !size) return;
    cudaStream_t st = cudaStreamPerThread;
    DevView v;
    if (!v.open(Fin, sizeof(vec2_t) * size_t(size), true, true, st)) return;
    void* tmp = nullptr;
    if (cudaMalloc(&tmp, sizeof(real_t) * size_t(size)) == cudaSuccess) {
        k_magnitude<<<blocks_for(size), 256, 0, st>>>(static_cast<const vec2_t*>(v.dev),
                                                       static_cast<real_t*>(tmp), size);
        count_launch();
        cudaMemcpyAsync(v.dev, tmp, sizeof(real_t) * size_t(size), cudaMemcpyDeviceToDevice, st);
        cudaStreamSynchronize(st);
        cudaFree(tmp);
    } else {
        cudaGetLastError();
    }
    v.close(st);
}

// sum / size with an FP64 tree reduction (kfft_math.c:139-148 sums in a
// racy OpenMP loop; the value it means is the mean)
KFFT_API kfft_scalar kfft_math_average(const kfft_scalar* Fin, uint32_t size) {
    if (!ensure_device() || !size) return kfft_scalar(0);
    cudaStream_t st = cudaStreamPerThread;
    DevView v;
    if (!v.open(Fin, sizeof(real_t) * size_t(size), true, false, st)) return kfft_scalar(0);
    const uint32_t nb = blocks_for(size);
    double* part = nullptr;
    double sum = 0.0;
    if (cudaMalloc(&part, sizeof(double) * nb) == cudaSuccess) {
        k_sum<<<nb, 256, 0, st>>>(static_cast<const real_t*>(v.dev), size, part);
        count_launch();
        double* h = new double[nb];
        cudaMemcpyAsync(h, part, sizeof(double) * nb, cudaMemcpyDeviceToHost, st);
        cudaStreamSynchronize(st);
        for (uint32_t b = 0; b < nb; ++b) sum += h[b];
        delete[] h;
        cudaFree(part);
    } else {
        cudaGetLastError();
    }
    v.close(st);
    return kfft_scalar(sum / double(size));
}

}  // extern "C"
