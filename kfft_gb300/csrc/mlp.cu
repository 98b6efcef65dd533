// Cost model of the plan tuner: a 3-layer MLP (in -> 64 -> 64 -> 1, ReLU)
// trained on the GPU by the kernels in this file.
//
// The model ranks plan variants from features of a length (prime-factor
// exponents, largest prime, batch, precision, variant); it never touches the
// transform arithmetic.  There is no counterpart in the reference: its
// planner has a single fixed factorisation rule (kfft_generic.c:129-151).
//
// Layout of the packed FP32 parameter vector (row-major weights):
//   W1[64][in] b1[64] W2[64][64] b2[64] W3[64] b3[1]
//
// Kernels
//   k_mlp_forward  one CTA of 64 threads per row at a time; thread j owns
//                  hidden unit j of both hidden layers; parameters in smem.
//   k_mlp_grad     forward + backward over a set of rows (given by an index
//                  array), 64 rows per CTA; per-thread register accumulators
//                  for its rows of W1/W2, reduced into the global gradient
//                  with atomics at the end of the CTA's rows.  The loss is
//                  summed likewise.
//   k_mlp_adam     Adam step over the packed parameters.
// All arithmetic is FP32; the sizes are tiny (tens of thousands of rows), so
// the kernels are latency-bound and need no tensor cores.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "engine.cuh"
#include "kfft.h"

namespace {

constexpr int kH = 64;      // hidden width
constexpr int kMaxIn = 64;  // largest feature vector
constexpr int kRowsPerCta = 64;

struct Offsets {
    uint32_t w1, b1, w2, b2, w3, b3, total;
};

__host__ __device__ inline Offsets offsets(uint32_t in) {
    Offsets o;
    o.w1 = 0;
    o.b1 = o.w1 + kH * in;
    o.w2 = o.b1 + kH;
    o.b2 = o.w2 + kH * kH;
    o.w3 = o.b2 + kH;
    o.b3 = o.w3 + kH;
    o.total = o.b3 + 1;
    return o;
}

// sum over the 64 threads of the CTA (two warps); every thread gets the sum
__device__ inline float cta_sum64(float v, float* red) {
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    const int w = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[w] = v;
    __syncthreads();
    return red[0] + red[1];
}

// forward of one row: x and the parameters in smem.  Leaves h1, h2 in smem
// and returns the output on every thread.
__device__ inline float forward_row(const float* sp, const Offsets& o, uint32_t in,
                                    const float* x, float* h1, float* h2, float* red) {
    const int j = threadIdx.x;
    float a = sp[o.b1 + j];
    const float* w1 = sp + o.w1 + j * in;
    for (uint32_t i = 0; i < in; ++i) a = fmaf(w1[i], x[i], a);
    h1[j] = fmaxf(a, 0.f);
    __syncthreads();
    float b = sp[o.b2 + j];
    const float* w2 = sp + o.w2 + j * kH;
#pragma unroll 16
    for (int k = 0; k < kH; ++k) b = fmaf(w2[k], h1[k], b);
    const float r2 = fmaxf(b, 0.f);
    h2[j] = r2;
    return cta_sum64(sp[o.w3 + j] * r2, red) + sp[o.b3];
}

__global__ void __launch_bounds__(kH) k_mlp_forward(const float* __restrict__ params, uint32_t in,
                                                    const float* __restrict__ X, uint32_t n,
                                                    float* __restrict__ out) {
    extern __shared__ float sm[];
    const Offsets o = offsets(in);
    float* sp = sm;
    float* x = sp + ((o.total + 3) & ~3u);
    float* h1 = x + kMaxIn;
    float* h2 = h1 + kH;
    float* red = h2 + kH;
    for (uint32_t i = threadIdx.x; i < o.total; i += kH) sp[i] = params[i];
    __syncthreads();
    for (uint32_t r = blockIdx.x; r < n; r += gridDim.x) {
        for (uint32_t i = threadIdx.x; i < in; i += kH) x[i] = X[size_t(r) * in + i];
        __syncthreads();
        const float y = forward_row(sp, o, in, x, h1, h2, red);
        if (threadIdx.x == 0) out[r] = y;
        __syncthreads();
    }
}

// Forward + backward over rows idx[0..n) (idx may be null: rows 0..n).  The
// gradient of loss = inv_n * sum (f(x)-y)^2 is added to grad, the loss to *loss.
__global__ void __launch_bounds__(kH) k_mlp_grad(const float* __restrict__ params, uint32_t in,
                                                 const float* __restrict__ X,
                                                 const float* __restrict__ Y,
                                                 const uint32_t* __restrict__ idx, uint32_t n,
                                                 float inv_n, float* __restrict__ grad,
                                                 float* __restrict__ loss) {
    extern __shared__ float sm[];
    const Offsets o = offsets(in);
    float* sp = sm;
    float* x = sp + ((o.total + 3) & ~3u);
    float* h1 = x + kMaxIn;
    float* h2 = h1 + kH;
    float* red = h2 + kH;
    float* dh2 = red + 4;
    for (uint32_t i = threadIdx.x; i < o.total; i += kH) sp[i] = params[i];
    __syncthreads();
    const int j = threadIdx.x;
    // register accumulators: row j of W2 and of W1, unit j's biases and W3
    float gw2[kH];
#pragma unroll
    for (int k = 0; k < kH; ++k) gw2[k] = 0.f;
    float gw1[kMaxIn];
#pragma unroll
    for (int i = 0; i < kMaxIn; ++i) gw1[i] = 0.f;
    float gb1 = 0.f, gb2 = 0.f, gw3 = 0.f, gb3 = 0.f, lsum = 0.f;
    const uint32_t first = blockIdx.x * kRowsPerCta;
    const uint32_t last = min(n, first + kRowsPerCta);
    for (uint32_t t = first; t < last; ++t) {
        const uint32_t r = idx ? idx[t] : t;
        for (uint32_t i = threadIdx.x; i < in; i += kH) x[i] = X[size_t(r) * in + i];
        __syncthreads();
        const float f = forward_row(sp, o, in, x, h1, h2, red);
        const float e = f - Y[r];
        lsum += e * e;  // identical on every thread; thread 0 adds it
        const float dout = 2.f * e * inv_n;
        gw3 = fmaf(dout, h2[j], gw3);
        gb3 += dout;
        const float d2 = h2[j] > 0.f ? dout * sp[o.w3 + j] : 0.f;
        dh2[j] = d2;
        gb2 += d2;
#pragma unroll
        for (int k = 0; k < kH; ++k) gw2[k] = fmaf(d2, h1[k], gw2[k]);
        __syncthreads();
        // back to hidden layer 1: dh1[j] = sum_k dh2[k] W2[k][j]
        float d1 = 0.f;
#pragma unroll 16
        for (int k = 0; k < kH; ++k) d1 = fmaf(dh2[k], sp[o.w2 + k * kH + j], d1);
        d1 = h1[j] > 0.f ? d1 : 0.f;
        gb1 += d1;
#pragma unroll
        for (int i = 0; i < kMaxIn; ++i)
            if (uint32_t(i) < in) gw1[i] = fmaf(d1, x[i], gw1[i]);
        __syncthreads();
    }
    if (first >= last) return;
    for (int k = 0; k < kH; ++k) atomicAdd(&grad[o.w2 + j * kH + k], gw2[k]);
#pragma unroll
    for (int i = 0; i < kMaxIn; ++i)
        if (uint32_t(i) < in) atomicAdd(&grad[o.w1 + j * in + i], gw1[i]);
    atomicAdd(&grad[o.b1 + j], gb1);
    atomicAdd(&grad[o.b2 + j], gb2);
    atomicAdd(&grad[o.w3 + j], gw3);
    if (j == 0) {
        atomicAdd(&grad[o.b3], gb3);
        atomicAdd(loss, lsum * inv_n);
    }
}

__global__ void k_mlp_adam(float* __restrict__ p, const float* __restrict__ g,
                           float* __restrict__ m, float* __restrict__ v, uint32_t count,
                           float lr, float b1, float b2, float c1, float c2, float eps) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double uniform01(uint64_t& s) { return double(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace

struct kfft_mlp {
    uint32_t in = 0;
    Offsets o{};
    float* params = nullptr;  // device
    float* grad = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* loss = nullptr;
    uint64_t step = 0;
    cudaStream_t st = nullptr;
};

namespace {

size_t smem_bytes(const kfft_mlp* M) {
    return (((M->o.total + 3) & ~3u) + kMaxIn + 2 * kH + 4 + kH) * sizeof(float);
}

bool ok(cudaError_t e) {
    if (e == cudaSuccess) return true;
    kfft::note_cuda_error(e);
    return false;
}

// device copies of host rows for one call
struct DevRows {
    float* X = nullptr;
    float* Y = nullptr;
    ~DevRows() {
        cudaFree(X);
        cudaFree(Y);
    }
    bool upload(const float* hx, const float* hy, uint32_t n, uint32_t in, cudaStream_t st) {
        if (!ok(cudaMalloc(&X, size_t(n) * in * sizeof(float) + 16))) return false;
        if (!ok(cudaMemcpyAsync(X, hx, size_t(n) * in * sizeof(float), cudaMemcpyHostToDevice, st)))
            return false;
        if (hy) {
            if (!ok(cudaMalloc(&Y, size_t(n) * sizeof(float) + 16))) return false;
            if (!ok(cudaMemcpyAsync(Y, hy, size_t(n) * sizeof(float), cudaMemcpyHostToDevice, st)))
                return false;
        }
        return true;
    }
};

bool launch_grad(kfft_mlp* M, const float* X, const float* Y, const uint32_t* idx, uint32_t n,
                 float inv_n) {
    const uint32_t blocks = (n + kRowsPerCta - 1) / kRowsPerCta;
    k_mlp_grad<<<blocks, kH, smem_bytes(M), M->st>>>(M->params, M->in, X, Y, idx, n, inv_n,
                                                      M->grad, M->loss);
    return ok(cudaGetLastError());
}

}  // namespace

extern "C" {

KFFT_API kfft_mlp* kfft_mlp_create(uint32_t in_dim, uint64_t seed) {
    if (in_dim == 0 || in_dim > uint32_t(kMaxIn)) return NULL;
    if (!kfft::ensure_device()) return NULL;
    kfft_mlp* M = new (std::nothrow) kfft_mlp();
    if (!M) return NULL;
    M->in = in_dim;
    M->o = offsets(in_dim);
    const size_t bytes = size_t(M->o.total) * sizeof(float);
    bool good = ok(cudaStreamCreateWithFlags(&M->st, cudaStreamNonBlocking)) &&
                ok(cudaMalloc(&M->params, bytes)) && ok(cudaMalloc(&M->grad, bytes)) &&
                ok(cudaMalloc(&M->m, bytes)) && ok(cudaMalloc(&M->v, bytes)) &&
                ok(cudaMalloc(&M->loss, sizeof(float)));
    if (good) {
        // He-uniform weights, zero biases
        std::vector<float> p(M->o.total, 0.f);
        uint64_t s = seed;
        auto fill = [&](uint32_t off, uint32_t count, uint32_t fan_in) {
            const double a = std::sqrt(6.0 / fan_in);
            for (uint32_t i = 0; i < count; ++i) p[off + i] = float((2.0 * uniform01(s) - 1.0) * a);
        };
        fill(M->o.w1, kH * in_dim, in_dim);
        fill(M->o.w2, kH * kH, kH);
        fill(M->o.w3, kH, kH);
        good = ok(cudaMemcpy(M->params, p.data(), bytes, cudaMemcpyHostToDevice)) &&
               ok(cudaMemset(M->m, 0, bytes)) && ok(cudaMemset(M->v, 0, bytes));
    }
    if (!good) {
        kfft_mlp_release(M);
        return NULL;
    }
    return M;
}

KFFT_API void kfft_mlp_release(kfft_mlp* M) {
    if (!M) return;
    cudaFree(M->params);
    cudaFree(M->grad);
    cudaFree(M->m);
    cudaFree(M->v);
    cudaFree(M->loss);
    if (M->st) cudaStreamDestroy(M->st);
    delete M;
}

KFFT_API uint32_t kfft_mlp_params(const kfft_mlp* M) { return M ? M->o.total : 0; }

KFFT_API kfft_return_t kfft_mlp_get(const kfft_mlp* M, float* params) {
    if (!M || !params) return KFFT_RET_BADARGUMENTS;
    return ok(cudaMemcpy(params, M->params, size_t(M->o.total) * sizeof(float),
                         cudaMemcpyDeviceToHost))
               ? KFFT_RET_SUCCESS
               : KFFT_RET_ALLOC_FAIL;
}

KFFT_API kfft_return_t kfft_mlp_set(kfft_mlp* M, const float* params) {
    if (!M || !params) return KFFT_RET_BADARGUMENTS;
    const size_t bytes = size_t(M->o.total) * sizeof(float);
    const bool good = ok(cudaMemcpy(M->params, params, bytes, cudaMemcpyHostToDevice)) &&
                      ok(cudaMemset(M->m, 0, bytes)) && ok(cudaMemset(M->v, 0, bytes));
    M->step = 0;
    return good ? KFFT_RET_SUCCESS : KFFT_RET_ALLOC_FAIL;
}

KFFT_API kfft_return_t kfft_mlp_predict(kfft_mlp* M, const float* X, uint32_t n, float* out) {
    if (!M || (n && (!X || !out))) return KFFT_RET_BADARGUMENTS;
    if (n == 0) return KFFT_RET_SUCCESS;
    DevRows d;
    float* dout = nullptr;
    if (!d.upload(X, nullptr, n, M->in, M->st)) return KFFT_RET_ALLOC_FAIL;
    if (!ok(cudaMalloc(&dout, size_t(n) * sizeof(float)))) return KFFT_RET_ALLOC_FAIL;
    const uint32_t blocks = std::min<uint32_t>(n, 152 * 8);
    k_mlp_forward<<<blocks, kH, smem_bytes(M), M->st>>>(M->params, M->in, d.X, n, dout);
    const bool good = ok(cudaGetLastError()) &&
                      ok(cudaMemcpyAsync(out, dout, size_t(n) * sizeof(float),
                                         cudaMemcpyDeviceToHost, M->st)) &&
                      ok(cudaStreamSynchronize(M->st));
    cudaFree(dout);
    return good ? KFFT_RET_SUCCESS : KFFT_RET_ALLOC_FAIL;
}

KFFT_API kfft_return_t kfft_mlp_loss_grad(kfft_mlp* M, const float* X, const float* y,
                                          uint32_t n, float* loss, float* grad) {
    if (!M || !X || !y || n == 0) return KFFT_RET_BADARGUMENTS;
    DevRows d;
    if (!d.upload(X, y, n, M->in, M->st)) return KFFT_RET_ALLOC_FAIL;
    const size_t bytes = size_t(M->o.total) * sizeof(float);
    bool good = ok(cudaMemsetAsync(M->grad, 0, bytes, M->st)) &&
                ok(cudaMemsetAsync(M->loss, 0, sizeof(float), M->st)) &&
                launch_grad(M, d.X, d.Y, nullptr, n, 1.f / float(n));
    float l = 0.f;
    if (good && grad)
        good = ok(cudaMemcpyAsync(grad, M->grad, bytes, cudaMemcpyDeviceToHost, M->st));
    if (good) good = ok(cudaMemcpyAsync(&l, M->loss, sizeof(float), cudaMemcpyDeviceToHost, M->st));
    if (good) good = ok(cudaStreamSynchronize(M->st));
    if (good && loss) *loss = l;
    return good ? KFFT_RET_SUCCESS : KFFT_RET_ALLOC_FAIL;
}

KFFT_API kfft_return_t kfft_mlp_train(kfft_mlp* M, const float* X, const float* y, uint32_t n,
                                      uint32_t epochs, uint32_t minibatch, float lr,
                                      uint64_t seed, float* loss) {
    if (!M || !X || !y || n == 0 || minibatch == 0) return KFFT_RET_BADARGUMENTS;
    DevRows d;
    if (!d.upload(X, y, n, M->in, M->st)) return KFFT_RET_ALLOC_FAIL;
    uint32_t* didx = nullptr;
    if (!ok(cudaMalloc(&didx, size_t(n) * sizeof(uint32_t)))) return KFFT_RET_ALLOC_FAIL;
    std::vector<uint32_t> perm(n);
    for (uint32_t i = 0; i < n; ++i) perm[i] = i;
    uint64_t s = seed;
    const size_t bytes = size_t(M->o.total) * sizeof(float);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    bool good = true;
    for (uint32_t ep = 0; good && ep < epochs; ++ep) {
        // the previous epoch's copy of perm must be done before perm changes
        good = ok(cudaStreamSynchronize(M->st));
        for (uint32_t i = n - 1; good && i > 0; --i)
            std::swap(perm[i], perm[splitmix(s) % (i + 1)]);
        good = good && ok(cudaMemcpyAsync(didx, perm.data(), size_t(n) * sizeof(uint32_t),
                                          cudaMemcpyHostToDevice, M->st));
        for (uint32_t b0 = 0; good && b0 < n; b0 += minibatch) {
            const uint32_t nb = std::min(minibatch, n - b0);
            M->step++;
            const float c1 = 1.f - std::pow(b1, float(M->step));
            const float c2 = 1.f - std::pow(b2, float(M->step));
            good = ok(cudaMemsetAsync(M->grad, 0, bytes, M->st)) &&
                   launch_grad(M, d.X, d.Y, didx + b0, nb, 1.f / float(nb));
            if (!good) break;
            k_mlp_adam<<<(M->o.total + 255) / 256, 256, 0, M->st>>>(
                M->params, M->grad, M->m, M->v, M->o.total, lr, b1, b2, c1, c2, eps);
            good = ok(cudaGetLastError());
        }
    }
    if (good) good = ok(cudaStreamSynchronize(M->st));
    cudaFree(didx);
    if (!good) return KFFT_RET_ALLOC_FAIL;
    if (loss) return kfft_mlp_loss_grad(M, X, y, n, loss, nullptr);
    return KFFT_RET_SUCCESS;
}

}  // extern "C"
