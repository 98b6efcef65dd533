// noalloc.cu -- a complex-transform entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc at the point where they transform: code
// running inside a CUDA graph capture or another library's stream-ordered
// region, real-time loops that forbid allocator calls (and the device-wide
// synchronisation cudaFree implies), and hosts whose allocator is owned by a
// framework that must see every allocation.  kfft_eval_cpx_noalloc serves
// them: it runs the multi-pass Stockham transform of a DIRECT plan (every
// prime factor <= 31) with its pass-to-pass scratch in a fixed, file-scope
// device array instead of a workspace from cudaMalloc, and it builds its pass
// descriptors in a fixed array on the host stack.
//
// The array holds kNoAllocScratchBytes (32 MiB) on every GPU that loads this
// library, for the life of the process.  Its device address is looked up once
// per device, on the first call made with that device current; that first call
// should come before any stream capture.  The first call with a given plan and
// batch may also do one-time set-up of the pass kernels it picks (their
// shared-memory limit and occupancy query, and the lazy load of their module),
// so run every (plan, batch) shape once before a region that must not do
// that.  All calls share the array and it
// keeps the last call's contents; nothing in it has to start at zero, because
// every pass writes its whole output before the next pass reads it.  Calls
// whose kernels overlap on the GPU (different streams, or different host
// threads without ordering) race on the array.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <mutex>

#include "engine.cuh"
#include "kfft.h"

using namespace kfft;

namespace {
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
constexpr int kMaxDevices = 64;
constexpr size_t kMaxPasses = 16;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};
// why this thread's last call was rejected ("" after a call that was not)
thread_local char g_noalloc_msg[256] = "";

// Device address of the scratch array on the current device (set-up on first use).
void* scratch_address(int dev) {
    if (dev < 0 || dev >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) {
            note_cuda_error(e);
            snprintf(g_noalloc_msg, sizeof(g_noalloc_msg), "cudaGetSymbolAddress failed: %s",
                     cudaGetErrorString(e));
            return nullptr;
        }
        g_scratch_addr[dev] = ptr;
    }
    return g_scratch_addr[dev];
}

bool device_pointer(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}
}  // namespace

extern "C" {

KFFT_API size_t kfft_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

KFFT_API const char* kfft_noalloc_last_message(void) { return g_noalloc_msg; }

KFFT_API kfft_return_t kfft_eval_cpx_noalloc(kfft_plan_cpx* plan, const kfft_cpx* fin,
                                             kfft_cpx* fout, uint32_t batch, void* stream) {
    g_noalloc_msg[0] = '\0';
    if (!plan || !fin || !fout) return KFFT_RET_BADARGUMENTS;
    if (plan->nfft == 0 || batch == 0) return KFFT_RET_SUCCESS;
    const FftPlan* fp = device_plan_of(plan);
    if (!fp) return KFFT_RET_IMPROPER_PLAN;
    const FftPlan& P = *fp;
    if (P.method != METHOD_DIRECT) {
        snprintf(g_noalloc_msg, sizeof(g_noalloc_msg),
                 "length %u has a prime factor above %u; only direct mixed-radix plans run "
                 "without allocation", P.N, kMaxDirectPrime);
        return KFFT_RET_BADARGUMENTS;
    }
    if (!device_pointer(fin) || !device_pointer(fout)) {
        snprintf(g_noalloc_msg, sizeof(g_noalloc_msg), "fin and fout must be device memory");
        return KFFT_RET_BADARGUMENTS;
    }
    const size_t m = P.passes.size();
    const size_t elems = size_t(P.N) * batch;
    const size_t per = (sizeof(vec2_t) * elems + 255) & ~size_t(255);
    const size_t need = m >= 3 ? 2 * per : (m == 2 ? per : 0);
    if (need > kNoAllocScratchBytes || m > kMaxPasses ||
        uint64_t(batch) * P.N >= (uint64_t(1) << 32)) {
        snprintf(g_noalloc_msg, sizeof(g_noalloc_msg),
                 "N=%u batch=%u needs %zu bytes of scratch; the no-allocation entry point has %zu",
                 P.N, batch, need, kNoAllocScratchBytes);
        return KFFT_RET_BADARGUMENTS;
    }
    cudaSetDevice(current_device());
    char* scratch = static_cast<char*>(need ? scratch_address(current_device()) : nullptr);
    if (need && !scratch) return KFFT_RET_BUFFER_FAIL;
    vec2_t* s1 = reinterpret_cast<vec2_t*>(scratch);
    vec2_t* s2 = reinterpret_cast<vec2_t*>(scratch + per);

    const real_t scale = ((plan->flags & KFFT_FLAG_INVERSE) && !(plan->flags & KFFT_FLAG_DISABLE_NORM))
                             ? real_t(1.0 / double(P.N))
                             : real_t(1);
    Layout l;
    l.batch = batch;
    l.bs = P.N;
    PassDesc descs[kMaxPasses];
    const vec2_t* cur = reinterpret_cast<const vec2_t*>(fin);
    for (size_t i = 0; i < m; ++i) {
        const bool last = (i + 1 == m);
        vec2_t* dst = last ? reinterpret_cast<vec2_t*>(fout) : ((i % 2 == 0) ? s1 : s2);
        descs[i] = make_pass_desc(P, i, cur, l, dst, l, last ? scale : real_t(1));
        cur = dst;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (size_t i = 0; i < m; ++i) launch_pass(descs[i], st);
    return take_pending_error() ? KFFT_RET_BUFFER_FAIL : KFFT_RET_SUCCESS;
}

}  // extern "C"
