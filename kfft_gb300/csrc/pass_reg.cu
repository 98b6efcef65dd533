// pass_reg.cu -- the register-resident pass kernel k_pass_reg.
#include "fft_device.cuh"

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <utility>

namespace kfft {

template <bool INV>
__global__ void __launch_bounds__(kPassThreads, KFFT_REG_MINBLOCKS) k_pass_reg(const __grid_constant__ PassDesc d,
                                                              const __grid_constant__ PassExtra x) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // power-of-two FP32 passes launch k_pass_spec / k_pass_pipe instead
    tile_body_reg<INV, false>(d, x, blockIdx.x, reinterpret_cast<vec2_t*>(smem_raw));
}

#if defined(KFFT_HALF_SCALAR)
// FP32 power-of-two passes, one kernel per pass length R so each kernel holds
// only its own body (a small instruction footprint):
// * k_pass_pipe: a plain prologue and more tiles than fit the GPU at once: a
//   grid of resident CTAs, each running many tiles with its next tile's loads
//   in flight (tile_loop_pipelined);
// * k_pass_spec: one tile per CTA otherwise.
// The FP64 build uses neither: the FP64 pipe, not index arithmetic or load
// latency, bounds that path, and its unrolled bodies would spill.
template <uint32_t R, bool INV>
__global__ void __launch_bounds__(kPassThreads, 2) k_pass_pipe(const __grid_constant__ PassDesc d) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    tile_loop_pipelined<R, INV>(d, reinterpret_cast<vec2_t*>(smem_raw));
}

// k_pass_pipe with twice the threads and twice the lanes per tile (8192
// points): multi-lane passes of 512 or 1024 points, whose 4096-point tiles
// hold only 8 or 4 lanes (64- or 32-byte row segments), read and write twice
// as wide segments.  One CTA per SM.  (256-point passes, whose 4096-point
// tiles already hold 16 lanes, measured slower on it.)
template <uint32_t R, bool INV>
__global__ void __launch_bounds__(2 * kPassThreads, 1) k_pass_pipe_wide(const __grid_constant__ PassDesc d) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    tile_loop_pipelined<R, INV>(d, reinterpret_cast<vec2_t*>(smem_raw));
}

template <uint32_t R, bool INV>
__global__ void __launch_bounds__(kPassThreads, KFFT_REG_MINBLOCKS) k_pass_spec(
    const __grid_constant__ PassDesc d) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    vec2_t* sm = reinterpret_cast<vec2_t*>(smem_raw);
    tile_body_spec<R, INV>(d, blockIdx.x * d.C, d.batch * d.lanes_j, sm, sm + d.C * d.lane_stride + 1);
}

// Set when a bulk-copy wait of k_pass_bulk ran out (only a failed or very
// slow copy can cause it); the CTA then ends without finishing its tiles.
// One word per host-thread slot: a launch passes its thread's slot, and the
// thread's next synchronous completion (take_wait_failures) reads and clears
// it, so the failure becomes that call's return code.
__device__ uint32_t g_bulk_wait_failed[kWaitSlots];

// Single-pass FP32 power-of-two batches of contiguous sequences: each tile's
// points arrive by one bulk copy (tile_loop_bulk).
template <uint32_t R, bool INV>
__global__ void __launch_bounds__(kPassThreads, 2) k_pass_bulk(const __grid_constant__ PassDesc d,
                                                               uint32_t slot, uint32_t max_polls) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    tile_loop_bulk<R, INV>(d, smem_raw, &g_bulk_wait_failed[slot], max_polls);
}

using SpecKernel = void (*)(PassDesc);
using BulkKernel = void (*)(PassDesc, uint32_t, uint32_t);

// shortest pass that runs on the wide tiles
#ifndef KFFT_WIDE_MIN_R
#define KFFT_WIDE_MIN_R 512
#endif

enum SpecKind { SPEC_ONE_TILE = 0, SPEC_PIPE = 1, SPEC_WIDE = 3 };

template <uint32_t R>
SpecKernel pick(int kind, bool inv) {
    if constexpr (R >= 256 && R <= 1024) {
        if (kind == SPEC_WIDE) return inv ? k_pass_pipe_wide<R, true> : k_pass_pipe_wide<R, false>;
    } else {
        if (kind == SPEC_WIDE) return nullptr;
    }
    if (kind == SPEC_PIPE) return inv ? k_pass_pipe<R, true> : k_pass_pipe<R, false>;
    return inv ? k_pass_spec<R, true> : k_pass_spec<R, false>;
}

template <uint32_t R>
BulkKernel pick_bulk(bool inv) {
    return inv ? k_pass_bulk<R, true> : k_pass_bulk<R, false>;
}

BulkKernel bulk_kernel(uint32_t spec, bool inv) {
    switch (spec) {
        case 4: return pick_bulk<16>(inv);
        case 5: return pick_bulk<32>(inv);
        case 6: return pick_bulk<64>(inv);
        case 7: return pick_bulk<128>(inv);
        case 8: return pick_bulk<256>(inv);
        case 9: return pick_bulk<512>(inv);
        case 10: return pick_bulk<1024>(inv);
        case 11: return pick_bulk<2048>(inv);
        case 12: return pick_bulk<4096>(inv);
        default: return nullptr;
    }
}

SpecKernel spec_kernel(uint32_t spec, int kind, bool inv) {
    switch (spec) {
        case 4: return pick<16>(kind, inv);
        case 5: return pick<32>(kind, inv);
        case 6: return pick<64>(kind, inv);
        case 7: return pick<128>(kind, inv);
        case 8: return pick<256>(kind, inv);
        case 9: return pick<512>(kind, inv);
        case 10: return pick<1024>(kind, inv);
        case 11: return pick<2048>(kind, inv);
        case 12: return pick<4096>(kind, inv);
        default: return nullptr;
    }
}
#endif

namespace {
std::atomic<uint32_t> g_bulk_polls{kBulkMaxPolls};
std::atomic<int> g_slot_next{0};
thread_local bool t_bulk_launched = false;

#if defined(KFFT_HALF_SCALAR)
uint32_t bulk_wait_polls() { return g_bulk_polls.load(std::memory_order_relaxed); }
void note_bulk_launch() { t_bulk_launched = true; }

// Raises the dynamic shared-memory limit of a kernel once and caches its
// resident CTAs per SM for a shared-memory size (thread-safe).
int prepare(const void* f, uint32_t smem, uint32_t threads = kPassThreads) {
    static std::mutex mu;
    static std::map<std::pair<const void*, uint64_t>, int> cache;
    static std::map<const void*, bool> configured;
    std::lock_guard<std::mutex> lk(mu);
    if (!configured[f]) {
        if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
            cudaSuccess) {
            cudaGetLastError();
            return -1;
        }
        configured[f] = true;
    }
    auto key = std::make_pair(f, (uint64_t(threads) << 32) | smem);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, f, int(threads), smem) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    cache[key] = n;
    return n;
}

int sm_count() {
    static const int n = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 1;
    }();
    return n;
}
#endif
}  // namespace

int wait_slot() {
    thread_local const int slot = g_slot_next.fetch_add(1) % kWaitSlots;
    return slot;
}

bool take_wait_failures(cudaStream_t st) {
#if defined(KFFT_HALF_SCALAR)
    if (!t_bulk_launched) return false;
    t_bulk_launched = false;
    static const uint32_t zero = 0;
    const size_t off = sizeof(uint32_t) * size_t(wait_slot());
    uint32_t v = 0;
    cudaMemcpyFromSymbolAsync(&v, g_bulk_wait_failed, sizeof(v), off, cudaMemcpyDeviceToHost, st);
    cudaMemcpyToSymbolAsync(g_bulk_wait_failed, &zero, sizeof(zero), off, cudaMemcpyHostToDevice,
                            st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        note_cuda_error(e);
        return true;
    }
    return v != 0;
#else
    (void)st;
    return false;
#endif
}

void launch_pass_reg(const PassDesc& d, const PassExtra& x, cudaStream_t st) {
    // one-time shared-memory limit of the generic kernels (thread-safe; a
    // failure is reported on every call)
    static const cudaError_t configured = [] {
        for (const void* f : {(const void*)k_pass_reg<false>, (const void*)k_pass_reg<true>}) {
            cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 227 * 1024);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return e;
            }
        }
        return cudaSuccess;
    }();
    if (configured != cudaSuccess) {
        note_cuda_error(configured);
        return;
    }
#if defined(KFFT_HALF_SCALAR)
    if (d.spec && d.threads == kPassThreads) {
        const bool inv = d.inv != 0;
        // one pass over whole contiguous sequences, 16-byte aligned: the
        // tiles arrive by bulk copy
        const bool contiguous = d.lanes_j == 1 && d.order == ORDER_J && d.in_es == 1 &&
                                d.in_bs == d.R && (reinterpret_cast<uintptr_t>(d.in) & 15u) == 0;
        if (d.pro_op == PRO_NONE && contiguous) {
            BulkKernel f = bulk_kernel(d.spec, inv);
            const uint32_t smem = 128 + d.C * d.R * uint32_t(sizeof(vec2_t)) + d.smem_bytes;
            const int per_sm = f ? prepare((const void*)f, smem) : -1;
            const uint32_t grid = uint32_t(std::max(per_sm, 0)) * uint32_t(sm_count());
            if (per_sm > 0 && d.tiles >= 2 * grid) {
                f<<<grid, kPassThreads, smem, st>>>(d, uint32_t(wait_slot()), bulk_wait_polls());
                note_cuda_error(cudaGetLastError());
                note_bulk_launch();
                count_launch();
                return;
            }
        }
        // multi-lane rows of 256-1024 points with a full 4096-point tile:
        // the same pass on 8192-point tiles of twice the lanes
        if (d.pro_op == PRO_NONE && d.order == ORDER_J && d.R >= KFFT_WIDE_MIN_R && d.R <= 1024 &&
            d.C * d.R == kRegTile && d.lanes_j >= 2 * d.C) {
            SpecKernel f = spec_kernel(d.spec, SPEC_WIDE, inv);
            PassDesc w = d;
            w.C = 2 * d.C;
            w.div_C.init(w.C);
            w.tiles = uint32_t((uint64_t(d.batch) * d.lanes_j + w.C - 1) / w.C);
            w.threads = 2 * kPassThreads;
            w.lane_stride = spec_lane_stride(d.R, w.C, d.load_mode == MODE_LANE,
                                             d.store_mode == MODE_LANE, w.threads);
            const uint32_t nbuf = d.R == 256 ? 1u : 2u;  // stages 16,16 or 16,16,T
            w.smem_bytes = nbuf * (w.C * w.lane_stride + 1u) * uint32_t(sizeof(vec2_t));
            const int per_sm = f ? prepare((const void*)f, w.smem_bytes, w.threads) : -1;
            const uint32_t grid = uint32_t(std::max(per_sm, 0)) * uint32_t(sm_count());
            if (per_sm > 0 && w.tiles >= 2 * grid) {
                f<<<grid, w.threads, w.smem_bytes, st>>>(w);
                note_cuda_error(cudaGetLastError());
                count_launch();
                return;
            }
        }
        if (d.pro_op == PRO_NONE) {
            SpecKernel f = spec_kernel(d.spec, SPEC_PIPE, inv);
            const int per_sm = f ? prepare((const void*)f, d.smem_bytes) : -1;
            const uint32_t grid = uint32_t(std::max(per_sm, 0)) * uint32_t(sm_count());
            if (per_sm > 0 && d.tiles >= 2 * grid) {
                f<<<grid, kPassThreads, d.smem_bytes, st>>>(d);
                note_cuda_error(cudaGetLastError());
                count_launch();
                return;
            }
        }
        SpecKernel f = spec_kernel(d.spec, SPEC_ONE_TILE, inv);
        if (f && prepare((const void*)f, d.smem_bytes) > 0) {
            f<<<d.tiles, kPassThreads, d.smem_bytes, st>>>(d);
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

extern "C" {
// Test hook: polls a bulk-copy wait makes before it gives up (0 restores the
// default of about a second).  Only a test that checks the failure path
// lowers it; see kfft_gb300.h.
KFFT_API void kfft_gb300_set_bulk_wait_polls(uint32_t polls) {
    kfft::g_bulk_polls.store(polls ? polls : kfft::kBulkMaxPolls);
}

// Synchronises `stream` and reports whether a bounded device wait of this
// thread's earlier asynchronous calls ran out (and clears the record).
KFFT_API int kfft_gb300_check_waits(void* stream) {
    const cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        kfft::note_cuda_error(e);
        return -1;
    }
    return kfft::take_wait_failures(static_cast<cudaStream_t>(stream)) ? 1 : 0;
}
}  // extern "C"
