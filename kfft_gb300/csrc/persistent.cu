// persistent.cu -- the persistent work-queue kernel: one launch drains a
// queue of (pass, tile) items ordered by dependency level, with bounded waits
// on per-pass tile counters (a wait that gives up sets an error word).
#include "fft_device.cuh"

#include <mutex>

namespace kfft {

// 1: publish a finished item with one release add by thread 0 after the
// CTA's barrier; 0: every thread fences before the barrier and thread 0 adds
// (uneven FP32 batch: 9.10 against 9.38 ms; FP64 unchanged)
#ifndef KFFT_QUEUE_RELEASE_ONE
#define KFFT_QUEUE_RELEASE_ONE 1
#endif
// resident CTAs per SM of the queue kernel (its tiles are capped at 2048
// points): four for FP32 (64 registers a thread), three for FP64 (80
// registers and about 2 KB of spills a thread, yet 84.1 against 87.7 ms for
// two on the FP64 uneven batch)
#ifndef KFFT_QUEUE_MINBLOCKS
#if defined(KFFT_HALF_SCALAR)
#define KFFT_QUEUE_MINBLOCKS 4
#else
#define KFFT_QUEUE_MINBLOCKS 3
#endif
#endif
__global__ void __launch_bounds__(kPassThreads, KFFT_QUEUE_MINBLOCKS) k_persistent(
    const PassDesc* __restrict__ descs, const PassExtra* __restrict__ extras,
    const int32_t* __restrict__ deps, const QueueItem* __restrict__ items, uint32_t nitems,
    uint32_t* head, uint32_t* done, uint32_t* error, uint32_t max_polls) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t s_next;
    __shared__ uint32_t s_ok;
    __shared__ __align__(16) PassDesc s_desc;
    vec2_t* buf = reinterpret_cast<vec2_t*>(smem_raw);
    // Each CTA claims its next item while the current one runs, so the
    // claim's round trip to L2 overlaps work.  This cannot deadlock: the item
    // of least queue position among those claimed and not finished has every
    // dependency (an earlier position) done or in a run of its own.
    if (threadIdx.x == 0) s_next = atomicAdd(head, 1u);
    __syncthreads();
    while (true) {
        const uint32_t it = s_next;
        __syncthreads();  // every thread has read s_next before it changes
        if (it >= nitems) return;
        const QueueItem q = items[it];
        if (threadIdx.x == 0) {
            s_next = atomicAdd(head, 1u);
            bool ok = true;
            const int32_t dep = deps[q.desc];
            if (dep >= 0) ok = wait_for(&done[dep], descs[dep].tiles, max_polls);
            if (!ok) atomicExch(error, 1u);
            s_ok = ok ? 1u : 0u;
        }
        // stage the descriptor in shared memory: one coalesced copy per item,
        // then broadcast reads (measured 14% faster on the uneven batch than
        // reading every field from global memory through L1)
        {
            const uint32_t* src = reinterpret_cast<const uint32_t*>(&descs[q.desc]);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&s_desc);
            for (uint32_t i = threadIdx.x; i < sizeof(PassDesc) / 4; i += blockDim.x) dst[i] = src[i];
        }
        __syncthreads();
        if (s_ok) {
            const PassExtra& x = extras[q.desc];
            if (s_desc.inv) tile_body_reg<true, true, false>(s_desc, x, q.tile, buf);
            else tile_body_reg<false, true, false>(s_desc, x, q.tile, buf);
        }
#if KFFT_QUEUE_RELEASE_ONE
        // the CTA's stores are ordered before thread 0's by the barrier, and
        // thread 0 publishes them all with one release add at GPU scope (the
        // waiting CTA's acquire load pairs with it)
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(&done[q.desc]), "r"(1u)
                         : "memory");
        }
#else
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) atomicAdd(&done[q.desc], 1u);
#endif
    }
}

bool launch_persistent(const PassDesc* descs, const void* extras, const int32_t* deps,
                       const void* items, uint32_t nitems, uint32_t* head, uint32_t* done,
                       uint32_t* error, uint32_t smem_bytes, cudaStream_t st,
                       uint32_t max_polls) {
    // the kernel's shared-memory limit and occupancy, set up under a lock (several
    // host threads may record queues at once)
    static std::mutex mu;
    static int blocks_per_sm = -1;
    static uint32_t configured_smem = 0;
    static int sms = 0;
    uint32_t grid;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (configured_smem < smem_bytes) {
            cudaError_t e = cudaFuncSetAttribute(
                k_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_bytes));
            if (e != cudaSuccess) {
                note_cuda_error(e);
                return false;
            }
            configured_smem = smem_bytes;
            blocks_per_sm = -1;
        }
        if (blocks_per_sm < 0) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_persistent,
                                                          kPassThreads, configured_smem);
            if (blocks_per_sm < 1) blocks_per_sm = 1;
        }
        grid = uint32_t(sms * blocks_per_sm);
    }
    if (grid > nitems) grid = nitems ? nitems : 1;
    k_persistent<<<grid, kPassThreads, smem_bytes, st>>>(
        descs, static_cast<const PassExtra*>(extras), deps, static_cast<const QueueItem*>(items),
        nitems, head, done, error, max_polls);
    note_cuda_error(cudaGetLastError());
    count_launch();
    return true;
}

}  // namespace kfft
