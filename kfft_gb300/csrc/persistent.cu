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
// threads per CTA of the queue kernel (its tile bodies stride over the
// CTA's threads, whatever their number).  Uneven FP32 batch: 256 threads,
// 2048-point tiles, 4 CTAs per SM 8.85 ms; 128 threads, 1024-point tiles,
// 256-point passes, 8 CTAs 9.05 ms (6 CTAs 10.17); 512 threads,
// 4096-point tiles, 2 CTAs 9.47 ms with 1024-point passes, 10.10 with 512.
#ifndef KFFT_QUEUE_THREADS
#define KFFT_QUEUE_THREADS 256
#endif
// 1: each CTA claims its items two ahead and copies the next item's record
// into shared memory while the current one runs; 0: one claim ahead, the
// record read when its turn comes (uneven FP32 batch: 8.93 against 9.13 ms;
// FP64 unchanged)
#ifndef KFFT_QUEUE_PREFETCH
#define KFFT_QUEUE_PREFETCH 1
#endif

__device__ __forceinline__ void publish_done(uint32_t* done) {
#if KFFT_QUEUE_RELEASE_ONE
    // the CTA's stores are ordered before thread 0's by the barrier, and
    // thread 0 publishes them all with one release add at GPU scope (the
    // waiting CTA's acquire load pairs with it)
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(done), "r"(1u) : "memory");
    }
#else
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(done, 1u);
#endif
}

// Thread 0's dependency wait for item q (a bounded spin that sets the error
// word instead of hanging); the result goes to every thread through *s_ok.
__device__ __forceinline__ void item_wait(const QueueItem& q, const uint32_t* done,
                                          uint32_t* error, uint32_t max_polls, uint32_t* s_ok) {
    bool ok = true;
    if (q.dep >= 0) ok = wait_for(&done[q.dep], q.need, max_polls);
    if (!ok) atomicExch(error, 1u);
    *s_ok = ok ? 1u : 0u;
}

// stage the descriptor in shared memory: one coalesced copy per item, then
// broadcast reads (measured 14% faster on the uneven batch than reading every
// field from global memory through L1)
__device__ __forceinline__ void stage_desc(const PassDesc* __restrict__ descs, uint32_t desc,
                                           PassDesc* s_desc) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&descs[desc]);
    uint32_t* dst = reinterpret_cast<uint32_t*>(s_desc);
    for (uint32_t i = threadIdx.x; i < sizeof(PassDesc) / 4; i += blockDim.x) dst[i] = src[i];
}

__device__ __forceinline__ void run_item(const PassDesc& d, const PassExtra& x, uint32_t tile,
                                         vec2_t* buf) {
    if (d.inv) tile_body_reg<true, true, false>(d, x, tile, buf);
    else tile_body_reg<false, true, false>(d, x, tile, buf);
}

__global__ void __launch_bounds__(KFFT_QUEUE_THREADS, KFFT_QUEUE_MINBLOCKS) k_persistent(
    const PassDesc* __restrict__ descs, const PassExtra* __restrict__ extras,
    const QueueItem* __restrict__ items, uint32_t nitems, uint32_t* head, uint32_t* done,
    uint32_t* error, uint32_t max_polls) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t s_ok;
    __shared__ __align__(16) PassDesc s_desc;
    vec2_t* buf = reinterpret_cast<vec2_t*>(smem_raw);
#if KFFT_QUEUE_PREFETCH
    // Items claimed two ahead, their records in a ring of three shared slots:
    // the current item, the next one (copied in during the previous item)
    // and the one after it (copied in during this item).  A CTA's claims
    // increase, so its current item is the earliest of its claims; the
    // earliest claimed and unfinished item of all then is some CTA's current
    // item, whose dependencies (earlier queue positions, all claimed) are
    // done: the queue cannot deadlock.
    constexpr uint32_t kEnd = 0xffffffffu;
    __shared__ __align__(16) QueueItem s_item[3];
    uint32_t claim = 0;  // thread 0: the queue position of the item after next
    if (threadIdx.x == 0) {
        const uint32_t a = atomicAdd(head, 1u);
        const uint32_t b = atomicAdd(head, 1u);
        s_item[0].desc = kEnd;
        s_item[1].desc = kEnd;
        if (a < nitems) s_item[0] = items[a];
        if (b < nitems) s_item[1] = items[b];
        claim = atomicAdd(head, 1u);
    }
    __syncthreads();
    uint32_t slot = 0;
    while (true) {
        const QueueItem q = s_item[slot];
        if (q.desc == kEnd) break;
        if (threadIdx.x == 0) {
            item_wait(q, done, error, max_polls, &s_ok);
            // the slot the previous item used (every thread read it before
            // the previous item's barriers) takes the record at `claim`
            const uint32_t s2 = slot == 0 ? 2u : slot - 1u;
            if (claim < nitems) {
                const uint32_t sa = uint32_t(__cvta_generic_to_shared(&s_item[s2]));
                asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(&items[claim])
                             : "memory");
            } else {
                s_item[s2].desc = kEnd;
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
            claim = atomicAdd(head, 1u);
        }
        stage_desc(descs, q.desc, &s_desc);
        __syncthreads();
        if (s_ok) run_item(s_desc, extras[q.desc], q.tile, buf);
        // the next item's record (the group before this item's) has landed
        if (threadIdx.x == 0) asm volatile("cp.async.wait_group 1;" ::: "memory");
        publish_done(&done[q.desc]);
        slot = slot == 2 ? 0u : slot + 1u;
    }
    if (threadIdx.x == 0) asm volatile("cp.async.wait_all;" ::: "memory");
#else
    __shared__ uint32_t s_next;
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
            item_wait(q, done, error, max_polls, &s_ok);
        }
        stage_desc(descs, q.desc, &s_desc);
        __syncthreads();
        if (s_ok) run_item(s_desc, extras[q.desc], q.tile, buf);
        publish_done(&done[q.desc]);
    }
#endif
}

bool launch_persistent(const PassDesc* descs, const void* extras,
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
                                                          KFFT_QUEUE_THREADS, configured_smem);
            if (blocks_per_sm < 1) blocks_per_sm = 1;
        }
        grid = uint32_t(sms * blocks_per_sm);
    }
    if (grid > nitems) grid = nitems ? nitems : 1;
    k_persistent<<<grid, KFFT_QUEUE_THREADS, smem_bytes, st>>>(
        descs, static_cast<const PassExtra*>(extras), static_cast<const QueueItem*>(items),
        nitems, head, done, error, max_polls);
    note_cuda_error(cudaGetLastError());
    count_launch();
    return true;
}

}  // namespace kfft
