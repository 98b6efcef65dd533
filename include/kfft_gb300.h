/*
 * kfft_gb300.h -- additive entry points of the GB300 FFT engine.
 *
 * The reference LibKFFT has no batch API: its callers loop over sequences on
 * the host (ext/2d/kfft_cpx2.c:100-104 is the pattern).  These entry points
 * are new symbols only; no reference signature changes.  They let a caller
 * hand many sequences to the GPU in one call, pass device pointers and a CUDA
 * stream, and run a whole batch of uneven lengths as one graph launch.
 */
#pragma once

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/*
 * Plan flag (additive, above the reference's bits 0-5): in the float build,
 * run the radix-16 stages of direct plans as FP16 split hi+lo matrix products
 * on tensor cores with FP32 accumulation.  Ignored by the double build.
 */
#define KFFT_FLAG_TENSOR_CORES (1u << 8)

/*
 * Batched complex transform: `batch` sequences of plan->nfft points stored back
 * to back.  fin/fout may be host or device memory (fin == fout allowed).
 * Synchronous, like kfft_eval_cpx.  Same return codes as kfft_eval_cpx.
 */
KFFT_API kfft_return_t kfft_eval_cpx_batch(kfft_plan_cpx* plan, const kfft_cpx* fin,
                                           kfft_cpx* fout, uint32_t batch);

/*
 * Asynchronous batched complex transform on `stream` (a cudaStream_t, NULL =
 * the legacy default stream).  fin/fout must be device memory.  Returns after
 * the kernels are queued.  Calls sharing a plan must be ordered on one stream.
 */
KFFT_API kfft_return_t kfft_eval_cpx_async(kfft_plan_cpx* plan, const kfft_cpx* fin,
                                           kfft_cpx* fout, uint32_t batch, void* stream);

/* Batched real transforms; the spectrum of sequence b starts at b * nbins,
 * nbins = N/2+1 for even N without KFFT_FLAG_EXPAND_SCALAR, else N. */
KFFT_API kfft_return_t kfft_eval_scalar_batch(kfft_plan_sclr* plan, const kfft_scalar* fin,
                                              kfft_cpx* fout, uint32_t batch);
KFFT_API kfft_return_t kfft_evali_scalar_batch(kfft_plan_sclr* plan, const kfft_cpx* fin,
                                               kfft_scalar* fout, uint32_t batch);

/*
 * Uneven-length batch: `count` complex sequences with lengths[i] points each,
 * packed back to back (sequence i starts at the sum of the previous lengths).
 * The plan groups equal lengths, builds one device plan per distinct length
 * and records the whole batch into a CUDA graph that kfft_eval_cpx_uneven
 * launches once per call.
 */
typedef struct kfft_plan_uneven kfft_plan_uneven;

KFFT_API kfft_plan_uneven* kfft_config_cpx_uneven(uint32_t count, const uint32_t* lengths,
                                                  uint32_t flags);
/* Host or device buffers of kfft_uneven_total(plan) points each; synchronous. */
KFFT_API kfft_return_t kfft_eval_cpx_uneven(kfft_plan_uneven* plan, const kfft_cpx* fin,
                                            kfft_cpx* fout);
/* Device buffers only; queued on `stream` (cudaStream_t). */
KFFT_API kfft_return_t kfft_eval_cpx_uneven_async(kfft_plan_uneven* plan, const kfft_cpx* fin,
                                                  kfft_cpx* fout, void* stream);
KFFT_API uint64_t kfft_uneven_total(const kfft_plan_uneven* plan);
KFFT_API void kfft_release_uneven(kfft_plan_uneven* plan);

/*
 * Complex transform that allocates nothing.  No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc (code inside a CUDA graph
 * capture or another library's stream-ordered region, real-time loops that
 * forbid allocator calls and the synchronisation cudaFree implies, or a host
 * whose framework must own every allocation).  fin/fout are device buffers of
 * `batch` back-to-back sequences; the work is queued on `stream` (a
 * cudaStream_t) and the call returns without waiting.  The plan must be a
 * direct mixed-radix plan (every prime factor of nfft <= 31).  Scratch between
 * passes lives in one file-scope device array of kfft_noalloc_scratch_bytes()
 * bytes (32 MiB) that every GPU loading this library holds until the process
 * exits; requests that need more return KFFT_RET_BADARGUMENTS and
 * kfft_noalloc_last_message() says why.  The first call on each device looks
 * up the array's device address and should be made before any stream capture.
 * All calls share the array: calls whose kernels overlap on the GPU race.
 */
KFFT_API kfft_return_t kfft_eval_cpx_noalloc(kfft_plan_cpx* plan, const kfft_cpx* fin,
                                             kfft_cpx* fout, uint32_t batch, void* stream);
KFFT_API size_t kfft_noalloc_scratch_bytes(void);
KFFT_API const char* kfft_noalloc_last_message(void);

/* Engine introspection (used by tests and the benchmark). */
typedef struct {
    uint64_t kernel_launches; /* kernels this library launched since load */
    uint64_t graph_launches;  /* CUDA graphs it launched */
    uint64_t device_bytes;    /* bytes of device memory it currently holds */
    int32_t device;           /* CUDA device ordinal in use, -1 if none */
    int32_t last_cuda_error;  /* last CUDA error seen (cudaError_t), 0 if none */
} kfft_gb300_stats_t;

KFFT_API void kfft_gb300_stats(kfft_gb300_stats_t* stats);
/* Human-readable description of the last CUDA error, "" if none. */
KFFT_API const char* kfft_gb300_last_error(void);
/* Passes of a plan as text ("R=64 Ns=1 radices=16,4 | ..."), for diagnostics. */
KFFT_API const char* kfft_gb300_describe(const kfft_plan_cpx* plan);

#ifdef __cplusplus
}
#endif
