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
 * kfft_noalloc_last_message() says why (per host thread; "" after a call that
 * was not rejected).  The first call on each device looks up the array's
 * device address and should be made before any stream capture; the first call
 * with each (plan, batch) shape may also set up the pass kernels it picks
 * (shared-memory limit, occupancy query, lazy module load), so run every shape
 * once before a region that must not do that.  All calls share the array:
 * calls whose kernels overlap on the GPU race.  A bounded bulk-copy wait that
 * runs out during this asynchronous call is reported by
 * kfft_gb300_check_waits(stream).
 */
KFFT_API kfft_return_t kfft_eval_cpx_noalloc(kfft_plan_cpx* plan, const kfft_cpx* fin,
                                             kfft_cpx* fout, uint32_t batch, void* stream);
KFFT_API size_t kfft_noalloc_scratch_bytes(void);
KFFT_API const char* kfft_noalloc_last_message(void);

/*
 * Plan variants and the tuning table.  The reference plans one way per length
 * (kfft_generic.c:129-151 factorisation); the engine can split a length into
 * passes several ways (largest pass length, lanes per tile, one fused pass or
 * several, shared-memory or register tiles, tensor-core radix-16 stages) and
 * lets a tuner choose.  Variant 0 is the built-in default; every variant
 * computes the same transform (the tensor-core variant only in the float
 * build and only for plans whose flags carry KFFT_FLAG_TENSOR_CORES, because
 * it trades accuracy for speed).
 *
 * kfft_config_cpx_variant builds a complex plan with an explicit variant and
 * otherwise behaves as kfft_config_cpx.  kfft_tune_set records that complex
 * plans of length nfft with the direction and tensor-core bits of `flags`
 * should use `variant`; every later kfft_config_cpx (and every complex plan a
 * scalar, 2D or convolution plan builds inside) then uses it.  An explicit or
 * tuned variant decides the tensor-core stages itself; without one,
 * KFFT_FLAG_TENSOR_CORES alone does.  The table is process-wide and
 * thread-safe.  kfft_tune_get returns the recorded variant or -1.
 */
KFFT_API uint32_t kfft_variant_count(void);
KFFT_API kfft_plan_cpx* kfft_config_cpx_variant(uint32_t nfft, uint32_t flags, uint32_t variant,
                                                kfft_pool_t* A, size_t* lenmem);
KFFT_API kfft_return_t kfft_tune_set(uint32_t nfft, uint32_t flags, uint32_t variant);
KFFT_API int kfft_tune_get(uint32_t nfft, uint32_t flags);
KFFT_API void kfft_tune_clear(void);

/*
 * Cost model of the tuner: a 3-layer MLP (in_dim -> 64 -> 64 -> 1, ReLU) kept
 * in device memory and trained by the engine's own CUDA kernels in FP32 with
 * Adam on mean squared error.  Rows of X are feature vectors (row-major,
 * n x in_dim, host memory, in_dim <= 64), y the targets.  The model only
 * ranks plan variants; it never touches transform arithmetic.  No
 * counterpart in the reference, whose planner has one fixed rule.
 *   kfft_mlp_create    new model with seeded He-uniform weights, NULL on error
 *   kfft_mlp_params    number of FP32 parameters (W1,b1,W2,b2,W3,b3 packed)
 *   kfft_mlp_get/set   copy the packed parameters out of / into the model
 *   kfft_mlp_predict   out[i] = f(X[i])
 *   kfft_mlp_loss_grad loss = mean (f(X)-y)^2 and its gradient (packed like
 *                      the parameters) over all n rows, without an update
 *   kfft_mlp_train     `epochs` passes of minibatch Adam; returns the final
 *                      full-set loss in *loss (may be NULL)
 */
typedef struct kfft_mlp kfft_mlp;
KFFT_API kfft_mlp* kfft_mlp_create(uint32_t in_dim, uint64_t seed);
KFFT_API void kfft_mlp_release(kfft_mlp* m);
KFFT_API uint32_t kfft_mlp_params(const kfft_mlp* m);
KFFT_API kfft_return_t kfft_mlp_get(const kfft_mlp* m, float* params);
KFFT_API kfft_return_t kfft_mlp_set(kfft_mlp* m, const float* params);
KFFT_API kfft_return_t kfft_mlp_predict(kfft_mlp* m, const float* X, uint32_t n, float* out);
KFFT_API kfft_return_t kfft_mlp_loss_grad(kfft_mlp* m, const float* X, const float* y,
                                          uint32_t n, float* loss, float* grad);
KFFT_API kfft_return_t kfft_mlp_train(kfft_mlp* m, const float* X, const float* y, uint32_t n,
                                      uint32_t epochs, uint32_t minibatch, float lr,
                                      uint64_t seed, float* loss);

/*
 * Failure-detection check of the uneven-batch queue kernel, without a GPU
 * fault: runs a queue of empty passes whose dependency is (satisfiable != 0)
 * or is not (0) ever met, with dependency waits limited to max_polls polls of
 * about 200 ns.  Returns the kernel's error word (0: every wait succeeded,
 * 1: a wait gave up and the kernel returned) or -1 on a CUDA error.
 */
KFFT_API int kfft_gb300_queue_selftest(uint32_t max_polls, int satisfiable);

/*
 * Bounded device waits.  The FP32 single-pass kernel that receives its tiles
 * by bulk copy waits on each copy with a bounded poll loop; if a wait runs out
 * (only a failed or very slow copy can cause that) its CTA stops and the
 * output is incomplete.  Synchronous entry points then return
 * KFFT_RET_BUFFER_FAIL.  For asynchronous entry points (kfft_eval_cpx_async,
 * kfft_eval_cpx_noalloc) kfft_gb300_check_waits synchronises `stream` and
 * returns 1 if such a wait of this host thread's earlier calls ran out, 0 if
 * none did, -1 on a CUDA error; it clears the record.
 * kfft_gb300_set_bulk_wait_polls is a test hook: the polls a wait makes
 * before it gives up (0 restores the default of about a second).
 */
KFFT_API int kfft_gb300_check_waits(void* stream);
KFFT_API void kfft_gb300_set_bulk_wait_polls(uint32_t polls);

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
