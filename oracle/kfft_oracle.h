/*
 * kfft_oracle.h -- TEST INFRASTRUCTURE ONLY: the FP64 CPU restatement of the
 * reference kfft transform path, used as the parity checker and as the timed
 * CPU baseline.  The product library never includes or links it.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The default build computes in double.  Compiled with -DORACLE_FLOAT it
 * follows the reference's float build (KFFT_HALF_SCALAR, incs/kfft_types.h:21-25):
 * data, butterflies and tables in float, tables computed in double and rounded
 * once.  The float flavour is the timed CPU baseline of float workloads. */
#ifdef ORACLE_FLOAT
typedef float oreal;
#else
typedef double oreal;
#endif

typedef struct {
    oreal r, i;
} ocpx;

/* flag and return values of the reference, incs/kfft_types.h:46-57, 82-94 */
enum {
    OR_FLAG_NORMAL = 0,
    OR_FLAG_INVERSE = 1 << 0,
    OR_FLAG_RENEW = 1 << 1,
    OR_FLAG_GENERIC = 1 << 2,
    OR_FLAG_GENERIC_ONLY = 1 << 3,
    OR_FLAG_EXPAND_SCALAR = 1 << 4,
    OR_FLAG_DISABLE_NORM = 1 << 5,
};
enum {
    OR_RET_SUCCESS = 0,
    OR_RET_ALLOC_FAIL = 1,
    OR_RET_BUFFER_FAIL = 2,
    OR_RET_FREE_NULL = 3,
    OR_RET_IMPROPER_PLAN = 4,
    OR_RET_BADARGUMENTS = 5,
};

void* oracle_plan_cpx(uint32_t nfft, uint32_t flags);
void oracle_plan_free(void* plan);
int oracle_exec_cpx(const void* plan, const ocpx* in, ocpx* out);
int oracle_exec_cpx_batch(const void* plan, const ocpx* in, ocpx* out, uint64_t batch,
                          int threads);
int oracle_fft_cpx(uint32_t nfft, uint32_t flags, const ocpx* in, ocpx* out);
void* oracle_uneven_create(uint32_t count, const uint32_t* lengths, uint32_t flags);
int oracle_uneven_exec(const void* u, const ocpx* in, ocpx* out, int threads);
void oracle_uneven_free(void* u);
int oracle_exec_uneven(uint32_t count, const uint32_t* lengths, uint32_t flags, const ocpx* in,
                       ocpx* out, int threads);
int oracle_rfft(uint32_t nfft, uint32_t flags, const oreal* in, ocpx* out);
int oracle_irfft(uint32_t nfft, uint32_t flags, const ocpx* in, oreal* out);
int oracle_fft2_cpx(uint32_t x, uint32_t y, uint32_t flags, const ocpx* in, ocpx* out);
int oracle_rfft2(uint32_t x, uint32_t y, uint32_t flags, const oreal* in, ocpx* out);
int oracle_irfft2(uint32_t x, uint32_t y, uint32_t flags, const ocpx* in, oreal* out);
int oracle_conv_cpx(uint32_t nfft, uint32_t flags, const ocpx* a, const ocpx* b, ocpx* out);
int oracle_conv_scalar(uint32_t nfft, uint32_t flags, const oreal* a, const oreal* b,
                       oreal* out);
int oracle_conv2_cpx(uint32_t x, uint32_t y, uint32_t flags, const ocpx* a, const ocpx* b,
                     ocpx* out);
int oracle_conv2_scalar(uint32_t x, uint32_t y, uint32_t flags, const oreal* a, const oreal* b,
                        oreal* out);
int oracle_dft_exact(uint32_t nfft, int inverse, const ocpx* in, ocpx* out);

#ifdef __cplusplus
}
#endif
