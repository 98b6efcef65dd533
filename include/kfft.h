/*
 * kfft.h -- drop-in C API of the GB300 FFT engine.
 *
 * Same names, types, flag values, return codes, ownership protocol and
 * struct-first-member convention as the reference LibKFFT v0.8.1 public
 * header (kfft.h:49-104 and the incs/ + ext/ headers it includes), so C code
 * written against the reference recompiles against this header and links
 * libkfft_gb300.so (double) or libkfft_gb300_f.so (float, KFFT_HALF_SCALAR)
 * instead.  Each declaration cites the reference declaration it replaces.
 *
 * Behind the API, plans live on the GPU (twiddle, Rader and Bluestein tables
 * generated in FP64 on the device and resident in HBM) and every transform
 * runs as sm_103a CUDA kernels.  Buffers passed to kfft_eval_* may be host
 * memory (staged through the device) or device memory (used in place).
 * There is no CPU fallback: when no GPU is usable, kfft_config_* returns NULL.
 */
#pragma once

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

/* version of the reference API this header mirrors (meson.build:2) */
#define KFFT_MAJOR_VERSION 0
#define KFFT_MINOR_VERSION 8
#define KFFT_PATCH_VERSION 1

#if defined(_WIN32)
#define KFFT_API __declspec(dllexport)
#else
#define KFFT_API __attribute__((visibility("default")))
#endif

/* ---- config.h.in:30-37: the 2D, convolution and 2D convolution extensions
 * are always built into this library, so code that tests for them (the tiny
 * API, kfft_tiny.h) sees them enabled. */
#ifndef KFFT_2D_ENABLE
#define KFFT_2D_ENABLE
#endif
#ifndef KFFT_CONV_ENABLE
#define KFFT_CONV_ENABLE
#endif
#ifndef KFFT_CONV2D_ENABLE
#define KFFT_CONV2D_ENABLE
#endif

/* ---- incs/kfft_macro.h:139-144 ------------------------------------------ */
#define KFFT_UNUSED_VAR(X) (void)(X)
#if defined(_MSC_VER)
#define KFFT_UNUSED_FUNC
#else
#define KFFT_UNUSED_FUNC __attribute__((__unused__))
#endif

/* ---- incs/kfft_types.h:21-31 ------------------------------------------- */
#if defined(KFFT_HALF_SCALAR)
typedef float kfft_scalar;
#else
typedef double kfft_scalar;
#endif

typedef struct {
    kfft_scalar r; /* real part */
    kfft_scalar i; /* imaginary part */
} kfft_cpx;

/* ---- incs/kfft_types.h:34-43: build information bits -------------------- */
enum kfft_info_flags {
    KFFT_INFO_TRACE = 1 << 0,
    KFFT_INFO_USE_SIMD = 1 << 1,
    KFFT_INFO_USE_ALLOCA = 1 << 2,
    KFFT_INFO_USE_SYSMATH = 1 << 3,
    KFFT_INFO_USE_OPENMP = 1 << 4,
    KFFT_INFO_RADER_ALGO = 1 << 5,
    KFFT_INFO_MEMLESS_MODE = 1 << 6,
    KFFT_INFO_HALF_SCALAR = 1 << 7,
};

/* ---- incs/kfft_types.h:46-57: plan flags -------------------------------- */
enum kfft_eval_flags {
    KFFT_FLAG_NORMAL = 0,
    KFFT_FLAG_INVERSE = 1 << 0,
    KFFT_FLAG_RENEW = 1 << 1,
    KFFT_FLAG_GENERIC = 1 << 2,       /* accepted; the GPU plan picks its own prime method */
    KFFT_FLAG_GENERIC_ONLY = 1 << 3,  /* accepted; computes the same DFT */
    KFFT_FLAG_EXPAND_SCALAR = 1 << 4, /* real forward: write all N bins */
    KFFT_FLAG_DISABLE_NORM = 1 << 5,  /* inverse: no 1/N */
};

/* incs/kfft_types.h:65 */
#define KFFT_CHECK_FLAGS(X) ((X) & (~KFFT_FLAG_RENEW))

/* incs/kfft_types.h:73-78 */
typedef struct {
    uint16_t vmajor;
    uint16_t vminor;
    uint16_t vpatch;
    uint16_t flags;
} kfft_info_t;

/* ---- incs/kfft_types.h:82-94: return codes ------------------------------ */
enum kfft_ret_flags {
    KFFT_RET_SUCCESS = 0x0000,
    KFFT_RET_ALLOC_FAIL = 0x0001,
    KFFT_RET_BUFFER_FAIL = 0x0002,
    KFFT_RET_FREE_NULL = 0x0003,
    KFFT_RET_IMPROPER_PLAN = 0x0004,
    KFFT_RET_BADARGUMENTS = 0x0005
};
typedef unsigned kfft_return_t;

/* incs/kfft_types.h:101-104 (kept for layout compatibility of kfft_pool_t) */
typedef struct {
    uint8_t arch;
    uint32_t ext;
} kfft_simd_t;

/* ---- incs/kfft_pool.h:14-75: plan memory pool --------------------------- */
/*
 * A bump allocator holding the host side of one or more plan trees.  The
 * device side of every plan allocated in a pool (its HBM arena) is registered
 * in the pool and released by kfft_pool_free / kfft_pool_clear / kfft_cleanup.
 */
typedef struct kfft_pool_s {
    size_t allocated; /* pool area size incl. header */
    uint8_t align;
    kfft_simd_t vex;

    uint8_t* head;
    uint8_t* tail;
    uint8_t* cur;

    void* device; /* registry of the device arenas of plans in this pool */

    uint8_t area[1];
} kfft_pool_t;

KFFT_API kfft_pool_t* kfft_pool_create(const size_t size);                /* kfft_pool.h:30 */
KFFT_API void* kfft_pool_alloc(kfft_pool_t* A, const size_t nmem);        /* kfft_pool.h:38 */
KFFT_API size_t kfft_pool_empty(const kfft_pool_t* A);                    /* kfft_pool.h:45 */
KFFT_API void kfft_pool_zmem(const kfft_pool_t* A, void* ptr, const size_t size); /* :52 */
KFFT_API void kfft_pool_clear(kfft_pool_t* A);                            /* kfft_pool.h:58 */
KFFT_API void kfft_pool_free(kfft_pool_t* A);                             /* kfft_pool.h:64 */
#define kfft_pool_free_and_null(A)                                                                 \
    do {                                                                                           \
        kfft_pool_free(A);                                                                         \
        A = NULL;                                                                                  \
    } while (0)

/* ---- incs/kfft_cpx.h:16-65: complex plan -------------------------------- */
#define MAX_FACTORS 32
#define MAX_ROOTS 32

typedef struct {
    kfft_pool_t* mmgr; /* first member of every plan (incs/kfft_cpx.h:21-23) */
} kfft_object_t;

struct kfft_gpu_plan; /* opaque device-resident plan */

typedef struct kfft_kstate {
    kfft_object_t object;

    uint32_t nfft;
    uint8_t level;
    uint32_t flags;

    uint8_t fac_count;                 /* number of passes of the GPU schedule */
    uint32_t factors[2 * MAX_FACTORS]; /* (pass length, remaining length) pairs */

    uint8_t prm_count; /* 1 when the length runs through Rader or Bluestein */
    uint32_t method;   /* 0 direct mixed radix, 1 Rader, 2 Bluestein */

    struct kfft_gpu_plan* gpu;
} kfft_plan_cpx;

/* incs/kfft_cpx.h:96-97 */
KFFT_API kfft_plan_cpx* kfft_config_cpx(const uint32_t nfft, const uint32_t flags, kfft_pool_t* A,
                                        size_t* lenmem);
/* incs/kfft_cpx.h:110-111 */
KFFT_API kfft_return_t kfft_eval_cpx(kfft_plan_cpx* plan, const kfft_cpx* fin, kfft_cpx* fout);

/* incs/kfft_cpx.h:118-138 */
#define KFFT_PLAN_MMGR(X) (*((kfft_pool_t**)(X)))
#define KFFT_PLAN_MMGR_NULL(X) ((X != NULL) ? KFFT_PLAN_MMGR((X)) : NULL)
#define KFFT_PLAN_ALIGN(X) ((X != NULL) ? KFFT_PLAN_MMGR((X))->align : 0)
#define KFFT_PLAN_VEX(X) KFFT_PLAN_MMGR((X))->vex

/* ---- incs/kfft_scalar.h:15-60: real ("scalar") plan --------------------- */
typedef struct kfft_state {
    kfft_object_t object;

    uint32_t nfft;
    uint32_t flags;

    kfft_plan_cpx* basis; /* N/2 (even N) or N (odd N) complex plan */
    struct kfft_gpu_plan* gpu;
} kfft_plan_sclr;

KFFT_API kfft_plan_sclr* kfft_config_scalar(const uint32_t nfft, const uint32_t flags,
                                            kfft_pool_t* A, size_t* lenmem); /* :35-36 */
KFFT_API kfft_return_t kfft_eval_scalar(kfft_plan_sclr* plan, const kfft_scalar* fin,
                                        kfft_cpx* fout); /* :46-47 */
KFFT_API kfft_return_t kfft_evali_scalar(kfft_plan_sclr* plan, const kfft_cpx* fin,
                                         kfft_scalar* fout); /* :59-60 */

/* ---- incs/kfft_ext.h:16-66: service functions --------------------------- */
KFFT_API void kfft_info(kfft_info_t* info);
KFFT_API uint32_t kfft_next_fast_size(uint32_t n);
KFFT_API void* kfft_malloc(uint32_t sz);
KFFT_API void kfft_free_null(void** mem);
#define kfft_free(X) (kfft_free_null((void**)(&(X))))
KFFT_API kfft_return_t kfft_cleanup(void* mem);
#define kfft_release(X)                                                                            \
    do {                                                                                           \
        if (kfft_cleanup((void*)(X)) == KFFT_RET_SUCCESS)                                          \
            (X) = NULL;                                                                            \
    } while (0)
KFFT_API const char* kfft_strerr(const kfft_return_t code);

/* ---- incs/kfft_shift.h:16-27: fftshift (forward) / ifftshift (inverse) ---- */
KFFT_API void kfft_shift_cpx(kfft_cpx* buf, const uint32_t size, const bool is_inverse,
                             kfft_pool_t* mmgr);
KFFT_API void kfft_shift_scalar(kfft_scalar* buf, const uint32_t size, const bool is_inverse,
                                kfft_pool_t* mmgr);

/* ---- incs/kfft_math.h:251-350: element-wise and layout helpers ----------- */
KFFT_API void kfft_math_hadamard_cpx(kfft_cpx* Fout, const kfft_cpx* Fin, uint32_t size);
KFFT_API void kfft_math_hadamard_scalar(kfft_scalar* Fout, const kfft_scalar* Fin, uint32_t size);
KFFT_API void kfft_math_transpose_cpx(const kfft_cpx* Fin, kfft_cpx* Fout, const uint32_t x,
                                      const uint32_t y);
KFFT_API void kfft_math_transpose_scalar(const kfft_scalar* Fin, kfft_scalar* Fout,
                                         const uint32_t x, const uint32_t y);
KFFT_API void kfft_math_transpose_ip_cpx(kfft_cpx* Fin, const uint32_t x, const uint32_t y);
KFFT_API void kfft_math_transpose_ip_scalar(kfft_scalar* Fin, const uint32_t x, const uint32_t y);
KFFT_API void kfft_math_magnitude(const kfft_cpx* Fin, kfft_scalar* Fout, uint32_t size);
KFFT_API void kfft_math_magnitude_ip(kfft_cpx* Fin, uint32_t size);
KFFT_API kfft_scalar kfft_math_average(const kfft_scalar* Fin, uint32_t size);

/* ---- ext/2d/kfft_cpx2.h:3-17, ext/2d/kfft_scalar2.h:3-19 ----------------- */
typedef struct {
    kfft_object_t object;

    uint32_t nfft, x, y;
    uint32_t flags;

    kfft_plan_cpx* plan_x;
    kfft_plan_cpx* plan_y;
} kfft_plan_c2d;

KFFT_API kfft_plan_c2d* kfft_config2_cpx(const uint32_t x_size, const uint32_t y_size,
                                         const uint32_t flags, kfft_pool_t* A, size_t* lenmem);
KFFT_API kfft_return_t kfft_eval2_cpx(kfft_plan_c2d* cfg, const kfft_cpx* fin, kfft_cpx* fout);
KFFT_API void kfft_shift2_cpx(kfft_cpx* buf, kfft_cpx* ftmp, const uint32_t sz_x,
                              const uint32_t sz_y, const bool is_inverse, kfft_pool_t* mmgr);

typedef struct {
    kfft_object_t object;

    uint32_t nfft, x, y;
    uint32_t flags;

    kfft_object_t* plan_x;
    kfft_object_t* plan_y;
} kfft_plan_s2d;

KFFT_API kfft_plan_s2d* kfft_config2_scalar(const uint32_t x_size, const uint32_t y_size,
                                            const uint32_t flags, kfft_pool_t* A, size_t* lenmem);
KFFT_API kfft_return_t kfft_eval2_scalar(kfft_plan_s2d* plan, const kfft_scalar* fin,
                                         kfft_cpx* fout);
KFFT_API kfft_return_t kfft_evali2_scalar(kfft_plan_s2d* plan, const kfft_cpx* fin,
                                          kfft_scalar* fout);
KFFT_API void kfft_shift2_scalar(kfft_scalar* buf, kfft_scalar* ftmp, const uint32_t sz_x,
                                 const uint32_t sz_y, const bool is_inverse, kfft_pool_t* mmgr);

/* ---- ext/conv/kfft_cpx_conv.h:5-21, ext/conv/kfft_scalar_conv.h:5-19 ----- */
typedef struct {
    kfft_object_t object;

    uint32_t nfft;
    uint32_t flags;

    kfft_plan_cpx* plan_fwd;
    kfft_plan_cpx* plan_inv;
} kfft_plan_ccnv;

#define KFFT_CHECK_FLAGS_CCNV(X) (KFFT_CHECK_FLAGS(X) & (~KFFT_FLAG_INVERSE))

KFFT_API kfft_plan_ccnv* kfft_config_conv_cpx(const uint32_t nfft, const uint32_t flags,
                                              kfft_pool_t* A, size_t* lenmem);
KFFT_API kfft_return_t kfft_eval_conv_cpx(kfft_plan_ccnv* plan, const kfft_cpx* fin_A,
                                          const kfft_cpx* fin_B, kfft_cpx* fout);

typedef struct {
    kfft_object_t object;

    uint32_t nfft;
    uint32_t flags;

    kfft_plan_sclr* plan_fwd;
    kfft_plan_sclr* plan_inv;
} kfft_plan_scnv;

KFFT_API kfft_plan_scnv* kfft_config_conv_scalar(const uint32_t nfft, const uint32_t flags,
                                                 kfft_pool_t* A, size_t* lenmem);
KFFT_API kfft_return_t kfft_eval_conv_scalar(kfft_plan_scnv* plan, const kfft_scalar* fin_A,
                                             const kfft_scalar* fin_B, kfft_scalar* fout);

/* ---- ext/conv2d/kfft_cpx_conv.h:5-23, ext/conv2d/kfft_scalar_conv.h:5-23 - */
typedef struct {
    kfft_object_t object;

    uint32_t nfft;
    uint32_t x;
    uint32_t y;

    uint32_t flags;

    kfft_plan_c2d* plan_fwd;
    kfft_plan_c2d* plan_inv;
} kfft_plan_c2cnv;

KFFT_API kfft_plan_c2cnv* kfft_config2_conv_cpx(const uint32_t x, const uint32_t y,
                                                const uint32_t flags, kfft_pool_t* A,
                                                size_t* lenmem);
KFFT_API kfft_return_t kfft_eval2_conv_cpx(kfft_plan_c2cnv* plan, const kfft_cpx* fin_A,
                                           const kfft_cpx* fin_B, kfft_cpx* fout);

typedef struct {
    kfft_object_t object;

    uint32_t nfft;
    uint32_t x;
    uint32_t y;

    uint32_t flags;

    kfft_plan_s2d* plan_fwd;
    kfft_plan_s2d* plan_inv;
} kfft_plan_s2cnv;

KFFT_API kfft_plan_s2cnv* kfft_config2_conv_scalar(const uint32_t x, const uint32_t y,
                                                   const uint32_t flags, kfft_pool_t* A,
                                                   size_t* lenmem);
KFFT_API kfft_return_t kfft_eval2_conv_scalar(kfft_plan_s2cnv* plan, const kfft_scalar* fin_A,
                                              const kfft_scalar* fin_B, kfft_scalar* fout);

/* ---- DYNAPI callback types (incs/kfft_cpx.h:145-152, incs/kfft_scalar.h:105-115,
 *      incs/kfft_ext.h:68-83, ext headers) ------------------------------- */
typedef kfft_plan_cpx* (*kfft_callback_config_cpx)(const uint32_t nfft, const uint32_t flags,
                                                   kfft_pool_t* A, size_t* lenmem);
typedef kfft_return_t (*kfft_callback_eval_cpx)(kfft_plan_cpx* plan, const kfft_cpx* fin,
                                                kfft_cpx* fout);
typedef kfft_plan_sclr* (*kfft_callback_config_scalar)(const uint32_t nfft, const uint32_t flags,
                                                       kfft_pool_t* A, size_t* lenmem);
typedef kfft_return_t (*kfft_callback_eval_scalar)(kfft_plan_sclr* plan, const kfft_scalar* fin,
                                                   kfft_cpx* fout);
typedef kfft_return_t (*kfft_callback_evali_scalar)(kfft_plan_sclr* plan, const kfft_cpx* fin,
                                                    kfft_scalar* fout);
typedef void (*kfft_callback_info)(kfft_info_t* info);
typedef uint32_t (*kfft_callback_next_fast_size)(uint32_t n);
typedef void* (*kfft_callback_malloc)(uint32_t sz);
typedef void (*kfft_callback_free_null)(void** mem);
typedef kfft_return_t (*kfft_callback_cleanup)(void* mem);
typedef const char* (*kfft_callback_strerr)(const kfft_return_t code);
/* incs/kfft_shift.h:29-36 */
typedef void (*kfft_callback_shift_cpx)(kfft_cpx* buf, const uint32_t size, const bool is_inverse,
                                        kfft_pool_t* mmgr);
typedef void (*kfft_callback_shift_scalar)(kfft_scalar* buf, const uint32_t size,
                                           const bool is_inverse, kfft_pool_t* mmgr);
/* ext/2d/kfft_cpx2.h, ext/2d/kfft_scalar2.h (DYNAPI blocks) */
typedef kfft_plan_c2d* (*kfft_callback_config2_cpx)(const uint32_t x_size, const uint32_t y_size,
                                                    const uint32_t flags, kfft_pool_t* A,
                                                    size_t* lenmem);
typedef kfft_return_t (*kfft_callback_eval2_cpx)(kfft_plan_c2d* cfg, const kfft_cpx* fin,
                                                 kfft_cpx* fout);
typedef void (*kfft_callback_shift2_cpx)(kfft_cpx* buf, kfft_cpx* ftmp, const uint32_t sz_x,
                                         const uint32_t sz_y, const bool is_inverse,
                                         kfft_pool_t* mmgr);
typedef kfft_plan_s2d* (*kfft_callback_config2_scalar)(const uint32_t x_size,
                                                       const uint32_t y_size, const uint32_t flags,
                                                       kfft_pool_t* A, size_t* lenmem);
typedef kfft_return_t (*kfft_callback_eval2_scalar)(kfft_plan_s2d* plan, const kfft_scalar* fin,
                                                    kfft_cpx* fout);
typedef kfft_return_t (*kfft_callback_evali2_scalar)(kfft_plan_s2d* plan, const kfft_cpx* fin,
                                                     kfft_scalar* fout);
typedef void (*kfft_callback_shift2_scalar)(kfft_scalar* buf, kfft_scalar* ftmp,
                                            const uint32_t sz_x, const uint32_t sz_y,
                                            const bool is_inverse, kfft_pool_t* mmgr);
/* ext/conv/kfft_cpx_conv.h, ext/conv/kfft_scalar_conv.h (DYNAPI blocks) */
typedef kfft_plan_ccnv* (*kfft_callback_config_conv_cpx)(const uint32_t nfft, const uint32_t flags,
                                                         kfft_pool_t* A, size_t* lenmem);
typedef kfft_return_t (*kfft_callback_eval_conv_cpx)(kfft_plan_ccnv* plan, const kfft_cpx* fin_A,
                                                     const kfft_cpx* fin_B, kfft_cpx* fout);
typedef kfft_plan_scnv* (*kfft_callback_config_conv_scalar)(const uint32_t nfft,
                                                            const uint32_t flags, kfft_pool_t* A,
                                                            size_t* lenmem);
typedef kfft_return_t (*kfft_callback_eval_conv_scalar)(kfft_plan_scnv* plan,
                                                        const kfft_scalar* fin_A,
                                                        const kfft_scalar* fin_B,
                                                        kfft_scalar* fout);
/* ext/conv2d/kfft_cpx_conv.h, ext/conv2d/kfft_scalar_conv.h (DYNAPI blocks) */
typedef kfft_plan_c2cnv* (*kfft_callback_config_conv2_cpx)(const uint32_t x, const uint32_t y,
                                                           const uint32_t flags, kfft_pool_t* A,
                                                           size_t* lenmem);
typedef kfft_return_t (*kfft_callback_eval_conv2_cpx)(kfft_plan_c2cnv* plan,
                                                      const kfft_cpx* fin_A,
                                                      const kfft_cpx* fin_B, kfft_cpx* fout);
typedef kfft_plan_s2cnv* (*kfft_callback_config_conv2_scalar)(const uint32_t x, const uint32_t y,
                                                              const uint32_t flags,
                                                              kfft_pool_t* A, size_t* lenmem);
typedef kfft_return_t (*kfft_callback_eval_conv2_scalar)(kfft_plan_s2cnv* plan,
                                                         const kfft_scalar* fin_A,
                                                         const kfft_scalar* fin_B,
                                                         kfft_scalar* fout);

#ifdef __cplusplus
}
#endif

#include "kfft_gb300.h"
