/*
 * kfft_tiny.h -- the reference's "tiny" convenience API (kfft_tiny.h:85-275
 * of kfft v0.8.1) over the GB300 engine: one type-erased plan handle for every
 * plan kind, created by kfft_configuration, run by kfft_evaluation or
 * kfft_convolution and released by kfft_finalization.
 *
 * The names, enum values, argument structs and macros are the reference's, so
 * a program written against its tiny header (docs/example/example_tiny.c)
 * compiles unchanged against this one; the implementation is this engine's
 * own.  Differences from the reference header:
 *   - every extension (2D, conv, conv2d) is always present, as in the engine;
 *   - the sparse plan kinds, disabled in the reference build, are not offered;
 *   - kfft_evaluation / kfft_convolution return KFFT_RET_BADARGUMENTS for a
 *     NULL plan instead of dereferencing it.
 * Buffers may be host or device memory (the engine stages host buffers).
 * Compile with -DKFFT_HALF_SCALAR against libkfft_gb300_f.so for the float
 * build, without it against libkfft_gb300.so.
 */
#pragma once

#include "kfft.h"

#ifdef __cplusplus
extern "C" {
#endif

/* plan kinds (kfft_tiny.h:21-32) */
enum ktiny_plan_type {
    KFFT_PLAN_COMPLEX = 0x0000,
    KFFT_PLAN_SCALAR = 0x0001,
    KFFT_PLAN_COMPLEX_2D = 0x0002,
    KFFT_PLAN_SCALAR_2D = 0x0003,
    KFFT_PLAN_COMPLEX_CONV = 0x0006,
    KFFT_PLAN_SCALAR_CONV = 0x0007,
    KFFT_PLAN_COMPLEX_CONV2D = 0x0008,
    KFFT_PLAN_SCALAR_CONV2D = 0x0009,
};

/* the type-erased handle: the typed plan's address and its kind */
typedef struct {
    uintptr_t state;
    int type;
} kfft_plan_t;
typedef kfft_plan_t* kfft_plan;

#define KTINY_CAST(type, X) (kfft_plan_##type*)((X)->state)
#define KTINY_FLAGS(type, X) (KTINY_CAST(type, (X)))->flags
#define KTINY_CPX(X) (kfft_cpx*)(X)
#define KTINY_SCLR(X) (kfft_scalar*)(X)

/* arguments of 1D and 2D plan kinds */
typedef struct {
    uint32_t nfft;
} kfft_args_norm;
typedef struct {
    uint32_t x; /* row length (contiguous) */
    uint32_t y; /* rows */
} kfft_args_2d;

#define kfft_configuration(T, F, A) kfft_tiny_config((T), (F), (uintptr_t)(A))
#define kfft_evaluation(P, Fi, Fo) kfft_tiny_eval(P, (kfft_scalar*)(Fi), (kfft_scalar*)(Fo))
#define kfft_convolution(P, Fi1, Fi2, Fo) \
    kfft_tiny_conv(P, (kfft_scalar*)(Fi1), (kfft_scalar*)(Fi2), (kfft_scalar*)(Fo))
#define kfft_finalization(P) kfft_tiny_release(&(P))

/* Creates the typed plan of kind `type` (a private pool; KFFT_FLAG_RENEW has
 * no meaning here and is dropped); NULL on failure or an unknown kind. */
static kfft_plan KFFT_UNUSED_FUNC kfft_tiny_config(unsigned type, uint32_t flags, uintptr_t args) {
    const kfft_args_norm* n = (const kfft_args_norm*)args;
    const kfft_args_2d* d = (const kfft_args_2d*)args;
    void* typed = NULL;
    kfft_plan plan;
    flags &= ~(uint32_t)KFFT_FLAG_RENEW;
    if (!args) return NULL;
    switch (type) {
        case KFFT_PLAN_COMPLEX: typed = kfft_config_cpx(n->nfft, flags, NULL, NULL); break;
        case KFFT_PLAN_SCALAR: typed = kfft_config_scalar(n->nfft, flags, NULL, NULL); break;
        case KFFT_PLAN_COMPLEX_2D: typed = kfft_config2_cpx(d->x, d->y, flags, NULL, NULL); break;
        case KFFT_PLAN_SCALAR_2D: typed = kfft_config2_scalar(d->x, d->y, flags, NULL, NULL); break;
        case KFFT_PLAN_COMPLEX_CONV: typed = kfft_config_conv_cpx(n->nfft, flags, NULL, NULL); break;
        case KFFT_PLAN_SCALAR_CONV: typed = kfft_config_conv_scalar(n->nfft, flags, NULL, NULL); break;
        case KFFT_PLAN_COMPLEX_CONV2D:
            typed = kfft_config2_conv_cpx(d->x, d->y, flags, NULL, NULL);
            break;
        case KFFT_PLAN_SCALAR_CONV2D:
            typed = kfft_config2_conv_scalar(d->x, d->y, flags, NULL, NULL);
            break;
        default: return NULL;
    }
    if (!typed) return NULL;
    plan = (kfft_plan)kfft_malloc(sizeof(kfft_plan_t));
    if (!plan) {
        kfft_cleanup(typed);
        return NULL;
    }
    plan->state = (uintptr_t)typed;
    plan->type = (int)type;
    return plan;
}

/* One transform; a real plan made with KFFT_FLAG_INVERSE runs the inverse
 * (spectrum in, real samples out), as the reference's tiny API does. */
static kfft_return_t KFFT_UNUSED_FUNC kfft_tiny_eval(const kfft_plan plan, const kfft_scalar* fin,
                                                     kfft_scalar* fout) {
    if (!plan) return KFFT_RET_BADARGUMENTS;
    switch (plan->type) {
        case KFFT_PLAN_COMPLEX:
            return kfft_eval_cpx(KTINY_CAST(cpx, plan), KTINY_CPX(fin), KTINY_CPX(fout));
        case KFFT_PLAN_SCALAR:
            if (KTINY_FLAGS(sclr, plan) & KFFT_FLAG_INVERSE)
                return kfft_evali_scalar(KTINY_CAST(sclr, plan), KTINY_CPX(fin), fout);
            return kfft_eval_scalar(KTINY_CAST(sclr, plan), fin, KTINY_CPX(fout));
        case KFFT_PLAN_COMPLEX_2D:
            return kfft_eval2_cpx(KTINY_CAST(c2d, plan), KTINY_CPX(fin), KTINY_CPX(fout));
        case KFFT_PLAN_SCALAR_2D:
            if (KTINY_FLAGS(s2d, plan) & KFFT_FLAG_INVERSE)
                return kfft_evali2_scalar(KTINY_CAST(s2d, plan), KTINY_CPX(fin), fout);
            return kfft_eval2_scalar(KTINY_CAST(s2d, plan), fin, KTINY_CPX(fout));
        default: return KFFT_RET_IMPROPER_PLAN;
    }
}

/* One circular convolution of two inputs (convolution plan kinds only). */
static kfft_return_t KFFT_UNUSED_FUNC kfft_tiny_conv(const kfft_plan plan, const kfft_scalar* fin1,
                                                     const kfft_scalar* fin2, kfft_scalar* fout) {
    if (!plan) return KFFT_RET_BADARGUMENTS;
    switch (plan->type) {
        case KFFT_PLAN_COMPLEX_CONV:
            return kfft_eval_conv_cpx(KTINY_CAST(ccnv, plan), KTINY_CPX(fin1), KTINY_CPX(fin2),
                                      KTINY_CPX(fout));
        case KFFT_PLAN_SCALAR_CONV:
            return kfft_eval_conv_scalar(KTINY_CAST(scnv, plan), fin1, fin2, fout);
        case KFFT_PLAN_COMPLEX_CONV2D:
            return kfft_eval2_conv_cpx(KTINY_CAST(c2cnv, plan), KTINY_CPX(fin1), KTINY_CPX(fin2),
                                       KTINY_CPX(fout));
        case KFFT_PLAN_SCALAR_CONV2D:
            return kfft_eval2_conv_scalar(KTINY_CAST(s2cnv, plan), fin1, fin2, fout);
        default: return KFFT_RET_IMPROPER_PLAN;
    }
}

/* Releases the typed plan and the handle, and sets the handle to NULL. */
static void KFFT_UNUSED_FUNC kfft_tiny_release(kfft_plan* plan) {
    if (!plan || !*plan) return;
    kfft_cleanup((void*)((*plan)->state));
    kfft_free(*plan);
}

#ifdef __cplusplus
}
#endif
