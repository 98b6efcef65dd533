/*
 * Runs every plan kind of the tiny API (include/kfft_tiny.h) through the
 * engine, on the calls the reference's docs/example/example_tiny.c makes
 * (complex 1D inverse with GENERIC_ONLY, scalar 1D, scalar and complex 2D
 * convolution of 50 x 50) plus the kinds it leaves out (complex and scalar
 * 2D, 1D convolutions, the real inverse).  Inputs are read from
 * <dir>/in.bin and every output is written to <dir>/out_<name>.bin, for
 * tests/test_gpu_tiny_api.py to compare against the oracle.  Buffers come
 * from kfft_malloc, as the example's do.  Exit status: 0, or the first
 * failing step's number.
 */
#include <stdio.h>
#include <string.h>

#include "kfft_tiny.h"

#define N1 100
#define NX 50
#define NY 50
#define N2 (NX * NY)

static const char* g_dir;

static int save(const char* name, const void* p, size_t bytes) {
    char path[1024];
    snprintf(path, sizeof(path), "%s/out_%s.bin", g_dir, name);
    FILE* f = fopen(path, "wb");
    if (!f) return 0;
    const size_t w = fwrite(p, 1, bytes, f);
    fclose(f);
    return w == bytes;
}

int main(int argc, char** argv) {
    if (argc < 2) return 100;
    g_dir = argv[1];
    char path[1024];
    snprintf(path, sizeof(path), "%s/in.bin", g_dir);
    /* inputs: a, b (complex, N2 each), ra, rb (real, N2 each) */
    const size_t cbytes = N2 * sizeof(kfft_cpx), rbytes = N2 * sizeof(kfft_scalar);
    kfft_cpx* a = (kfft_cpx*)kfft_malloc((uint32_t)cbytes);
    kfft_cpx* b = (kfft_cpx*)kfft_malloc((uint32_t)cbytes);
    kfft_scalar* ra = (kfft_scalar*)kfft_malloc((uint32_t)rbytes);
    kfft_scalar* rb = (kfft_scalar*)kfft_malloc((uint32_t)rbytes);
    kfft_cpx* out = (kfft_cpx*)kfft_malloc((uint32_t)(2 * cbytes));
    kfft_scalar* rout = (kfft_scalar*)kfft_malloc((uint32_t)(2 * rbytes));
    if (!a || !b || !ra || !rb || !out || !rout) return 101;
    FILE* f = fopen(path, "rb");
    if (!f) return 102;
    int ok = fread(a, 1, cbytes, f) == cbytes && fread(b, 1, cbytes, f) == cbytes &&
             fread(ra, 1, rbytes, f) == rbytes && fread(rb, 1, rbytes, f) == rbytes;
    fclose(f);
    if (!ok) return 103;

    kfft_args_norm n1 = {N1};
    kfft_args_2d d2 = {NX, NY};
    kfft_plan p;

    /* 1: complex 1D forward */
    p = kfft_configuration(KFFT_PLAN_COMPLEX, KFFT_FLAG_NORMAL, &n1);
    if (!p || kfft_evaluation(p, a, out) != KFFT_RET_SUCCESS || !save("cpx_fwd", out, N1 * sizeof(kfft_cpx)))
        return 1;
    kfft_finalization(p);
    if (p) return 1;
    /* 2: complex 1D inverse with GENERIC_ONLY, as the example's first call */
    p = kfft_configuration(KFFT_PLAN_COMPLEX, KFFT_FLAG_INVERSE | KFFT_FLAG_GENERIC_ONLY, &n1);
    if (!p || kfft_evaluation(p, a, out) != KFFT_RET_SUCCESS || !save("cpx_inv", out, N1 * sizeof(kfft_cpx)))
        return 2;
    kfft_finalization(p);
    /* 3: scalar 1D forward, 4: scalar 1D inverse of its spectrum */
    p = kfft_configuration(KFFT_PLAN_SCALAR, KFFT_FLAG_NORMAL, &n1);
    if (!p || kfft_evaluation(p, ra, out) != KFFT_RET_SUCCESS ||
        !save("sclr_fwd", out, (N1 / 2 + 1) * sizeof(kfft_cpx)))
        return 3;
    kfft_finalization(p);
    p = kfft_configuration(KFFT_PLAN_SCALAR, KFFT_FLAG_INVERSE, &n1);
    if (!p || kfft_evaluation(p, out, rout) != KFFT_RET_SUCCESS || !save("sclr_inv", rout, N1 * sizeof(kfft_scalar)))
        return 4;
    kfft_finalization(p);
    /* 5: complex 2D forward, 6: scalar 2D forward */
    p = kfft_configuration(KFFT_PLAN_COMPLEX_2D, KFFT_FLAG_NORMAL, &d2);
    if (!p || kfft_evaluation(p, a, out) != KFFT_RET_SUCCESS || !save("cpx2_fwd", out, cbytes))
        return 5;
    kfft_finalization(p);
    p = kfft_configuration(KFFT_PLAN_SCALAR_2D, KFFT_FLAG_NORMAL, &d2);
    if (!p || kfft_evaluation(p, ra, out) != KFFT_RET_SUCCESS || !save("sclr2_fwd", out, cbytes))
        return 6;
    kfft_finalization(p);
    /* 7: complex 1D convolution, 8: scalar 1D convolution */
    p = kfft_configuration(KFFT_PLAN_COMPLEX_CONV, KFFT_FLAG_NORMAL, &n1);
    if (!p || kfft_convolution(p, a, b, out) != KFFT_RET_SUCCESS || !save("conv_cpx", out, N1 * sizeof(kfft_cpx)))
        return 7;
    kfft_finalization(p);
    p = kfft_configuration(KFFT_PLAN_SCALAR_CONV, KFFT_FLAG_NORMAL, &n1);
    if (!p || kfft_convolution(p, ra, rb, rout) != KFFT_RET_SUCCESS ||
        !save("conv_sclr", rout, N1 * sizeof(kfft_scalar)))
        return 8;
    kfft_finalization(p);
    /* 9: scalar 2D convolution and 10: complex 2D convolution (GENERIC flag), as the example */
    p = kfft_configuration(KFFT_PLAN_SCALAR_CONV2D, KFFT_FLAG_NORMAL, &d2);
    if (!p || kfft_convolution(p, ra, rb, rout) != KFFT_RET_SUCCESS || !save("conv2_sclr", rout, rbytes))
        return 9;
    kfft_finalization(p);
    p = kfft_configuration(KFFT_PLAN_COMPLEX_CONV2D, KFFT_FLAG_GENERIC, &d2);
    if (!p || kfft_convolution(p, a, b, out) != KFFT_RET_SUCCESS || !save("conv2_cpx", out, cbytes))
        return 10;
    kfft_finalization(p);
    /* 11: a NULL plan and an unknown kind are errors, not crashes */
    if (kfft_evaluation((kfft_plan)NULL, a, out) != KFFT_RET_BADARGUMENTS) return 11;
    if (kfft_configuration(0x0004, 0, &n1) != NULL) return 11;

    kfft_free(a);
    kfft_free(b);
    kfft_free(ra);
    kfft_free(rb);
    kfft_free(out);
    kfft_free(rout);
    if (a || b || ra || rb || out || rout) return 12;
    printf("tiny api ok\n");
    return 0;
}
