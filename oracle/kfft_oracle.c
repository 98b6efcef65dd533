/*
 * kfft_oracle.c -- TEST INFRASTRUCTURE ONLY (the parity oracle).
 *
 * A plain-C, FP64 restatement of the reference kfft v0.8.1 transform path
 * (SkyMaverick/kfft), written from its published behaviour.  It is the checker
 * for the GPU library and the timed CPU baseline ("port") of the benchmark.
 * Nothing in the product links, loads or calls this file.
 *
 * What it restates (file:line inside the reference project):
 *   - radix schedule: 4s first, then 2, then odd p ascending, trial division up
 *     to floor(sqrt(N))                     -- kfft_cpx.c:103-143 (SYSMATH sqrt)
 *   - Rader registration: level < 7, p > 5, p >= RADER_LIMIT (25)
 *                                            -- kfft_cpx.c:131-136
 *   - twiddles exp(-+2 pi i k / N)           -- incs/kfft_math.h:206-216
 *   - recursive decimation in time           -- kfft_work.c:1-59
 *   - radix 2/3/4/5 butterflies              -- kfft_bfly.c:1-152
 *   - generic O(p^2) butterfly               -- kfft_generic.c:9-36
 *   - Rader prime butterfly (m == 1 only)    -- kfft_generic.c:38-80, kfft_rader.c:1-63
 *   - primitive root / inverse generator     -- kfft_math.c:5-38
 *   - 1/N inverse normalisation at level 0 unless DISABLE_NORM, always in
 *     sub-plans                              -- kfft_cpx.c:351-363
 *   - real ("scalar") transform, trivial (odd N) and nyquist (even N) paths,
 *     including the even-N inverse returning 2*x -- kfft_scalar.c:9-329
 *   - 2D complex / scalar                    -- ext/2d/kfft_cpx2.c:92-124,
 *                                               ext/2d/kfft_scalar2.c:120-246
 *   - circular convolution 1D / 2D           -- ext/conv/kfft_*_conv.c, ext/conv2d/kfft_*_conv.c
 *
 * The oracle computes in double; a float build of the library is compared
 * against it with a float tolerance.  Compiled with -DORACLE_FLOAT the same
 * source follows the reference's float build (KFFT_HALF_SCALAR,
 * incs/kfft_types.h:21-25): data and tables in float (tables computed in
 * double and rounded once).  That flavour is only the timed CPU baseline of
 * float workloads, never a checker.
 */
#include "kfft_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_RADER_LIMIT 25u
#define OR_PLAN_LEVEL 7u
#define OR_BFLY_LEVEL 5u
#define OR_MAX_FACTORS 32

static const double OR_PI = 3.14159265358979323846264338327950288;
#define OR_HALF ((oreal)0.5)

/* ------------------------------------------------------------------------- */
/* complex helpers                                                           */
/* ------------------------------------------------------------------------- */
static inline ocpx cmul(ocpx a, ocpx b) {
    ocpx r = {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r};
    return r;
}
static inline ocpx cadd(ocpx a, ocpx b) {
    ocpx r = {a.r + b.r, a.i + b.i};
    return r;
}
static inline ocpx csub(ocpx a, ocpx b) {
    ocpx r = {a.r - b.r, a.i - b.i};
    return r;
}

/* exp(-+2 pi i k / n), the reference's kfft_kernel_twiddle (incs/kfft_math.h:206-216) */
static ocpx twiddle(uint32_t k, uint32_t n, int inverse) {
    double phase = -2.0 * OR_PI * (double)k / (double)n;
    if (inverse) phase = -phase;
    ocpx r = {(oreal)cos(phase), (oreal)sin(phase)};
    return r;
}

static uint32_t modpow(uint32_t x, uint32_t y, uint32_t m) {
    uint64_t result = 1 % m, base = x % m;
    while (y) {
        if (y & 1u) result = (result * base) % m;
        base = (base * base) % m;
        y >>= 1;
    }
    return (uint32_t)result;
}

/* smallest primitive root of prime p (kfft_math.c:5-33) */
static uint32_t primitive_root(uint32_t p) {
    uint32_t phi = p - 1, n = phi, fac[32], cnt = 0;
    for (uint32_t i = 2; (uint64_t)i * i <= n; i++)
        if (n % i == 0) {
            fac[cnt++] = i;
            while (n % i == 0) n /= i;
        }
    if (n > 1) fac[cnt++] = n;
    for (uint32_t g = 2; g <= p; g++) {
        int ok = 1;
        for (uint32_t i = 0; i < cnt && ok; i++)
            if (modpow(g, phi / fac[i], p) == 1) ok = 0;
        if (ok) return g;
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* complex plan                                                              */
/* ------------------------------------------------------------------------- */
typedef struct oplan oplan;

typedef struct {
    uint32_t prime;
    uint32_t *qidx, *pidx; /* g^i mod p and g^-i mod p */
    ocpx* shuffle;         /* FFT_{p-1} of the permuted twiddles */
    oplan *fwd, *inv;      /* (p-1)-point sub-plans */
} orader;

struct oplan {
    uint32_t nfft, flags, level;
    uint32_t nfac;
    uint32_t factors[2 * OR_MAX_FACTORS];
    uint32_t nrader;
    orader rader[OR_MAX_FACTORS];
    ocpx* tw;
};

static oplan* plan_create(uint32_t nfft, uint32_t flags, uint32_t level);
static int plan_exec(const oplan* P, const ocpx* in, ocpx* out);

static void plan_destroy(oplan* P) {
    if (!P) return;
    for (uint32_t i = 0; i < P->nrader; i++) {
        free(P->rader[i].qidx);
        free(P->rader[i].pidx);
        free(P->rader[i].shuffle);
        plan_destroy(P->rader[i].fwd);
        plan_destroy(P->rader[i].inv);
    }
    free(P->tw);
    free(P);
}

/* kf_factor, kfft_cpx.c:103-143 (system sqrt, as in the SYSMATH build) */
static void factorize(oplan* P) {
    uint32_t p = 4, n = P->nfft;
    uint32_t fsqrt = (uint32_t)sqrt((double)P->nfft);
    do {
        while (n % p) {
            if (p == 4) p = 2;
            else if (p == 2) p = 3;
            else p += 2;
            if (p > fsqrt) p = n;
        }
        if (P->level < OR_PLAN_LEVEL && p > OR_BFLY_LEVEL && p >= OR_RADER_LIMIT) {
            P->rader[P->nrader++].prime = p;
        }
        n /= p;
        P->factors[2 * P->nfac] = p;
        P->factors[2 * P->nfac + 1] = n;
        P->nfac++;
    } while (n > 1);
}

static oplan* plan_create(uint32_t nfft, uint32_t flags, uint32_t level) {
    oplan* P = (oplan*)calloc(1, sizeof(oplan));
    if (!P) return NULL;
    P->nfft = nfft;
    P->flags = flags;
    P->level = level;
    if (nfft == 0) return P;
    factorize(P);
    int inverse = (flags & OR_FLAG_INVERSE) != 0;
    P->tw = (ocpx*)malloc(sizeof(ocpx) * nfft);
    if (!P->tw) {
        plan_destroy(P);
        return NULL;
    }
    for (uint32_t i = 0; i < nfft; i++) P->tw[i] = twiddle(i, nfft, inverse);

    if (flags & OR_FLAG_GENERIC_ONLY) return P;
    /* kfft_kinit Rader part, kfft_cpx.c:165-212 */
    for (uint32_t r = 0; r < P->nrader; r++) {
        orader* R = &P->rader[r];
        uint32_t len = R->prime - 1;
        uint32_t g = primitive_root(R->prime);
        uint32_t ginv = modpow(g, R->prime - 2, R->prime);
        R->qidx = (uint32_t*)malloc(sizeof(uint32_t) * len);
        R->pidx = (uint32_t*)malloc(sizeof(uint32_t) * len);
        R->shuffle = (ocpx*)malloc(sizeof(ocpx) * len);
        uint32_t subflags = flags & ~(uint32_t)(OR_FLAG_RENEW);
        R->fwd = plan_create(len, subflags & ~(uint32_t)OR_FLAG_INVERSE, level + 1);
        R->inv = plan_create(len, subflags | OR_FLAG_INVERSE, level + 1);
        if (!R->qidx || !R->pidx || !R->shuffle || !R->fwd || !R->inv) {
            plan_destroy(P);
            return NULL;
        }
        for (uint32_t i = 0; i < len; i++) {
            R->qidx[i] = modpow(g, i, R->prime);
            R->pidx[i] = modpow(ginv, i, R->prime);
        }
        ocpx* tmp = (ocpx*)malloc(sizeof(ocpx) * len);
        if (!tmp) {
            plan_destroy(P);
            return NULL;
        }
        for (uint32_t j = 0; j < len; j++) tmp[j] = twiddle(R->pidx[j], R->prime, inverse);
        plan_exec(R->fwd, tmp, R->shuffle);
        free(tmp);
    }
    return P;
}

/* kf_bfly2, kfft_bfly.c:1-16 */
static void bfly2(ocpx* F, uint32_t fstride, const oplan* P, uint32_t m) {
    ocpx* F2 = F + m;
    for (uint32_t u = 0; u < m; u++) {
        ocpx t = cmul(F2[u], P->tw[u * fstride]);
        F2[u] = csub(F[u], t);
        F[u] = cadd(F[u], t);
    }
}

/* kf_bfly4, kfft_bfly.c:18-57 */
static void bfly4(ocpx* F, uint32_t fstride, const oplan* P, uint32_t m) {
    int inverse = (P->flags & OR_FLAG_INVERSE) != 0;
    for (uint32_t u = 0; u < m; u++) {
        ocpx s0 = cmul(F[u + m], P->tw[u * fstride]);
        ocpx s1 = cmul(F[u + 2 * m], P->tw[2 * u * fstride]);
        ocpx s2 = cmul(F[u + 3 * m], P->tw[3 * u * fstride]);
        ocpx s5 = csub(F[u], s1);
        ocpx a = cadd(F[u], s1);
        ocpx s3 = cadd(s0, s2);
        ocpx s4 = csub(s0, s2);
        F[u + 2 * m] = csub(a, s3);
        F[u] = cadd(a, s3);
        if (inverse) {
            F[u + m].r = s5.r - s4.i;
            F[u + m].i = s5.i + s4.r;
            F[u + 3 * m].r = s5.r + s4.i;
            F[u + 3 * m].i = s5.i - s4.r;
        } else {
            F[u + m].r = s5.r + s4.i;
            F[u + m].i = s5.i - s4.r;
            F[u + 3 * m].r = s5.r - s4.i;
            F[u + 3 * m].i = s5.i + s4.r;
        }
    }
}

/* kf_bfly3, kfft_bfly.c:59-95 */
static void bfly3(ocpx* F, uint32_t fstride, const oplan* P, uint32_t m) {
    ocpx e = P->tw[fstride * m]; /* exp(-+2 pi i / 3) */
    for (uint32_t u = 0; u < m; u++) {
        ocpx s1 = cmul(F[u + m], P->tw[u * fstride]);
        ocpx s2 = cmul(F[u + 2 * m], P->tw[2 * u * fstride]);
        ocpx s3 = cadd(s1, s2);
        ocpx s0 = csub(s1, s2);
        ocpx a = {F[u].r - OR_HALF * s3.r, F[u].i - OR_HALF * s3.i};
        s0.r *= e.i;
        s0.i *= e.i;
        F[u] = cadd(F[u], s3);
        F[u + 2 * m].r = a.r + s0.i;
        F[u + 2 * m].i = a.i - s0.r;
        F[u + m].r = a.r - s0.i;
        F[u + m].i = a.i + s0.r;
    }
}

/* kf_bfly5, kfft_bfly.c:97-152 */
static void bfly5(ocpx* F, uint32_t fstride, const oplan* P, uint32_t m) {
    ocpx ya = P->tw[fstride * m], yb = P->tw[2 * fstride * m];
    ocpx* F0 = F;
    ocpx* F1 = F + m;
    ocpx* F2 = F + 2 * m;
    ocpx* F3 = F + 3 * m;
    ocpx* F4 = F + 4 * m;
    for (uint32_t u = 0; u < m; u++) {
        ocpx s0 = F0[u];
        ocpx s1 = cmul(F1[u], P->tw[u * fstride]);
        ocpx s2 = cmul(F2[u], P->tw[2 * u * fstride]);
        ocpx s3 = cmul(F3[u], P->tw[3 * u * fstride]);
        ocpx s4 = cmul(F4[u], P->tw[4 * u * fstride]);
        ocpx s7 = cadd(s1, s4), s10 = csub(s1, s4);
        ocpx s8 = cadd(s2, s3), s9 = csub(s2, s3);
        F0[u].r = s0.r + s7.r + s8.r;
        F0[u].i = s0.i + s7.i + s8.i;
        ocpx s5 = {s0.r + s7.r * ya.r + s8.r * yb.r, s0.i + s7.i * ya.r + s8.i * yb.r};
        ocpx s6 = {s10.i * ya.i + s9.i * yb.i, -s10.r * ya.i - s9.r * yb.i};
        F1[u] = csub(s5, s6);
        F4[u] = cadd(s5, s6);
        ocpx s11 = {s0.r + s7.r * yb.r + s8.r * ya.r, s0.i + s7.i * yb.r + s8.i * ya.r};
        ocpx s12 = {-s10.i * yb.i + s9.i * ya.i, s10.r * yb.i - s9.r * ya.i};
        F2[u] = cadd(s11, s12);
        F3[u] = csub(s11, s12);
    }
}

/* std_method_eval, kfft_generic.c:9-36 */
static void bfly_std(ocpx* F, ocpx* tmp, uint32_t fstride, const oplan* P, uint32_t u, uint32_t m,
                     uint32_t p) {
    for (uint32_t q = 0; q < p; q++) tmp[q] = F[u + q * m];
    for (uint32_t q1 = 0; q1 < p; q1++) {
        uint32_t k = u + q1 * m;
        uint64_t step = ((uint64_t)fstride * k) % P->nfft;
        uint64_t tw = 0;
        ocpx acc = tmp[0];
        for (uint32_t q = 1; q < p; q++) {
            tw += step;
            if (tw >= P->nfft) tw -= P->nfft;
            acc = cadd(acc, cmul(tmp[q], P->tw[tw]));
        }
        F[k] = acc;
    }
}

/* rader_method_eval + kfft_part_convolution, kfft_rader.c:1-63 */
static int bfly_rader(ocpx* F, ocpx* tmp, const oplan* P, uint32_t p) {
    const orader* R = NULL;
    for (uint32_t i = 0; i < P->nrader; i++)
        if (P->rader[i].prime == p) {
            R = &P->rader[i];
            break;
        }
    if (!R) return OR_RET_BADARGUMENTS;
    ocpx x0 = F[0];
    ocpx sum = {0.0, 0.0};
    for (uint32_t q = 1; q < p; q++) {
        tmp[q] = F[R->qidx[q - 1]];
        sum = cadd(sum, F[q]);
    }
    uint32_t len = p - 1;
    ocpx* buf = (ocpx*)malloc(sizeof(ocpx) * len);
    if (!buf) return OR_RET_BUFFER_FAIL;
    int ret = plan_exec(R->fwd, tmp + 1, buf);
    if (ret == OR_RET_SUCCESS) {
        for (uint32_t i = 0; i < len; i++) buf[i] = cmul(buf[i], R->shuffle[i]);
        ret = plan_exec(R->inv, buf, tmp + 1);
    }
    free(buf);
    if (ret != OR_RET_SUCCESS) return ret;
    F[0] = cadd(x0, sum);
    for (uint32_t q = 1; q < p; q++) F[R->pidx[q - 1]] = cadd(tmp[q], x0);
    return OR_RET_SUCCESS;
}

/* kf_bfly_generic, kfft_generic.c:38-80 */
static int bfly_generic(ocpx* F, uint32_t fstride, const oplan* P, uint32_t m, uint32_t p) {
    ocpx* tmp = (ocpx*)malloc(sizeof(ocpx) * p);
    if (!tmp) return OR_RET_BUFFER_FAIL;
    int ret = OR_RET_SUCCESS;
    int use_rader = (m == 1) && (p >= OR_RADER_LIMIT) &&
                    !(P->flags & (OR_FLAG_GENERIC | OR_FLAG_GENERIC_ONLY)) && P->nrader;
    for (uint32_t u = 0; u < m && ret == OR_RET_SUCCESS; u++) {
        if (use_rader)
            ret = bfly_rader(F, tmp, P, p);
        else
            bfly_std(F, tmp, fstride, P, u, m, p);
    }
    free(tmp);
    return ret;
}

/* kf_work, kfft_work.c:1-59 */
static int work(ocpx* out, const ocpx* in, uint32_t fstride, const uint32_t* fac, const oplan* P) {
    uint32_t p = fac[0], m = fac[1];
    if (m == 1) {
        for (uint32_t q = 0; q < p; q++) out[q] = in[(size_t)q * fstride];
    } else {
        for (uint32_t q = 0; q < p; q++) {
            int r = work(out + (size_t)q * m, in + (size_t)q * fstride, fstride * p, fac + 2, P);
            if (r != OR_RET_SUCCESS) return r;
        }
    }
    switch (p) {
    case 2: bfly2(out, fstride, P, m); break;
    case 3: bfly3(out, fstride, P, m); break;
    case 4: bfly4(out, fstride, P, m); break;
    case 5: bfly5(out, fstride, P, m); break;
    default: return bfly_generic(out, fstride, P, m, p);
    }
    return OR_RET_SUCCESS;
}

/* kfft_eval_cpx, kfft_cpx.c:321-366 */
static int plan_exec(const oplan* P, const ocpx* in, ocpx* out) {
    if (P->nfft == 0) return OR_RET_SUCCESS;
    int ret;
    if (P->flags & OR_FLAG_GENERIC_ONLY) {
        if (in != out) memcpy(out, in, sizeof(ocpx) * P->nfft);
        ret = bfly_generic(out, 1, P, 1, P->nfft);
    } else if (in == out) {
        ocpx* tmp = (ocpx*)malloc(sizeof(ocpx) * P->nfft);
        if (!tmp) return OR_RET_BUFFER_FAIL;
        ret = work(tmp, in, 1, P->factors, P);
        if (ret == OR_RET_SUCCESS) memcpy(out, tmp, sizeof(ocpx) * P->nfft);
        free(tmp);
    } else {
        ret = work(out, in, 1, P->factors, P);
    }
    if (ret == OR_RET_SUCCESS && (P->flags & OR_FLAG_INVERSE)) {
        if (P->level > 0 || !(P->flags & OR_FLAG_DISABLE_NORM)) {
            for (uint32_t i = 0; i < P->nfft; i++) {
                out[i].r = out[i].r / (oreal)P->nfft;
                out[i].i = out[i].i / (oreal)P->nfft;
            }
        }
    }
    return ret;
}

/* ------------------------------------------------------------------------- */
/* public oracle API                                                         */
/* ------------------------------------------------------------------------- */
void* oracle_plan_cpx(uint32_t nfft, uint32_t flags) {
    return plan_create(nfft, flags & ~(uint32_t)OR_FLAG_RENEW, 0);
}
void oracle_plan_free(void* plan) { plan_destroy((oplan*)plan); }

int oracle_exec_cpx(const void* plan, const ocpx* in, ocpx* out) {
    return plan_exec((const oplan*)plan, in, out);
}

static int resolve_threads(int threads) {
#ifdef _OPENMP
    return threads > 0 ? threads : omp_get_max_threads();
#else
    (void)threads;
    return 1;
#endif
}

/* Host-loop batch over one shared plan, the pattern of ext/2d/kfft_cpx2.c:100-104. */
int oracle_exec_cpx_batch(const void* plan, const ocpx* in, ocpx* out, uint64_t batch,
                          int threads) {
    const oplan* P = (const oplan*)plan;
    int ret = OR_RET_SUCCESS;
    int nt = resolve_threads(threads);
    (void)nt;
#pragma omp parallel for schedule(static) num_threads(nt) reduction(| : ret)
    for (int64_t b = 0; b < (int64_t)batch; b++)
        ret |= plan_exec(P, in + (size_t)b * P->nfft, out + (size_t)b * P->nfft);
    return ret;
}

/* Uneven batch: sequences of lengths[i] packed back to back, one plan per
 * distinct length built once, OpenMP over sequences at execution (the
 * host-loop pattern of ext/2d/kfft_cpx2.c:100-104 applied to a list of
 * lengths). */
typedef struct {
    uint32_t count;
    uint64_t* off;
    oplan** plans; /* per sequence; equal lengths share one plan */
    uint8_t* owner;
} ouneven;

void* oracle_uneven_create(uint32_t count, const uint32_t* lengths, uint32_t flags) {
    ouneven* U = (ouneven*)calloc(1, sizeof(ouneven));
    if (!U) return NULL;
    U->count = count;
    U->off = (uint64_t*)malloc(sizeof(uint64_t) * (count + 1));
    U->plans = (oplan**)calloc(count ? count : 1, sizeof(oplan*));
    U->owner = (uint8_t*)calloc(count ? count : 1, 1);
    if (!U->off || !U->plans || !U->owner) {
        oracle_uneven_free(U);
        return NULL;
    }
    U->off[0] = 0;
    for (uint32_t i = 0; i < count; i++) U->off[i + 1] = U->off[i] + lengths[i];
    for (uint32_t i = 0; i < count; i++) {
        for (uint32_t j = 0; j < i; j++)
            if (lengths[j] == lengths[i]) {
                U->plans[i] = U->plans[j];
                break;
            }
        if (!U->plans[i]) {
            U->plans[i] = (oplan*)oracle_plan_cpx(lengths[i], flags);
            U->owner[i] = 1;
            if (!U->plans[i]) {
                oracle_uneven_free(U);
                return NULL;
            }
        }
    }
    return U;
}

int oracle_uneven_exec(const void* u, const ocpx* in, ocpx* out, int threads) {
    const ouneven* U = (const ouneven*)u;
    int ret = OR_RET_SUCCESS;
    int nt = resolve_threads(threads);
    (void)nt;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt) reduction(| : ret)
    for (int64_t i = 0; i < (int64_t)U->count; i++)
        ret |= plan_exec(U->plans[i], in + U->off[i], out + U->off[i]);
    return ret;
}

void oracle_uneven_free(void* u) {
    ouneven* U = (ouneven*)u;
    if (!U) return;
    if (U->plans && U->owner)
        for (uint32_t i = 0; i < U->count; i++)
            if (U->owner[i]) plan_destroy(U->plans[i]);
    free(U->plans);
    free(U->owner);
    free(U->off);
    free(U);
}

int oracle_exec_uneven(uint32_t count, const uint32_t* lengths, uint32_t flags, const ocpx* in,
                       ocpx* out, int threads) {
    void* U = oracle_uneven_create(count, lengths, flags);
    if (!U) return OR_RET_ALLOC_FAIL;
    int r = oracle_uneven_exec(U, in, out, threads);
    oracle_uneven_free(U);
    return r;
}

int oracle_fft_cpx(uint32_t nfft, uint32_t flags, const ocpx* in, ocpx* out) {
    oplan* P = (oplan*)oracle_plan_cpx(nfft, flags);
    if (!P) return OR_RET_ALLOC_FAIL;
    int r = plan_exec(P, in, out);
    plan_destroy(P);
    return r;
}

/* ---- real ("scalar") transform, kfft_scalar.c ---------------------------- */
/* kfft_sclr_twiddle, kfft_scalar.c:9-18 */
static ocpx super_twiddle(uint32_t i, uint32_t half, int inverse) {
    double phase = -OR_PI * ((double)(i + 1) / (double)half + 0.5);
    if (inverse) phase = -phase;
    ocpx r = {(oreal)cos(phase), (oreal)sin(phase)};
    return r;
}

int oracle_rfft(uint32_t nfft, uint32_t flags, const oreal* in, ocpx* out) {
    if (flags & OR_FLAG_INVERSE) return OR_RET_IMPROPER_PLAN;
    if (nfft == 0) return OR_RET_SUCCESS;
    uint32_t cflags = flags & ~(uint32_t)OR_FLAG_RENEW;
    if (nfft % 2) { /* eval_trivial, kfft_scalar.c:78-98 */
        ocpx* buf = (ocpx*)calloc(nfft, sizeof(ocpx));
        if (!buf) return OR_RET_BUFFER_FAIL;
        for (uint32_t i = 0; i < nfft; i++) buf[i].r = in[i];
        int r = oracle_fft_cpx(nfft, cflags, buf, out);
        free(buf);
        return r;
    }
    /* eval_nyquist + rebuild_forward, kfft_scalar.c:174-216, 244-266 */
    uint32_t h = nfft / 2;
    ocpx* z = (ocpx*)calloc(h + 1, sizeof(ocpx));
    if (!z) return OR_RET_BUFFER_FAIL;
    int r = oracle_fft_cpx(h, cflags, (const ocpx*)in, z);
    if (r != OR_RET_SUCCESS) {
        free(z);
        return r;
    }
    out[0].r = z[0].r + z[0].i;
    out[h].r = z[0].r - z[0].i;
    out[0].i = out[h].i = 0.0;
    for (uint32_t k = 1; k <= h / 2; k++) {
        ocpx fpk = z[k];
        ocpx fpnk = {z[h - k].r, -z[h - k].i};
        ocpx f1k = cadd(fpk, fpnk), f2k = csub(fpk, fpnk);
        ocpx tw = cmul(f2k, super_twiddle(k - 1, h, 0));
        out[k].r = OR_HALF * (f1k.r + tw.r);
        out[k].i = OR_HALF * (f1k.i + tw.i);
        out[h - k].r = OR_HALF * (f1k.r - tw.r);
        out[h - k].i = OR_HALF * (tw.i - f1k.i);
    }
    if (flags & OR_FLAG_EXPAND_SCALAR)
        for (uint32_t k = 1; k < nfft; k++) {
            out[nfft - k].r = out[k].r;
            out[nfft - k].i = -out[k].i;
        }
    free(z);
    return OR_RET_SUCCESS;
}

int oracle_irfft(uint32_t nfft, uint32_t flags, const ocpx* in, oreal* out) {
    if (!(flags & OR_FLAG_INVERSE)) return OR_RET_IMPROPER_PLAN;
    if (nfft == 0) return OR_RET_SUCCESS;
    uint32_t cflags = flags & ~(uint32_t)OR_FLAG_RENEW;
    if (nfft % 2) { /* evali_trivial, kfft_scalar.c:100-118 */
        ocpx* buf = (ocpx*)malloc(sizeof(ocpx) * nfft);
        if (!buf) return OR_RET_BUFFER_FAIL;
        int r = oracle_fft_cpx(nfft, cflags, in, buf);
        for (uint32_t i = 0; i < nfft; i++) out[i] = buf[i].r;
        free(buf);
        return r;
    }
    /* rebuild_inverse + evali_nyquist, kfft_scalar.c:218-242, 268-289 */
    uint32_t h = nfft / 2;
    ocpx* f = (ocpx*)calloc(h + 1, sizeof(ocpx));
    if (!f) return OR_RET_BUFFER_FAIL;
    f[0].r = in[0].r + in[h].r;
    f[0].i = in[0].r - in[h].r;
    for (uint32_t k = 1; k <= h / 2; k++) {
        ocpx fk = in[k];
        ocpx fnkc = {in[h - k].r, -in[h - k].i};
        ocpx fek = cadd(fk, fnkc), t = csub(fk, fnkc);
        ocpx fok = cmul(t, super_twiddle(k - 1, h, 1));
        f[k] = cadd(fek, fok);
        f[h - k] = csub(fek, fok);
        f[h - k].i = -f[h - k].i;
    }
    int r = oracle_fft_cpx(h, cflags, f, (ocpx*)out);
    free(f);
    return r;
}

/* ---- 2D, ext/2d ------------------------------------------------------------ */
/* column transform helper: columns of a (rows x cols) row-major complex array */
static int columns_cpx(uint32_t rows, uint32_t cols, uint32_t flags, ocpx* data) {
    oplan* P = (oplan*)oracle_plan_cpx(rows, flags);
    if (!P) return OR_RET_ALLOC_FAIL;
    int ret = OR_RET_SUCCESS;
#pragma omp parallel
    {
        ocpx* a = (ocpx*)malloc(sizeof(ocpx) * rows);
        ocpx* b = (ocpx*)malloc(sizeof(ocpx) * rows);
#pragma omp for schedule(static)
        for (int64_t c = 0; c < (int64_t)cols; c++) {
            for (uint32_t r = 0; r < rows; r++) a[r] = data[(size_t)r * cols + c];
            int rr = plan_exec(P, a, b);
            if (rr) {
#pragma omp atomic write
                ret = rr;
            }
            for (uint32_t r = 0; r < rows; r++) data[(size_t)r * cols + c] = b[r];
        }
        free(a);
        free(b);
    }
    plan_destroy(P);
    return ret;
}

/* kfft_eval2_cpx, ext/2d/kfft_cpx2.c:92-186: x = row length (contiguous), y = rows */
int oracle_fft2_cpx(uint32_t x, uint32_t y, uint32_t flags, const ocpx* in, ocpx* out) {
    size_t n = (size_t)x * y;
    if (n == 0) return OR_RET_SUCCESS;
    ocpx* tmp = (ocpx*)malloc(sizeof(ocpx) * n);
    if (!tmp) return OR_RET_BUFFER_FAIL;
    oplan* P = (oplan*)oracle_plan_cpx(x, flags);
    int ret = oracle_exec_cpx_batch(P, in, tmp, y, 0);
    plan_destroy(P);
    if (ret == OR_RET_SUCCESS) ret = columns_cpx(y, x, flags, tmp);
    if (ret == OR_RET_SUCCESS) memcpy(out, tmp, sizeof(ocpx) * n);
    free(tmp);
    return ret;
}

/* kfft_eval2_scalar, ext/2d/kfft_scalar2.c:120-150 */
int oracle_rfft2(uint32_t x, uint32_t y, uint32_t flags, const oreal* in, ocpx* out) {
    if (flags & OR_FLAG_INVERSE) return OR_RET_IMPROPER_PLAN;
    size_t n = (size_t)x * y;
    if (n == 0) return OR_RET_SUCCESS;
    uint32_t rflags = (flags & ~(uint32_t)OR_FLAG_RENEW) | OR_FLAG_EXPAND_SCALAR;
    int ret = OR_RET_SUCCESS;
    for (uint32_t r = 0; r < y && ret == OR_RET_SUCCESS; r++)
        ret = oracle_rfft(x, rflags, in + (size_t)r * x, out + (size_t)r * x);
    if (ret == OR_RET_SUCCESS) ret = columns_cpx(y, x, flags & ~(uint32_t)OR_FLAG_RENEW, out);
    return ret;
}

/* kfft_evali2_scalar, ext/2d/kfft_scalar2.c:185-246 */
int oracle_irfft2(uint32_t x, uint32_t y, uint32_t flags, const ocpx* in, oreal* out) {
    if (!(flags & OR_FLAG_INVERSE)) return OR_RET_IMPROPER_PLAN;
    size_t n = (size_t)x * y;
    if (n == 0) return OR_RET_SUCCESS;
    uint32_t cflags = flags & ~(uint32_t)OR_FLAG_RENEW;
    ocpx* rows = (ocpx*)malloc(sizeof(ocpx) * n);
    ocpx* col = (ocpx*)malloc(sizeof(ocpx) * y);
    oreal* colr = (oreal*)malloc(sizeof(oreal) * (y + 2));
    if (!rows || !col || !colr) {
        free(rows);
        free(col);
        free(colr);
        return OR_RET_BUFFER_FAIL;
    }
    oplan* P = (oplan*)oracle_plan_cpx(x, cflags);
    int ret = oracle_exec_cpx_batch(P, in, rows, y, 0);
    plan_destroy(P);
    for (uint32_t c = 0; c < x && ret == OR_RET_SUCCESS; c++) {
        for (uint32_t r = 0; r < y; r++) col[r] = rows[(size_t)r * x + c];
        ret = oracle_irfft(y, cflags | OR_FLAG_EXPAND_SCALAR, col, colr);
        for (uint32_t r = 0; r < y; r++) out[(size_t)r * x + c] = colr[r];
    }
    free(rows);
    free(col);
    free(colr);
    return ret;
}

/* ---- convolution, ext/conv and ext/conv2d ------------------------------------ */
static void hadamard(ocpx* b, const ocpx* a, size_t n) {
    for (size_t i = 0; i < n; i++) b[i] = cmul(b[i], a[i]);
}

/* kfft_eval_conv_cpx, ext/conv/kfft_cpx_conv.c:75-104 */
int oracle_conv_cpx(uint32_t nfft, uint32_t flags, const ocpx* a, const ocpx* b, ocpx* out) {
    uint32_t f = flags & ~(uint32_t)(OR_FLAG_RENEW | OR_FLAG_INVERSE);
    ocpx* A = (ocpx*)malloc(sizeof(ocpx) * (nfft ? nfft : 1));
    ocpx* B = (ocpx*)malloc(sizeof(ocpx) * (nfft ? nfft : 1));
    if (!A || !B) {
        free(A);
        free(B);
        return OR_RET_BUFFER_FAIL;
    }
    int r = oracle_fft_cpx(nfft, f, a, A);
    if (!r) r = oracle_fft_cpx(nfft, f, b, B);
    if (!r) {
        hadamard(B, A, nfft);
        r = oracle_fft_cpx(nfft, f | OR_FLAG_INVERSE, B, out);
    }
    free(A);
    free(B);
    return r;
}

/* kfft_eval_conv_scalar, ext/conv/kfft_scalar_conv.c:74-100 */
int oracle_conv_scalar(uint32_t nfft, uint32_t flags, const oreal* a, const oreal* b,
                       oreal* out) {
    uint32_t f = flags & ~(uint32_t)(OR_FLAG_RENEW | OR_FLAG_INVERSE);
    ocpx* A = (ocpx*)calloc(nfft + 1, sizeof(ocpx));
    ocpx* B = (ocpx*)calloc(nfft + 1, sizeof(ocpx));
    if (!A || !B) {
        free(A);
        free(B);
        return OR_RET_BUFFER_FAIL;
    }
    int r = oracle_rfft(nfft, f, a, A);
    if (!r) r = oracle_rfft(nfft, f, b, B);
    if (!r) {
        hadamard(B, A, nfft);
        r = oracle_irfft(nfft, f | OR_FLAG_INVERSE, B, out);
    }
    free(A);
    free(B);
    return r;
}

/* kfft_eval2_conv_cpx, ext/conv2d/kfft_cpx_conv.c:81-110 */
int oracle_conv2_cpx(uint32_t x, uint32_t y, uint32_t flags, const ocpx* a, const ocpx* b,
                     ocpx* out) {
    size_t n = (size_t)x * y;
    uint32_t f = flags & ~(uint32_t)(OR_FLAG_RENEW | OR_FLAG_INVERSE);
    ocpx* A = (ocpx*)malloc(sizeof(ocpx) * (n ? n : 1));
    ocpx* B = (ocpx*)malloc(sizeof(ocpx) * (n ? n : 1));
    if (!A || !B) {
        free(A);
        free(B);
        return OR_RET_BUFFER_FAIL;
    }
    int r = oracle_fft2_cpx(x, y, f, a, A);
    if (!r) r = oracle_fft2_cpx(x, y, f, b, B);
    if (!r) {
        hadamard(B, A, n);
        r = oracle_fft2_cpx(x, y, f | OR_FLAG_INVERSE, B, out);
    }
    free(A);
    free(B);
    return r;
}

/* kfft_eval2_conv_scalar, ext/conv2d/kfft_scalar_conv.c:79-107 */
int oracle_conv2_scalar(uint32_t x, uint32_t y, uint32_t flags, const oreal* a, const oreal* b,
                        oreal* out) {
    size_t n = (size_t)x * y;
    uint32_t f = flags & ~(uint32_t)(OR_FLAG_RENEW | OR_FLAG_INVERSE);
    ocpx* A = (ocpx*)malloc(sizeof(ocpx) * (n ? n : 1));
    ocpx* B = (ocpx*)malloc(sizeof(ocpx) * (n ? n : 1));
    if (!A || !B) {
        free(A);
        free(B);
        return OR_RET_BUFFER_FAIL;
    }
    int r = oracle_rfft2(x, y, f, a, A);
    if (!r) r = oracle_rfft2(x, y, f, b, B);
    if (!r) {
        hadamard(B, A, n);
        r = oracle_irfft2(x, y, f | OR_FLAG_INVERSE, B, out);
    }
    free(A);
    free(B);
    return r;
}

/* exact O(N^2) DFT with integer phase reduction, a precision cross-check */
int oracle_dft_exact(uint32_t nfft, int inverse, const ocpx* in, ocpx* out) {
    for (uint32_t k = 0; k < nfft; k++) {
        long double sr = 0.0L, si = 0.0L;
        for (uint32_t n = 0; n < nfft; n++) {
            uint64_t ph = ((uint64_t)n * k) % nfft;
            long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)ph /
                            (long double)nfft;
            if (inverse) a = -a;
            long double c = cosl(a), s = sinl(a);
            sr += (long double)in[n].r * c - (long double)in[n].i * s;
            si += (long double)in[n].r * s + (long double)in[n].i * c;
        }
        out[k].r = (oreal)sr;
        out[k].i = (oreal)si;
    }
    return OR_RET_SUCCESS;
}
