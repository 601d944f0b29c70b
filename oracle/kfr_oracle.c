/*
 * kfr_oracle: CPU restatement of KFR 7.0.1's DFT hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * Only the test suite, the smoke check and the CPU-baseline leg of the benchmark load this library, and
 * only as the checker or as the timed CPU baseline; the GPU library never links or calls it.
 *
 * The f64 entry points are the parity reference for every GPU result.  The f32 entry points run the
 * same algorithm in single precision and are the CPU baseline ("port") timed beside the GPU.  Batches
 * are split over POSIX threads, one signal at a time, with one shared read-only plan and a private
 * scratch buffer per thread (the reference's own threading contract: execute is const,
 * include/kfr/dft/fft.hpp:265-272).
 *
 * Algorithms and the reference lines they follow are listed in oracle_core.h.
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define REAL double
#define SFX _f64
#include "oracle_core.h"
#undef REAL
#undef SFX
#undef FN

#define REAL float
#define SFX _f32
#include "oracle_core.h"
#undef REAL
#undef SFX
#undef FN

#define EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------------------------------ */
/* Thread pool helper: run fn(ctx, i) for i in [0, count) over `threads` POSIX threads.              */
/* ------------------------------------------------------------------------------------------------ */

typedef void (*orc_job_fn)(void* ctx, size_t begin, size_t end);

typedef struct
{
    orc_job_fn fn;
    void* ctx;
    size_t begin, end;
} orc_job;

static void* orc_job_entry(void* arg)
{
    orc_job* j = (orc_job*)arg;
    j->fn(j->ctx, j->begin, j->end);
    return NULL;
}

static void orc_parallel(orc_job_fn fn, void* ctx, size_t count, int threads)
{
    if (threads < 1)
        threads = 1;
    if ((size_t)threads > count)
        threads = (int)(count ? count : 1);
    if (threads == 1)
    {
        fn(ctx, 0, count);
        return;
    }
    pthread_t tids[256];
    orc_job jobs[256];
    if (threads > 256)
        threads = 256;
    for (int t = 0; t < threads; t++)
    {
        jobs[t].fn    = fn;
        jobs[t].ctx   = ctx;
        jobs[t].begin = count * (size_t)t / (size_t)threads;
        jobs[t].end   = count * (size_t)(t + 1) / (size_t)threads;
        pthread_create(&tids[t], NULL, orc_job_entry, &jobs[t]);
    }
    for (int t = 0; t < threads; t++)
        pthread_join(tids[t], NULL);
}

/* ------------------------------------------------------------------------------------------------ */
/* Precision-generic API, instantiated for f64 and f32 below.                                        */
/* ------------------------------------------------------------------------------------------------ */

#define ORC_API(REALT, SFXT)                                                                             \
    typedef struct                                                                                       \
    {                                                                                                    \
        const ORC_CAT(orc_plan, SFXT) * plan;                                                            \
        ORC_CAT(cpx, SFXT) * out;                                                                        \
        const ORC_CAT(cpx, SFXT) * in;                                                                   \
        size_t n, ostride, istride;                                                                      \
        int inverse, kind, ccs;                                                                          \
    } ORC_CAT(orc_ctx, SFXT);                                                                            \
                                                                                                         \
    /* kind 0: complex DFT; 1: real forward; 2: real inverse; 3: DCT-II; 4: DCT-III */                   \
    static void ORC_CAT(orc_worker, SFXT)(void* vctx, size_t b0, size_t b1)                              \
    {                                                                                                    \
        typedef ORC_CAT(cpx, SFXT) C;                                                                    \
        ORC_CAT(orc_ctx, SFXT)* c = (ORC_CAT(orc_ctx, SFXT)*)vctx;                                       \
        const size_t ps           = ORC_CAT(plan_scratch, SFXT)(c->plan);                                \
        const size_t n            = c->n;                                                                \
        C* scratch                = (C*)malloc(sizeof(C) * (ps + 6 * n + 16));                           \
        C* t1                     = scratch + ps + n + 2;                                                \
        C* t2                     = t1 + n + 2;                                                          \
        for (size_t b = b0; b < b1; b++)                                                                 \
        {                                                                                                \
            C* out      = c->out + b * c->ostride;                                                       \
            const C* in = c->in + b * c->istride;                                                        \
            if (c->kind == 0)                                                                            \
                ORC_CAT(dft_one, SFXT)(c->plan, out, in, c->inverse, scratch);                           \
            else if (c->kind == 1)                                                                       \
            {                                                                                            \
                /* real forward: in holds n/2 complex (the n reals) */                                   \
                ORC_CAT(execute_plan, SFXT)(c->plan, t1, in, scratch);                                   \
                ORC_CAT(real_repack_fwd, SFXT)(2 * c->plan->n, out, t1, c->ccs);                         \
            }                                                                                            \
            else if (c->kind == 2)                                                                       \
            {                                                                                            \
                ORC_CAT(real_repack_inv, SFXT)(2 * c->plan->n, t1, in, c->ccs);                          \
                ORC_CAT(dft_one, SFXT)(c->plan, out, t1, 1, scratch);                                    \
            }                                                                                            \
            else                                                                                         \
            {                                                                                            \
                /* DCT (include/kfr/dft/fft.hpp:932-970); in/out hold n reals in .re/.im pairs */        \
                const REALT* rin = (const REALT*)in;                                                     \
                REALT* rout      = (REALT*)out;                                                          \
                const size_t N = n, half = n / 2;                                                        \
                if (c->kind == 3)                                                                        \
                {                                                                                        \
                    for (size_t i = 0; i < half; i++)                                                    \
                    {                                                                                    \
                        t1[i]         = ORC_CAT(cmk, SFXT)(rin[2 * i], 0);                               \
                        t1[N - 1 - i] = ORC_CAT(cmk, SFXT)(rin[2 * i + 1], 0);                           \
                    }                                                                                    \
                    if (N % 2)                                                                           \
                        t1[half] = ORC_CAT(cmk, SFXT)(rin[N - 1], 0);                                    \
                    ORC_CAT(execute_plan, SFXT)(c->plan, t2, t1, scratch);                               \
                    for (size_t k = 0; k < N; k++)                                                       \
                    {                                                                                    \
                        const double t = (double)k * M_PI / (double)(2 * N);                             \
                        rout[k] = (REALT)((double)t2[k].re * cos(t) + (double)t2[k].im * sin(t));        \
                    }                                                                                    \
                }                                                                                        \
                else                                                                                     \
                {                                                                                        \
                    for (size_t k = 0; k < N; k++)                                                       \
                    {                                                                                    \
                        const double t = (double)k * M_PI / (double)(2 * N);                             \
                        t1[k] = ORC_CAT(cmk, SFXT)((REALT)(rin[k] * cos(t)), (REALT)(rin[k] * -sin(t))); \
                    }                                                                                    \
                    t1[0] = ORC_CAT(cscale, SFXT)(t1[0], (REALT)0.5);                                    \
                    ORC_CAT(execute_plan, SFXT)(c->plan, t2, t1, scratch);                               \
                    for (size_t i = 0; i < half; i++)                                                    \
                    {                                                                                    \
                        rout[2 * i]     = t2[i].re;                                                      \
                        rout[2 * i + 1] = t2[N - 1 - i].re;                                              \
                    }                                                                                    \
                    if (N % 2)                                                                           \
                        rout[N - 1] = t2[half].re;                                                       \
                }                                                                                        \
            }                                                                                            \
        }                                                                                                \
        free(scratch);                                                                                   \
    }                                                                                                    \
                                                                                                         \
    static int ORC_CAT(orc_run, SFXT)(int kind, void* out, const void* in, size_t n, size_t plan_n,      \
                                      size_t ostride, size_t istride, size_t batch, int inverse, int ccs, \
                                      int threads)                                                       \
    {                                                                                                    \
        ORC_CAT(orc_ctx, SFXT) c;                                                                        \
        ORC_CAT(orc_plan, SFXT)* p = ORC_CAT(plan_create, SFXT)(plan_n);                                 \
        c.plan                     = p;                                                                  \
        c.out                      = (ORC_CAT(cpx, SFXT)*)out;                                           \
        c.in                       = (const ORC_CAT(cpx, SFXT)*)in;                                      \
        c.n                        = n;                                                                  \
        c.ostride                  = ostride;                                                            \
        c.istride                  = istride;                                                            \
        c.inverse                  = inverse;                                                            \
        c.kind                     = kind;                                                               \
        c.ccs                      = ccs;                                                                \
        orc_parallel(ORC_CAT(orc_worker, SFXT), &c, batch, threads);                                     \
        ORC_CAT(plan_free, SFXT)(p);                                                                     \
        return 0;                                                                                        \
    }                                                                                                    \
                                                                                                         \
    /* complex DFT of `batch` contiguous signals of n complex values (interleaved re, im) */             \
    EXPORT int ORC_CAT(orc_dft, SFXT)(REALT * out, const REALT* in, size_t n, size_t batch, int inverse, \
                                      int threads)                                                       \
    {                                                                                                    \
        if (n == 0)                                                                                      \
            return 0;                                                                                    \
        return ORC_CAT(orc_run, SFXT)(0, out, in, n, n, n, n, batch, inverse, 0, threads);               \
    }                                                                                                    \
    /* real forward DFT (dft_plan_real): n reals -> n/2+1 (ccs) or n/2 (perm) complex per signal */      \
    EXPORT int ORC_CAT(orc_dft_real, SFXT)(REALT * out, const REALT* in, size_t n, int ccs, size_t batch, \
                                           int threads)                                                  \
    {                                                                                                    \
        if (n == 0 || n % 2)                                                                             \
            return -1;                                                                                   \
        return ORC_CAT(orc_run, SFXT)(1, out, in, n / 2, n / 2, ccs ? n / 2 + 1 : n / 2, n / 2, batch, 0, \
                                      ccs, threads);                                                     \
    }                                                                                                    \
    /* real inverse DFT: n/2+1 (ccs) or n/2 (perm) complex -> n reals per signal, unscaled */            \
    EXPORT int ORC_CAT(orc_dft_real_inverse, SFXT)(REALT * out, const REALT* in, size_t n, int ccs,      \
                                                   size_t batch, int threads)                            \
    {                                                                                                    \
        if (n == 0 || n % 2)                                                                             \
            return -1;                                                                                   \
        return ORC_CAT(orc_run, SFXT)(2, out, in, n / 2, n / 2, n / 2, ccs ? n / 2 + 1 : n / 2, batch, 1, \
                                      ccs, threads);                                                     \
    }                                                                                                    \
    /* DCT-II (inverse=0) or DCT-III with X0/2 (inverse=1), n reals per signal, unscaled.              */ \
    /* Reals are addressed through the complex stride, so signals are packed two reals per complex:    */ \
    /* the caller passes contiguous reals and we convert strides here.                                 */ \
    EXPORT int ORC_CAT(orc_dct, SFXT)(REALT * out, const REALT* in, size_t n, int inverse, size_t batch, \
                                      int threads)                                                       \
    {                                                                                                    \
        if (n == 0)                                                                                      \
            return 0;                                                                                    \
        int rc = 0;                                                                                      \
        if (n % 2 == 0)                                                                                  \
            rc = ORC_CAT(orc_run, SFXT)(inverse ? 4 : 3, out, in, n, n, n / 2, n / 2, batch, 0, 0,       \
                                        threads);                                                        \
        else                                                                                             \
            for (size_t b = 0; b < batch && rc == 0; b++)                                                \
                rc = ORC_CAT(orc_run, SFXT)(inverse ? 4 : 3, out + b * n, in + b * n, n, n, 0, 0, 1, 0,  \
                                            0, 1);                                                       \
        return rc;                                                                                       \
    }                                                                                                    \
    /* convolve / correlate (src/dft/convolution-impl.cpp:106-128).  Real (is_complex=0) or complex    */ \
    /* inputs; returns the output length n1+n2-1.                                                      */ \
    EXPORT size_t ORC_CAT(orc_convolve, SFXT)(REALT * out, const REALT* a, size_t na, const REALT* b,    \
                                              size_t nb, int correlate, int is_complex)                  \
    {                                                                                                    \
        typedef ORC_CAT(cpx, SFXT) C;                                                                    \
        if (na == 0 || nb == 0)                                                                          \
            return 0;                                                                                    \
        const size_t olen = na + nb - 1;                                                                 \
        const size_t size = ORC_CAT(next_pow2, SFXT)(olen);                                              \
        C* p1             = (C*)calloc(size, sizeof(C));                                                 \
        C* p2             = (C*)calloc(size, sizeof(C));                                                 \
        for (size_t i = 0; i < na; i++)                                                                  \
            p1[i] = is_complex ? ORC_CAT(cmk, SFXT)(a[2 * i], a[2 * i + 1]) : ORC_CAT(cmk, SFXT)(a[i], 0); \
        for (size_t i = 0; i < nb; i++)                                                                  \
        {                                                                                                \
            const size_t j = correlate ? nb - 1 - i : i;                                                 \
            p2[j] = is_complex ? ORC_CAT(cmk, SFXT)(b[2 * i], b[2 * i + 1]) : ORC_CAT(cmk, SFXT)(b[i], 0); \
        }                                                                                                \
        ORC_CAT(orc_plan, SFXT)* p = ORC_CAT(plan_create, SFXT)(size);                                   \
        C* scratch = (C*)malloc(sizeof(C) * (ORC_CAT(plan_scratch, SFXT)(p) + size + 4));                \
        ORC_CAT(dft_one, SFXT)(p, p1, p1, 0, scratch);                                                   \
        ORC_CAT(dft_one, SFXT)(p, p2, p2, 0, scratch);                                                   \
        for (size_t i = 0; i < size; i++)                                                                \
            p1[i] = ORC_CAT(cmul, SFXT)(p1[i], p2[i]);                                                   \
        ORC_CAT(dft_one, SFXT)(p, p1, p1, 1, scratch);                                                   \
        const REALT inv = (REALT)1 / (REALT)size;                                                        \
        for (size_t i = 0; i < olen; i++)                                                                \
        {                                                                                                \
            if (is_complex)                                                                              \
            {                                                                                            \
                /* the reference keeps only the real part for complex inputs too:                      */ \
                /* truncate(real(src1padded), ...) at src/dft/convolution-impl.cpp:127                 */ \
                out[2 * i]     = p1[i].re * inv;                                                         \
                out[2 * i + 1] = 0;                                                                      \
            }                                                                                            \
            else                                                                                         \
                out[i] = p1[i].re * inv;                                                                 \
        }                                                                                                \
        free(scratch);                                                                                   \
        ORC_CAT(plan_free, SFXT)(p);                                                                     \
        free(p1);                                                                                        \
        free(p2);                                                                                        \
        return olen;                                                                                     \
    }                                                                                                    \
    /* convolve_filter: streaming object (real or complex samples) */                                   \
    EXPORT void* ORC_CAT(orc_filter_create, SFXT)(const REALT* taps, size_t ntaps, size_t block,         \
                                                  int is_complex)                                        \
    {                                                                                                    \
        typedef ORC_CAT(cpx, SFXT) C;                                                                    \
        C* t = (C*)calloc(ntaps + 1, sizeof(C));                                                         \
        for (size_t i = 0; i < ntaps; i++)                                                               \
            t[i] = is_complex ? ORC_CAT(cmk, SFXT)(taps[2 * i], taps[2 * i + 1])                         \
                              : ORC_CAT(cmk, SFXT)(taps[i], 0);                                          \
        void* f = ORC_CAT(filt_create, SFXT)(t, ntaps, block, is_complex);                               \
        free(t);                                                                                         \
        return f;                                                                                        \
    }                                                                                                    \
    EXPORT void ORC_CAT(orc_filter_process, SFXT)(void* vf, REALT* out, const REALT* in, size_t n)       \
    {                                                                                                    \
        typedef ORC_CAT(cpx, SFXT) C;                                                                    \
        ORC_CAT(orc_filter, SFXT)* f = (ORC_CAT(orc_filter, SFXT)*)vf;                                   \
        if (f->is_complex)                                                                               \
        {                                                                                                \
            ORC_CAT(filt_process, SFXT)(f, (C*)out, (const C*)in, n);                                    \
            return;                                                                                      \
        }                                                                                                \
        C* ci = (C*)calloc(n + 1, sizeof(C));                                                            \
        C* co = (C*)calloc(n + 1, sizeof(C));                                                            \
        for (size_t i = 0; i < n; i++)                                                                   \
            ci[i] = ORC_CAT(cmk, SFXT)(in[i], 0);                                                        \
        ORC_CAT(filt_process, SFXT)(f, co, ci, n);                                                       \
        for (size_t i = 0; i < n; i++)                                                                   \
            out[i] = co[i].re;                                                                           \
        free(ci);                                                                                        \
        free(co);                                                                                        \
    }                                                                                                    \
    EXPORT void ORC_CAT(orc_filter_reset, SFXT)(void* f)                                                 \
    {                                                                                                    \
        ORC_CAT(filt_reset, SFXT)((ORC_CAT(orc_filter, SFXT)*)f);                                        \
    }                                                                                                    \
    EXPORT void ORC_CAT(orc_filter_delete, SFXT)(void* f)                                                \
    {                                                                                                    \
        ORC_CAT(filt_free, SFXT)((ORC_CAT(orc_filter, SFXT)*)f);                                         \
    }                                                                                                    \
    /* fir_filter: direct-form streaming FIR (real samples) */                                          \
    EXPORT void* ORC_CAT(orc_fir_create, SFXT)(const REALT* taps, size_t ntaps)                          \
    {                                                                                                    \
        return ORC_CAT(fir_create, SFXT)(taps, ntaps);                                                   \
    }                                                                                                    \
    EXPORT void ORC_CAT(orc_fir_process, SFXT)(void* f, REALT* out, const REALT* in, size_t n)           \
    {                                                                                                    \
        ORC_CAT(fir_process, SFXT)((ORC_CAT(orc_fir, SFXT)*)f, out, in, n);                              \
    }                                                                                                    \
    EXPORT void ORC_CAT(orc_fir_reset, SFXT)(void* f) { ORC_CAT(fir_reset, SFXT)((ORC_CAT(orc_fir, SFXT)*)f); } \
    EXPORT void ORC_CAT(orc_fir_delete, SFXT)(void* f) { ORC_CAT(fir_free, SFXT)((ORC_CAT(orc_fir, SFXT)*)f); } \
    /* fft_multiply (acc NULL) / three-operand fft_multiply_accumulate over n complex values */          \
    EXPORT void ORC_CAT(orc_fft_multiply, SFXT)(REALT * dst, const REALT* acc, const REALT* a,           \
                                                const REALT* b, size_t n, int perm)                      \
    {                                                                                                    \
        typedef ORC_CAT(cpx, SFXT) C;                                                                    \
        if (acc)                                                                                         \
            ORC_CAT(fft_mac3, SFXT)((C*)dst, (const C*)acc, (const C*)a, (const C*)b, n, perm);          \
        else                                                                                             \
            ORC_CAT(fft_mul, SFXT)((C*)dst, (const C*)a, (const C*)b, n, perm);                          \
    }                                                                                                    \
    /* plan description for tests: returns number of passes (0 for Bluestein), fills radices */         \
    EXPORT int ORC_CAT(orc_plan_info, SFXT)(size_t n, int* radices, int max_radices, size_t* bluestein_m) \
    {                                                                                                    \
        ORC_CAT(orc_plan, SFXT)* p = ORC_CAT(plan_create, SFXT)(n);                                      \
        int np                     = p->npasses;                                                         \
        for (int i = 0; i < np && i < max_radices; i++)                                                  \
            radices[i] = p->radix[i];                                                                    \
        *bluestein_m = p->bluestein ? p->m : 0;                                                          \
        ORC_CAT(plan_free, SFXT)(p);                                                                     \
        return np;                                                                                       \
    }

ORC_API(double, _f64)
ORC_API(float, _f32)

/* Streaming filter over a batch of independent channels that share one tap set (each channel gets its
 * own filter state), split over threads: the CPU baseline for batched FFT convolution. */
typedef struct
{
    const float* taps;
    size_t ntaps, block, len;
    float* out;
    const float* in;
} orc_fbatch_ctx;

static void orc_fbatch_worker(void* vctx, size_t b0, size_t b1)
{
    orc_fbatch_ctx* c = (orc_fbatch_ctx*)vctx;
    void* f           = orc_filter_create_f32(c->taps, c->ntaps, c->block, 0);
    for (size_t b = b0; b < b1; b++)
    {
        orc_filter_reset_f32(f);
        orc_filter_process_f32(f, c->out + b * c->len, c->in + b * c->len, c->len);
    }
    orc_filter_delete_f32(f);
}

EXPORT void orc_filter_batch_f32(float* out, const float* in, size_t len, size_t channels, const float* taps,
                                 size_t ntaps, size_t block, int threads)
{
    orc_fbatch_ctx c = { taps, ntaps, block, len, out, in };
    orc_parallel(orc_fbatch_worker, &c, channels, threads);
}
