/*
 * Oracle core for the KFR DFT hot path: test infrastructure only.
 *
 * This file is included twice by kfr_oracle.c, once with REAL=double (the parity reference every GPU
 * result is checked against) and once with REAL=float (the timed CPU baseline "port").  It restates, in
 * plain C, the algorithms of KFR 7.0.1 that the GPU library replaces:
 *
 *   - twiddles with quadrant folding ............ src/dft/ft.hpp:1797-1827 (calculate_twiddle)
 *   - plan factorisation: radices 10..2 greedily,
 *     Bluestein when the cofactor is >= 101 ..... src/dft/dft-impl.hpp:512-583 (init_dft)
 *   - mixed-radix stages with per-stage twiddles . src/dft/dft-impl.hpp:56-150, src/dft/ft.hpp:1535-1729
 *   - Bluestein chirp-z (integer chirp phase) .... src/dft/dft-impl.hpp:199-278
 *   - real DFT repack (CCs / Perm) ............... src/dft/fft-impl.hpp:1789-1896, 2070-2131
 *   - DCT-II / DCT-III ........................... include/kfr/dft/fft.hpp:926-978
 *   - fft_multiply(_accumulate) .................. include/kfr/dft/fft.hpp:983-1020
 *   - convolve / correlate ....................... src/dft/convolution-impl.cpp:106-128
 *   - convolve_filter (streaming, partitioned) ... src/dft/convolution-impl.cpp:37-84, 134-228
 *   - fir_filter (direct form, delay line) ....... include/kfr/dsp/fir.hpp:64-113, src/dsp/fir.cpp:54-57
 *
 * The stage structure is a self-sorting (Stockham) sweep over the factor list rather than KFR's in-place
 * stages plus digit-reverse permutation: the arithmetic of each radix-r butterfly and of each twiddle is
 * the same DFT, and only the memory order of intermediates differs.  Inverse transforms are unscaled, as
 * in KFR (include/kfr/dft/fft.hpp:262).
 *
 * Required macros: REAL (float or double), SFX (name suffix, e.g. _f64).
 */

#define ORC_CAT_(a, b) a##b
#define ORC_CAT(a, b) ORC_CAT_(a, b)
#define FN(name) ORC_CAT(name, SFX)

typedef struct
{
    REAL re, im;
} FN(cpx);
#define CPX FN(cpx)

static inline CPX FN(cmk)(REAL re, REAL im)
{
    CPX r;
    r.re = re;
    r.im = im;
    return r;
}
static inline CPX FN(cadd)(CPX a, CPX b) { return FN(cmk)(a.re + b.re, a.im + b.im); }
static inline CPX FN(csub)(CPX a, CPX b) { return FN(cmk)(a.re - b.re, a.im - b.im); }
static inline CPX FN(cmul)(CPX a, CPX b)
{
    return FN(cmk)(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
static inline CPX FN(cconj)(CPX a) { return FN(cmk)(a.re, -a.im); }
static inline CPX FN(cscale)(CPX a, REAL s) { return FN(cmk)(a.re * s, a.im * s); }

/* e^{-2 pi i n / size}, evaluated in double with the quadrant folding of calculate_twiddle
 * (src/dft/ft.hpp:1803-1827) and then rounded to REAL. */
static CPX FN(twiddle)(size_t n, size_t size)
{
    n     = n % size;
    int q = 0;
    if (size % 2 == 0 && n >= size / 2)
    {
        q += 2;
        n -= size / 2;
    }
    if (size % 4 == 0 && n >= size / 4)
    {
        q += 1;
        n -= size / 4;
    }
    double re = 1.0, im = 0.0;
    if (n != 0)
    {
        double kth = 2.0 * M_PI * ((double)n / (double)size);
        re         = cos(kth);
        im         = -sin(kth);
    }
    if (q & 1)
    { /* multiply by -i */
        double t = re;
        re       = im;
        im       = -t;
    }
    if (q & 2)
    {
        re = -re;
        im = -im;
    }
    return FN(cmk)((REAL)re, (REAL)im);
}

/* ------------------------------------------------------------------------------------------------ */
/* Plan                                                                                              */
/* ------------------------------------------------------------------------------------------------ */

#define ORC_MAX_PASSES 64

typedef struct FN(orc_plan)
{
    size_t n;
    int bluestein;
    int npasses;
    int radix[ORC_MAX_PASSES];
    size_t ns[ORC_MAX_PASSES];
    CPX* tw[ORC_MAX_PASSES];  /* pass twiddles: tw[p][(r-1)*Ns + k] = W_{Ns*R}^{k*r} */
    CPX* wr[ORC_MAX_PASSES];  /* generic radix roots: wr[p][m] = W_R^m */
    /* Bluestein */
    size_t m;
    CPX* chirp;               /* chirp[n] = e^{-i pi n^2 / N}  (dft-impl.hpp:217-226) */
    CPX* bhat;                /* conj(FFT_M(symmetric chirp)) / M (dft-impl.hpp:228-239) */
    struct FN(orc_plan) * inner;
} FN(orc_plan);
#define PLAN FN(orc_plan)

static size_t FN(next_pow2)(size_t x)
{
    size_t p = 1;
    while (p < x)
        p <<= 1;
    return p;
}

static void FN(plan_free)(PLAN* p)
{
    if (!p)
        return;
    for (int i = 0; i < p->npasses; i++)
    {
        free(p->tw[i]);
        free(p->wr[i]);
    }
    free(p->chirp);
    free(p->bhat);
    FN(plan_free)(p->inner);
    free(p);
}

static void FN(execute_plan)(const PLAN* p, CPX* out, const CPX* in, CPX* scratch);

static void FN(add_pass)(PLAN* p, int r, size_t* ns)
{
    int i        = p->npasses++;
    p->radix[i]  = r;
    p->ns[i]     = *ns;
    size_t L     = *ns * (size_t)r;
    p->tw[i]     = (CPX*)malloc(sizeof(CPX) * (size_t)(r - 1) * (*ns) + sizeof(CPX));
    for (int q = 1; q < r; q++)
        for (size_t k = 0; k < *ns; k++)
            p->tw[i][(size_t)(q - 1) * (*ns) + k] = FN(twiddle)(k * (size_t)q, L);
    p->wr[i] = (CPX*)malloc(sizeof(CPX) * (size_t)r);
    for (int q = 0; q < r; q++)
        p->wr[i][q] = FN(twiddle)((size_t)q, (size_t)r);
    *ns = L;
}

/* Plan construction.  The decision between mixed radix and Bluestein follows init_dft
 * (src/dft/dft-impl.hpp:524-547): strip radices 10..2 greedily; a cofactor >= 101 selects Bluestein for
 * the whole length.  Power-of-two lengths always take the FFT path (src/dft/fft-impl.hpp:1903-1918). */
static PLAN* FN(plan_create)(size_t n)
{
    PLAN* p = (PLAN*)calloc(1, sizeof(PLAN));
    p->n    = n;
    if (n <= 1)
        return p;
    size_t cur = n;
    for (size_t r = 10; r >= 2; r--)
        while (cur % r == 0)
            cur /= r;
    if (cur >= 101)
    {
        /* dft_arblen_stage_impl (src/dft/dft-impl.hpp:212-244) */
        p->bluestein = 1;
        p->m         = FN(next_pow2)(2 * n - 1);
        p->inner     = FN(plan_create)(p->m);
        p->chirp     = (CPX*)malloc(sizeof(CPX) * n);
        p->chirp[0]  = FN(cmk)(1, 0);
        size_t k     = 0;
        for (size_t mm = 1; mm < n; ++mm)
        {
            k += 2 * mm - 1;
            if (k >= 2 * n)
                k -= 2 * n;
            p->chirp[mm] = FN(twiddle)(k, 2 * n);
        }
        CPX* b         = (CPX*)calloc(p->m, sizeof(CPX));
        CPX* bs        = (CPX*)malloc(sizeof(CPX) * p->m);
        const REAL fct = (REAL)(1.0 / (double)p->m);
        for (size_t i = 0; i < n; i++)
            b[i] = FN(cscale)(p->chirp[i], fct);
        for (size_t i = 1; i < n; i++)
            b[p->m - i] = FN(cscale)(p->chirp[i], fct);
        p->bhat = (CPX*)malloc(sizeof(CPX) * p->m);
        FN(execute_plan)(p->inner, p->bhat, b, bs);
        for (size_t i = 0; i < p->m; i++)
            p->bhat[i] = FN(cconj)(p->bhat[i]);
        free(b);
        free(bs);
        return p;
    }
    /* Mixed radix: radices 8, 4, 2, 9, 3, 5, 7, then the prime cofactor < 101. */
    size_t ns = 1;
    cur       = n;
    while (cur % 8 == 0)
    {
        FN(add_pass)(p, 8, &ns);
        cur /= 8;
    }
    while (cur % 4 == 0)
    {
        FN(add_pass)(p, 4, &ns);
        cur /= 4;
    }
    while (cur % 2 == 0)
    {
        FN(add_pass)(p, 2, &ns);
        cur /= 2;
    }
    const int small[4] = { 9, 3, 5, 7 };
    for (int i = 0; i < 4; i++)
        while (cur % (size_t)small[i] == 0)
        {
            FN(add_pass)(p, small[i], &ns);
            cur /= (size_t)small[i];
        }
    if (cur > 1)
        FN(add_pass)(p, (int)cur, &ns);
    return p;
}

/* ------------------------------------------------------------------------------------------------ */
/* Butterflies (forward direction, W = e^{-2 pi i / R})                                               */
/* ------------------------------------------------------------------------------------------------ */

static inline void FN(bfly2)(CPX* v)
{
    CPX a = v[0], b = v[1];
    v[0]  = FN(cadd)(a, b);
    v[1]  = FN(csub)(a, b);
}

static inline CPX FN(mul_mi)(CPX a) { return FN(cmk)(a.im, -a.re); } /* a * (-i) */

static inline void FN(bfly4)(CPX* v)
{
    CPX a0 = FN(cadd)(v[0], v[2]), a1 = FN(csub)(v[0], v[2]);
    CPX b0 = FN(cadd)(v[1], v[3]), b1 = FN(mul_mi)(FN(csub)(v[1], v[3]));
    v[0]   = FN(cadd)(a0, b0);
    v[2]   = FN(csub)(a0, b0);
    v[1]   = FN(cadd)(a1, b1);
    v[3]   = FN(csub)(a1, b1);
}

static inline void FN(bfly8)(CPX* v)
{
    const REAL h = (REAL)0.70710678118654752440084436210485;
    CPX e[4]     = { v[0], v[2], v[4], v[6] };
    CPX o[4]     = { v[1], v[3], v[5], v[7] };
    FN(bfly4)(e);
    FN(bfly4)(o);
    /* o[k] *= W8^k */
    o[1] = FN(cmk)(h * (o[1].re + o[1].im), h * (o[1].im - o[1].re));
    o[2] = FN(mul_mi)(o[2]);
    o[3] = FN(cmk)(h * (o[3].im - o[3].re), -h * (o[3].re + o[3].im));
    for (int k = 0; k < 4; k++)
    {
        v[k]     = FN(cadd)(e[k], o[k]);
        v[k + 4] = FN(csub)(e[k], o[k]);
    }
}

static inline void FN(bfly3)(CPX* v)
{
    const REAL c = (REAL)-0.5, s = (REAL)0.86602540378443864676372317075294;
    CPX t1 = FN(cadd)(v[1], v[2]), t2 = FN(csub)(v[1], v[2]);
    CPX m1 = FN(cmk)(v[0].re + c * t1.re, v[0].im + c * t1.im);
    /* -i * s * t2 */
    CPX m2 = FN(cmk)(s * t2.im, -s * t2.re);
    v[0]   = FN(cadd)(v[0], t1);
    v[1]   = FN(cadd)(m1, m2);
    v[2]   = FN(csub)(m1, m2);
}

static inline void FN(bfly5)(CPX* v)
{
    const REAL c1 = (REAL)0.30901699437494742410, c2 = (REAL)-0.80901699437494742410;
    const REAL s1 = (REAL)0.95105651629515357212, s2 = (REAL)0.58778525229247312917;
    const CPX t1 = FN(cadd)(v[1], v[4]), t2 = FN(cadd)(v[2], v[3]);
    const CPX t3 = FN(csub)(v[1], v[4]), t4 = FN(csub)(v[2], v[3]);
    const CPX x0 = v[0];
    const CPX a1 = FN(cmk)(x0.re + c1 * t1.re + c2 * t2.re, x0.im + c1 * t1.im + c2 * t2.im);
    const CPX a2 = FN(cmk)(x0.re + c2 * t1.re + c1 * t2.re, x0.im + c2 * t1.im + c1 * t2.im);
    const CPX b1 = FN(cmk)(s1 * t3.re + s2 * t4.re, s1 * t3.im + s2 * t4.im);
    const CPX b2 = FN(cmk)(s2 * t3.re - s1 * t4.re, s2 * t3.im - s1 * t4.im);
    v[0]         = FN(cadd)(x0, FN(cadd)(t1, t2));
    v[1]         = FN(cmk)(a1.re + b1.im, a1.im - b1.re);
    v[4]         = FN(cmk)(a1.re - b1.im, a1.im + b1.re);
    v[2]         = FN(cmk)(a2.re + b2.im, a2.im - b2.re);
    v[3]         = FN(cmk)(a2.re - b2.im, a2.im + b2.re);
}

/* odd radix by the symmetric pairing x_m +/- x_{r-m}; cs[k-1], sn[k-1] = cos, sin of 2 pi k / r */
static inline void FN(bfly_odd)(CPX* v, int r, const double* cs, const double* sn)
{
    const int h = (r - 1) / 2;
    CPX s[8], d[8];
    CPX x0 = v[0], sum = v[0];
    for (int m = 1; m <= h; m++)
    {
        s[m - 1] = FN(cadd)(v[m], v[r - m]);
        d[m - 1] = FN(csub)(v[m], v[r - m]);
        sum      = FN(cadd)(sum, s[m - 1]);
    }
    for (int k = 1; k <= h; k++)
    {
        REAL ar = x0.re, ai = x0.im, br = 0, bi = 0;
        for (int m = 1; m <= h; m++)
        {
            int km = (k * m) % r;
            REAL c, sg;
            if (km == 0) /* composite r (9): k*m can be a multiple of r */
            {
                c  = 1;
                sg = 0;
            }
            else if (km <= h)
            {
                c  = (REAL)cs[km - 1];
                sg = (REAL)sn[km - 1];
            }
            else
            {
                c  = (REAL)cs[r - km - 1];
                sg = -(REAL)sn[r - km - 1];
            }
            ar += c * s[m - 1].re;
            ai += c * s[m - 1].im;
            br += sg * d[m - 1].re;
            bi += sg * d[m - 1].im;
        }
        /* X_k = a - i b, X_{r-k} = a + i b */
        v[k]     = FN(cmk)(ar + bi, ai - br);
        v[r - k] = FN(cmk)(ar - bi, ai + br);
    }
    v[0] = sum;
}

#ifndef ORC_ODD_CONSTANTS
#define ORC_ODD_CONSTANTS
static const double ORC_COS5[2] = { 0.30901699437494742410, -0.80901699437494742410 };
static const double ORC_SIN5[2] = { 0.95105651629515357212, 0.58778525229247312917 };
static const double ORC_COS7[3] = { 0.62348980185873353053, -0.22252093395631440429, -0.90096886790241912624 };
static const double ORC_SIN7[3] = { 0.78183148246802980871, 0.97492791218182360702, 0.43388373911755812048 };
static const double ORC_COS9[4] = { 0.76604444311897803520, 0.17364817766693034885, -0.5, -0.93969262078590838405 };
static const double ORC_SIN9[4] = { 0.64278760968653932632, 0.98480775301220805937, 0.86602540378443864676,
                                    0.34202014332566873304 };
#endif

static inline void FN(bfly_generic)(CPX* v, int r, const CPX* wr)
{
    CPX tmp[128];
    for (int k = 0; k < r; k++)
    {
        double sr = 0, si = 0;
        for (int j = 0; j < r; j++)
        {
            CPX w = wr[(size_t)((j * k) % r)];
            sr += (double)v[j].re * w.re - (double)v[j].im * w.im;
            si += (double)v[j].re * w.im + (double)v[j].im * w.re;
        }
        tmp[k] = FN(cmk)((REAL)sr, (REAL)si);
    }
    for (int k = 0; k < r; k++)
        v[k] = tmp[k];
}

/* One self-sorting pass: for butterfly j, inputs src[j + q*N/R] (q < R), twiddled by W_{Ns*R}^{(j%Ns)*q},
 * an R-point DFT, outputs dst[(j/Ns)*Ns*R + j%Ns + q*Ns]. */
static void FN(pass)(const PLAN* p, int pi, CPX* dst, const CPX* src)
{
    const size_t n  = p->n;
    const int r     = p->radix[pi];
    const size_t ns = p->ns[pi];
    const size_t nb = n / (size_t)r;
    const CPX* tw   = p->tw[pi];
    CPX v[128];
    for (size_t j0 = 0; j0 < nb; j0 += ns)
    {
        for (size_t k = 0; k < ns; k++)
        {
            const size_t j = j0 + k;
            v[0]           = src[j];
            for (int q = 1; q < r; q++)
                v[q] = FN(cmul)(src[j + (size_t)q * nb], tw[(size_t)(q - 1) * ns + k]);
            switch (r)
            {
            case 2: FN(bfly2)(v); break;
            case 3: FN(bfly3)(v); break;
            case 4: FN(bfly4)(v); break;
            case 8: FN(bfly8)(v); break;
            case 5: FN(bfly5)(v); break;
            case 7: FN(bfly_odd)(v, 7, ORC_COS7, ORC_SIN7); break;
            case 9: FN(bfly_odd)(v, 9, ORC_COS9, ORC_SIN9); break;
            default: FN(bfly_generic)(v, r, p->wr[pi]); break;
            }
            const size_t d = j0 * (size_t)r + k;
            for (int q = 0; q < r; q++)
                dst[d + (size_t)q * ns] = v[q];
        }
    }
}

/* Forward DFT of one signal.  scratch holds max(n, 2*m) values. out may alias in. */
static void FN(execute_plan)(const PLAN* p, CPX* out, const CPX* in, CPX* scratch)
{
    const size_t n = p->n;
    if (n == 0)
        return;
    if (n == 1)
    {
        out[0] = in[0];
        return;
    }
    if (p->bluestein)
    {
        /* dft_arblen_stage_impl::do_execute (src/dft/dft-impl.hpp:248-272) */
        const size_t m = p->m;
        CPX* xp        = scratch;
        CPX* tmp       = scratch + m;
        for (size_t i = 0; i < n; i++)
            xp[i] = FN(cmul)(in[i], p->chirp[i]);
        for (size_t i = n; i < m; i++)
            xp[i] = FN(cmk)(0, 0);
        FN(execute_plan)(p->inner, xp, xp, tmp);
        /* multiply by bhat, then inverse FFT via conj(FFT(conj(.))) */
        for (size_t i = 0; i < m; i++)
            xp[i] = FN(cconj)(FN(cmul)(xp[i], p->bhat[i]));
        FN(execute_plan)(p->inner, xp, xp, tmp);
        for (size_t i = 0; i < n; i++)
            out[i] = FN(cmul)(FN(cconj)(xp[i]), p->chirp[i]);
        return;
    }
    /* ping-pong between scratch and out; the last pass must land in out. */
    const int np = p->npasses;
    CPX* bufs[2];
    if (out == in)
    {
        memcpy(scratch + n, in, sizeof(CPX) * n);
        in = scratch + n;
    }
    bufs[np % 2 == 1 ? 0 : 1] = out;
    bufs[np % 2 == 1 ? 1 : 0] = scratch;
    /* bufs[(pi+1)%2]... choose so that pass np-1 writes to out */
    const CPX* src = in;
    for (int pi = 0; pi < np; pi++)
    {
        CPX* dst = ((np - 1 - pi) % 2 == 0) ? out : scratch;
        FN(pass)(p, pi, dst, src);
        src = dst;
    }
    (void)bufs;
}

static size_t FN(plan_scratch)(const PLAN* p)
{
    if (p->bluestein)
        return 2 * p->m + FN(plan_scratch)(p->inner);
    return 2 * p->n + 2;
}

static void FN(dft_one)(const PLAN* p, CPX* out, const CPX* in, int inverse, CPX* scratch)
{
    const size_t n = p->n;
    if (!inverse)
    {
        FN(execute_plan)(p, out, in, scratch);
        return;
    }
    /* unscaled inverse: conj(DFT(conj(x))) */
    CPX* tin = scratch + FN(plan_scratch)(p);
    for (size_t i = 0; i < n; i++)
        tin[i] = FN(cconj)(in[i]);
    FN(execute_plan)(p, out, tin, scratch);
    for (size_t i = 0; i < n; i++)
        out[i] = FN(cconj)(out[i]);
}

/* ------------------------------------------------------------------------------------------------ */
/* Real DFT (dft_plan_real): N/2-point complex DFT + repack.                                         */
/* ------------------------------------------------------------------------------------------------ */

/* Forward repack, as to_fmt (src/dft/fft-impl.hpp:1799-1841): Z = DFT_{N/2}(x viewed as complex). */
static void FN(real_repack_fwd)(size_t nreal, CPX* out, const CPX* z, int fmt_ccs)
{
    const size_t c = nreal / 2;
    const CPX dc   = z[0];
    for (size_t k = 1; k < c; k++)
    {
        const CPX zk = z[k], znk = FN(cconj)(z[c - k]);
        const CPX e  = FN(cscale)(FN(cadd)(zk, znk), (REAL)0.5);
        const CPX d  = FN(cscale)(FN(csub)(zk, znk), (REAL)0.5);
        /* O = d / i = -i d ; X = E + W_N^k O */
        const CPX o  = FN(mul_mi)(d);
        const CPX w  = FN(twiddle)(k, nreal);
        out[k]       = FN(cadd)(e, FN(cmul)(w, o));
    }
    if (fmt_ccs)
    {
        out[0] = FN(cmk)(dc.re + dc.im, 0);
        out[c] = FN(cmk)(dc.re - dc.im, 0);
    }
    else
        out[0] = FN(cmk)(dc.re + dc.im, dc.re - dc.im);
}

/* Inverse repack, as from_fmt (src/dft/fft-impl.hpp:1852-1896).  Only the real parts of the DC and
 * Nyquist bins are used. */
static void FN(real_repack_inv)(size_t nreal, CPX* z, const CPX* in, int fmt_ccs)
{
    const size_t c  = nreal / 2;
    const REAL x0   = in[0].re;
    const REAL xnyq = fmt_ccs ? in[c].re : in[0].im;
    for (size_t k = 1; k < c; k++)
    {
        const CPX xk = in[k], xnk = FN(cconj)(in[c - k]);
        const CPX f1 = FN(cadd)(xk, xnk), f2 = FN(csub)(xk, xnk);
        /* t = i * e^{+2 pi i k / N} * f2 */
        CPX w        = FN(cconj)(FN(twiddle)(k, nreal));
        CPX t        = FN(cmul)(w, f2);
        t            = FN(cmk)(-t.im, t.re);
        z[k]         = FN(cadd)(f1, t);
    }
    z[0] = FN(cmk)(x0 + xnyq, x0 - xnyq);
}

/* ------------------------------------------------------------------------------------------------ */
/* convolve_filter: restatement of the streaming partitioned overlap-add                             */
/* (src/dft/convolution-impl.cpp:37-84, 134-228).  Real T uses a real DFT of 2B in Perm format,      */
/* complex T a complex DFT of 2B (include/kfr/dft/convolution.hpp:80-95).                             */
/* ------------------------------------------------------------------------------------------------ */

typedef struct FN(orc_filter)
{
    int is_complex;
    size_t data_size, block, fftsize, csize, nseg;
    PLAN* plan; /* complex plan of fftsize (complex filter) or fftsize/2 (real filter) */
    CPX** segments;
    CPX** ir_segments;
    size_t position, input_position;
    CPX* saved_input; /* block values (real filters use .re only) */
    CPX *premul, *cscratch, *scratch1, *scratch2, *overlap, *work;
} FN(orc_filter);
#define FILT FN(orc_filter)

/* forward transform of scratch (fftsize values) to spectrum (csize values) */
static void FN(filt_fwd)(FILT* f, CPX* spec, const CPX* x)
{
    if (f->is_complex)
    {
        FN(execute_plan)(f->plan, spec, x, f->work);
        return;
    }
    /* pack reals into N/2 complex, DFT, repack Perm */
    const size_t c = f->csize;
    CPX* z         = f->work + FN(plan_scratch)(f->plan);
    for (size_t i = 0; i < c; i++)
        z[i] = FN(cmk)(x[2 * i].re, x[2 * i + 1].re);
    CPX* zz = z + c;
    FN(execute_plan)(f->plan, zz, z, f->work);
    FN(real_repack_fwd)(f->fftsize, spec, zz, 0);
}

static void FN(filt_inv)(FILT* f, CPX* y, const CPX* spec)
{
    const size_t c = f->csize;
    if (f->is_complex)
    {
        FN(dft_one)(f->plan, y, spec, 1, f->work);
        return;
    }
    CPX* z = f->work + FN(plan_scratch)(f->plan) + c + 2 * c;
    FN(real_repack_inv)(f->fftsize, z, spec, 0);
    CPX* zz = z + c;
    FN(dft_one)(f->plan, zz, z, 1, f->work);
    for (size_t i = 0; i < c; i++)
    {
        y[2 * i]     = FN(cmk)(zz[i].re, 0);
        y[2 * i + 1] = FN(cmk)(zz[i].im, 0);
    }
}

/* fft_multiply / fft_multiply_accumulate (include/kfr/dft/fft.hpp:983-1020); perm selects the special
 * DC/Nyquist product. */
static void FN(fft_mul)(CPX* dst, const CPX* a, const CPX* b, size_t n, int perm)
{
    const CPX f0 = FN(cmk)(a[0].re * b[0].re, a[0].im * b[0].im);
    for (size_t i = 0; i < n; i++)
        dst[i] = FN(cmul)(a[i], b[i]);
    if (perm)
        dst[0] = f0;
}
static void FN(fft_mac)(CPX* dst, const CPX* a, const CPX* b, size_t n, int perm)
{
    const CPX f0 = FN(cmk)(dst[0].re + a[0].re * b[0].re, dst[0].im + a[0].im * b[0].im);
    for (size_t i = 0; i < n; i++)
        dst[i] = FN(cadd)(dst[i], FN(cmul)(a[i], b[i]));
    if (perm)
        dst[0] = f0;
}
static void FN(fft_mac3)(CPX* dst, const CPX* s1, const CPX* a, const CPX* b, size_t n, int perm)
{
    const CPX f0 = FN(cmk)(s1[0].re + a[0].re * b[0].re, s1[0].im + a[0].im * b[0].im);
    for (size_t i = 0; i < n; i++)
        dst[i] = FN(cadd)(s1[i], FN(cmul)(a[i], b[i]));
    if (perm)
        dst[0] = f0;
}

static void FN(filt_reset)(FILT* f)
{
    for (size_t i = 0; i < f->nseg; i++)
        memset(f->segments[i], 0, sizeof(CPX) * f->csize);
    f->position = 0;
    memset(f->saved_input, 0, sizeof(CPX) * f->block);
    f->input_position = 0;
    memset(f->overlap, 0, sizeof(CPX) * f->block);
}

/* taps: data_size values (CPX; real filters use .re only). */
static FILT* FN(filt_create)(const CPX* taps, size_t ntaps, size_t block, int is_complex)
{
    FILT* f       = (FILT*)calloc(1, sizeof(FILT));
    f->is_complex = is_complex;
    f->data_size  = ntaps;
    f->block      = FN(next_pow2)(block ? block : 1024);
    f->fftsize    = 2 * f->block;
    f->csize      = is_complex ? f->fftsize : f->fftsize / 2;
    f->plan       = FN(plan_create)(is_complex ? f->fftsize : f->fftsize / 2);
    f->nseg       = (ntaps + f->block - 1) / f->block;
    f->segments   = (CPX**)calloc(f->nseg ? f->nseg : 1, sizeof(CPX*));
    f->ir_segments = (CPX**)calloc(f->nseg ? f->nseg : 1, sizeof(CPX*));
    const size_t ws = FN(plan_scratch)(f->plan) + 8 * f->fftsize + 8;
    f->work        = (CPX*)calloc(ws, sizeof(CPX));
    f->saved_input = (CPX*)calloc(f->block, sizeof(CPX));
    f->premul      = (CPX*)calloc(f->csize + 1, sizeof(CPX));
    f->cscratch    = (CPX*)calloc(f->csize + 1, sizeof(CPX));
    f->scratch1    = (CPX*)calloc(f->fftsize, sizeof(CPX));
    f->scratch2    = (CPX*)calloc(f->fftsize, sizeof(CPX));
    f->overlap     = (CPX*)calloc(f->block, sizeof(CPX));
    CPX* input     = (CPX*)calloc(f->fftsize, sizeof(CPX));
    const REAL ifs = (REAL)1 / (REAL)f->fftsize;
    for (size_t i = 0; i < f->nseg; i++)
    {
        f->segments[i]    = (CPX*)calloc(f->csize + 1, sizeof(CPX));
        f->ir_segments[i] = (CPX*)calloc(f->csize + 1, sizeof(CPX));
        memset(input, 0, sizeof(CPX) * f->fftsize);
        for (size_t j = 0; j < f->block && i * f->block + j < ntaps; j++)
            input[j] = taps[i * f->block + j];
        FN(filt_fwd)(f, f->ir_segments[i], input);
        for (size_t j = 0; j < f->csize; j++)
            f->ir_segments[i][j] = FN(cscale)(f->ir_segments[i][j], ifs);
    }
    free(input);
    FN(filt_reset)(f);
    return f;
}

static void FN(filt_free)(FILT* f)
{
    if (!f)
        return;
    for (size_t i = 0; i < f->nseg; i++)
    {
        free(f->segments[i]);
        free(f->ir_segments[i]);
    }
    free(f->segments);
    free(f->ir_segments);
    FN(plan_free)(f->plan);
    free(f->work);
    free(f->saved_input);
    free(f->premul);
    free(f->cscratch);
    free(f->scratch1);
    free(f->scratch2);
    free(f->overlap);
    free(f);
}

/* process_buffer_impl (src/dft/convolution-impl.cpp:134-228) */
static void FN(filt_process)(FILT* f, CPX* output, const CPX* input, size_t size)
{
    const int perm   = !f->is_complex;
    const size_t B   = f->block;
    size_t processed = 0;
    if (f->nseg == 0)
    {
        for (size_t i = 0; i < size; i++)
            output[i] = FN(cmk)(0, 0);
        return;
    }
    while (processed < size)
    {
        size_t processing = size - processed;
        if (processing > B - f->input_position)
            processing = B - f->input_position;
        memset(f->scratch1, 0, sizeof(CPX) * f->fftsize);
        if (processing == B)
            memcpy(f->scratch1, input + processed, processing * sizeof(CPX));
        else
        {
            memcpy(f->saved_input + f->input_position, input + processed, processing * sizeof(CPX));
            memcpy(f->scratch1, f->saved_input, B * sizeof(CPX));
        }
        FN(filt_fwd)(f, f->segments[f->position], f->scratch1);
        if (f->nseg == 1)
            FN(fft_mul)(f->cscratch, f->ir_segments[0], f->segments[0], f->csize, perm);
        else
        {
            if (f->input_position == 0)
            {
                FN(fft_mul)(f->premul, f->ir_segments[1], f->segments[(f->position + 1) % f->nseg], f->csize,
                            perm);
                for (size_t i = 2; i < f->nseg; i++)
                {
                    const size_t nn = (f->position + i) % f->nseg;
                    FN(fft_mac)(f->premul, f->ir_segments[i], f->segments[nn], f->csize, perm);
                }
            }
            FN(fft_mac3)(f->cscratch, f->premul, f->ir_segments[0], f->segments[f->position], f->csize, perm);
        }
        FN(filt_inv)(f, f->scratch2, f->cscratch);
        for (size_t i = 0; i < processing; i++)
            output[processed + i] =
                FN(cadd)(f->scratch2[f->input_position + i], f->overlap[f->input_position + i]);
        f->input_position += processing;
        processed += processing;
        if (f->input_position == B)
        {
            f->input_position      = 0;
            const size_t remaining = size - processed;
            if (remaining < B && remaining > 0)
                memset(f->saved_input, 0, sizeof(CPX) * B);
            memcpy(f->overlap, f->scratch2 + B, B * sizeof(CPX));
            f->position = f->position > 0 ? f->position - 1 : f->nseg - 1;
        }
    }
}

#undef CPX
#undef PLAN
#undef FILT

/* fir_filter<T> (include/kfr/dsp/fir.hpp:64-113, src/dsp/fir.cpp:54-57): direct form
 * y[n] = sum_k taps[k] x[n - k] with a delay line of the last ntaps inputs, zero after creation and after
 * reset, kept across process calls. */
typedef struct FN(orc_fir)
{
    size_t ntaps;
    REAL* taps;
    REAL* hist; /* the last ntaps inputs, oldest first */
} FN(orc_fir);

static FN(orc_fir) * FN(fir_create)(const REAL* taps, size_t ntaps)
{
    FN(orc_fir)* f = (FN(orc_fir)*)calloc(1, sizeof(FN(orc_fir)));
    f->ntaps       = ntaps;
    f->taps        = (REAL*)calloc(ntaps + 1, sizeof(REAL));
    f->hist        = (REAL*)calloc(ntaps + 1, sizeof(REAL));
    for (size_t i = 0; i < ntaps; i++)
        f->taps[i] = taps[i];
    return f;
}

static void FN(fir_reset)(FN(orc_fir) * f) { memset(f->hist, 0, sizeof(REAL) * (f->ntaps + 1)); }

static void FN(fir_process)(FN(orc_fir) * f, REAL* out, const REAL* in, size_t n)
{
    const size_t m = f->ntaps;
    for (size_t i = 0; i < n; i++)
    {
        if (m)
        {
            memmove(f->hist, f->hist + 1, sizeof(REAL) * (m - 1));
            f->hist[m - 1] = in[i];
        }
        REAL acc = 0;
        for (size_t k = 0; k < m; k++)
            acc += f->taps[k] * f->hist[m - 1 - k];
        out[i] = acc;
    }
}

static void FN(fir_free)(FN(orc_fir) * f)
{
    if (!f)
        return;
    free(f->taps);
    free(f->hist);
    free(f);
}
