// Device building blocks of the GB300 DFT engine: complex arithmetic, radix-R DFT codelets held in
// registers, and the shared-memory block FFT that every transform kernel runs.
//
// The block FFT is a self-sorting (Stockham) mixed-radix sweep.  Pass p with radix R and
// Ns = R_0 * ... * R_{p-1} turns butterfly j (0 <= j < N/R) into
//     v[r] = buf[j + r*N/R] * W_{Ns*R}^{(j mod Ns)*r},   V = DFT_R(v),
//     buf[(j - j mod Ns)*R + j mod Ns + r*Ns] = V[r],
// so the result comes out in natural order with no digit-reverse pass.  This replaces the reference's
// in-place stages plus reorder stage (src/dft/dft-impl.hpp:85-150, 368-494) and its radix-4 DIF passes plus
// bit reversal (src/dft/fft-impl.hpp:846-1001).  Each pass reads all of its butterflies into registers,
// synchronises, and writes them back, so a signal needs only N (+1/16 padding) slots of shared memory.
#pragma once

#include "ct_table.hpp"

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "fft_desc.hpp"

namespace kfr_gpu
{

template <typename T>
struct alignas(2 * sizeof(T)) cpx
{
    T x, y;
};

template <typename T>
__device__ __forceinline__ cpx<T> mk(T x, T y)
{
    cpx<T> r;
    r.x = x;
    r.y = y;
    return r;
}
template <typename T>
__device__ __forceinline__ cpx<T> operator+(cpx<T> a, cpx<T> b)
{
    return mk(a.x + b.x, a.y + b.y);
}
template <typename T>
__device__ __forceinline__ cpx<T> operator-(cpx<T> a, cpx<T> b)
{
    return mk(a.x - b.x, a.y - b.y);
}
template <typename T>
__device__ __forceinline__ cpx<T> operator*(cpx<T> a, cpx<T> b)
{
    return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename T>
__device__ __forceinline__ cpx<T> scale(cpx<T> a, T s)
{
    return mk(a.x * s, a.y * s);
}
template <typename T>
__device__ __forceinline__ cpx<T> conj(cpx<T> a)
{
    return mk(a.x, -a.y);
}
// a * (-i)
template <typename T>
__device__ __forceinline__ cpx<T> mul_mi(cpx<T> a)
{
    return mk(a.y, -a.x);
}
// a * (+i)
template <typename T>
__device__ __forceinline__ cpx<T> mul_pi(cpx<T> a)
{
    return mk(-a.y, a.x);
}
template <typename T>
__device__ __forceinline__ cpx<T> conj_if(cpx<T> a, bool c)
{
    return c ? mk(a.x, -a.y) : a;
}

// Read-only cached load of one complex value.
__device__ __forceinline__ cpx<float> ldg(const cpx<float>* p)
{
    const float2 v = __ldg(reinterpret_cast<const float2*>(p));
    return mk(v.x, v.y);
}
__device__ __forceinline__ cpx<double> ldg(const cpx<double>* p)
{
    const double2 v = __ldg(reinterpret_cast<const double2*>(p));
    return mk(v.x, v.y);
}

// Shared-memory padding: one spare slot every 16 (8-byte elements) or 8 (16-byte elements) slots keeps
// the power-of-two strided writes of the early passes free of bank conflicts.
template <typename T>
struct smem_pad
{
    static constexpr int shift = sizeof(T) == 4 ? 4 : 3;
};
template <typename T>
__device__ __forceinline__ int pidx(int i)
{
    return i + (i >> smem_pad<T>::shift);
}
// padding with an explicit shift (0: none), used by the compile-time lengths
template <int PS>
__device__ __forceinline__ int pidx_s(int i)
{
    return PS ? i + (i >> PS) : i;
}
template <typename T>
__host__ __device__ constexpr int padded_len(int n)
{
    return n + (n >> smem_pad<T>::shift) + 1;
}

// --------------------------------------------------------------------------------------------------
// Codelets: forward DFT_R in registers, W_R = e^{-2 pi i / R}.
// --------------------------------------------------------------------------------------------------

template <typename T>
__device__ __forceinline__ void dft2(cpx<T>& a, cpx<T>& b)
{
    cpx<T> t = a;
    a        = t + b;
    b        = t - b;
}

template <typename T>
__device__ __forceinline__ void dft4(cpx<T>& x0, cpx<T>& x1, cpx<T>& x2, cpx<T>& x3)
{
    cpx<T> a0 = x0 + x2, a1 = x0 - x2;
    cpx<T> b0 = x1 + x3, b1 = mul_mi(x1 - x3);
    x0        = a0 + b0;
    x2        = a0 - b0;
    x1        = a1 + b1;
    x3        = a1 - b1;
}

// cos / sin of 2*pi*k/R for odd R and k = 0..(R-1)/2, folded to constants once k is unrolled.
__host__ __device__ constexpr double odd_cos(int R, int k)
{
    if (k == 0) // k*m can be a multiple of a composite radix (9)
        return 1.0;
    switch (R * 32 + k)
    {
    case 3 * 32 + 1: return -0.4999999999999998;
    case 5 * 32 + 1: return 0.30901699437494745;
    case 5 * 32 + 2: return -0.8090169943749473;
    case 7 * 32 + 1: return 0.6234898018587336;
    case 7 * 32 + 2: return -0.22252093395631434;
    case 7 * 32 + 3: return -0.900968867902419;
    case 9 * 32 + 1: return 0.766044443118978;
    case 9 * 32 + 2: return 0.17364817766693041;
    case 9 * 32 + 3: return -0.4999999999999998;
    case 9 * 32 + 4: return -0.9396926207859083;
    case 11 * 32 + 1: return 0.8412535328311812;
    case 11 * 32 + 2: return 0.41541501300188644;
    case 11 * 32 + 3: return -0.142314838273285;
    case 11 * 32 + 4: return -0.654860733945285;
    case 11 * 32 + 5: return -0.9594929736144974;
    case 13 * 32 + 1: return 0.8854560256532099;
    case 13 * 32 + 2: return 0.5680647467311559;
    case 13 * 32 + 3: return 0.120536680255323;
    case 13 * 32 + 4: return -0.35460488704253545;
    case 13 * 32 + 5: return -0.7485107481711012;
    case 13 * 32 + 6: return -0.970941817426052;
    default: return 0.0;
    }
}
__host__ __device__ constexpr double odd_sin(int R, int k)
{
    switch (R * 32 + k)
    {
    case 3 * 32 + 1: return 0.8660254037844387;
    case 5 * 32 + 1: return 0.9510565162951535;
    case 5 * 32 + 2: return 0.5877852522924732;
    case 7 * 32 + 1: return 0.7818314824680298;
    case 7 * 32 + 2: return 0.9749279121818236;
    case 7 * 32 + 3: return 0.43388373911755823;
    case 9 * 32 + 1: return 0.6427876096865393;
    case 9 * 32 + 2: return 0.984807753012208;
    case 9 * 32 + 3: return 0.8660254037844387;
    case 9 * 32 + 4: return 0.3420201433256689;
    case 11 * 32 + 1: return 0.5406408174555976;
    case 11 * 32 + 2: return 0.9096319953545183;
    case 11 * 32 + 3: return 0.9898214418809328;
    case 11 * 32 + 4: return 0.7557495743542583;
    case 11 * 32 + 5: return 0.28173255684142967;
    case 13 * 32 + 1: return 0.4647231720437685;
    case 13 * 32 + 2: return 0.8229838658936564;
    case 13 * 32 + 3: return 0.992708874098054;
    case 13 * 32 + 4: return 0.9350162426854148;
    case 13 * 32 + 5: return 0.6631226582407952;
    case 13 * 32 + 6: return 0.23931566428755768;
    default: return 0.0;
    }
}

// Odd-radix DFT by the symmetric pairing x_m +/- x_{R-m}:
//   X_k = x0 + sum_m cos(2 pi k m / R)(x_m + x_{R-m}) - i sum_m sin(2 pi k m / R)(x_m - x_{R-m}),
//   X_{R-k} = same with +i.
template <typename T, int R>
__device__ __forceinline__ void dft_odd(cpx<T>* v)
{
    constexpr int H = (R - 1) / 2;
    cpx<T> s[H], d[H];
#pragma unroll
    for (int m = 1; m <= H; m++)
    {
        s[m - 1] = v[m] + v[R - m];
        d[m - 1] = v[m] - v[R - m];
    }
    cpx<T> x0 = v[0];
    cpx<T> sum = x0;
#pragma unroll
    for (int m = 0; m < H; m++)
        sum = sum + s[m];
#pragma unroll
    for (int k = 1; k <= H; k++)
    {
        cpx<T> a = x0;
        cpx<T> b = mk<T>(0, 0);
#pragma unroll
        for (int m = 1; m <= H; m++)
        {
            const int km = (k * m) % R;
            // cos(2 pi km / R), sin(2 pi km / R) from the first-half tables
            const int idx = km <= H ? km : R - km;
            const T c     = T(odd_cos(R, idx));
            const T sn    = km <= H ? T(odd_sin(R, idx)) : -T(odd_sin(R, idx));
            a.x += c * s[m - 1].x;
            a.y += c * s[m - 1].y;
            b.x += sn * d[m - 1].x;
            b.y += sn * d[m - 1].y;
        }
        v[k]     = a + mul_mi(b);
        v[R - k] = a + mul_pi(b);
    }
    v[0] = sum;
}

template <typename T>
__device__ __forceinline__ void dft8(cpx<T>* v)
{
    const T h = T(0.70710678118654752440084436210485);
    dft4(v[0], v[2], v[4], v[6]);
    dft4(v[1], v[3], v[5], v[7]);
    cpx<T> o1 = mk(h * (v[3].x + v[3].y), h * (v[3].y - v[3].x)); // * W8
    cpx<T> o2 = mul_mi(v[5]);                                    // * W8^2
    cpx<T> o3 = mk(h * (v[7].y - v[7].x), -h * (v[7].x + v[7].y)); // * W8^3
    cpx<T> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    cpx<T> o0 = v[1];
    v[0]      = e0 + o0;
    v[4]      = e0 - o0;
    v[1]      = e1 + o1;
    v[5]      = e1 - o1;
    v[2]      = e2 + o2;
    v[6]      = e2 - o2;
    v[3]      = e3 + o3;
    v[7]      = e3 - o3;
}

// 16 = 4 x 4: column DFT4s, twiddles W16^{q k1}, row DFT4s done in place, so X[k1 + 4 k2] ends up in
// v[4 k1 + k2] (a transposed order; see codelet_out).
template <typename T>
__device__ __forceinline__ void dft16(cpx<T>* v)
{
    const T c = T(0.92387953251128675612818318939679);
    const T s = T(0.38268343236508977172845998403040);
    const T h = T(0.70710678118654752440084436210485);
#pragma unroll
    for (int q = 0; q < 4; q++)
        dft4(v[q], v[q + 4], v[q + 8], v[q + 12]);
    // y[q][k1] lives in v[q + 4*k1]
    v[5]  = v[5] * mk(c, -s);   // q=1,k1=1: W^1
    v[9]  = v[9] * mk(h, -h);   // q=1,k1=2: W^2
    v[13] = v[13] * mk(s, -c);  // q=1,k1=3: W^3
    v[6]  = v[6] * mk(h, -h);   // q=2,k1=1: W^2
    v[10] = mul_mi(v[10]);      // q=2,k1=2: W^4
    v[14] = v[14] * mk(-h, -h); // q=2,k1=3: W^6
    v[7]  = v[7] * mk(s, -c);   // q=3,k1=1: W^3
    v[11] = v[11] * mk(-h, -h); // q=3,k1=2: W^6
    v[15] = v[15] * mk(-c, s);  // q=3,k1=3: W^9
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++)
        dft4(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
}

// 3-point DFT in place: X1,2 = a - (b + c)/2 -/+ i (sqrt(3)/2)(b - c).
template <typename T>
__device__ __forceinline__ void dft3(cpx<T>& a, cpx<T>& b, cpx<T>& c)
{
    const T h      = T(0.86602540378443864676372317075294);
    const cpx<T> t = b + c;
    const cpx<T> d = b - c;
    const cpx<T> m = mk(a.x - T(0.5) * t.x, a.y - T(0.5) * t.y);
    a              = a + t;
    b              = mk(m.x + h * d.y, m.y - h * d.x);
    c              = mk(m.x - h * d.y, m.y + h * d.x);
}

// 9 = 3 x 3: DFT3 down each column, twiddles W9^{n1 k2}, DFT3 along each row, so X[k2 + 3 k1] ends up in
// v[3 k2 + k1] (a transposed order; see codelet_out).  About two thirds of the arithmetic of the direct
// symmetric form.
template <typename T>
__device__ __forceinline__ void dft9(cpx<T>* v)
{
    const T c1 = T(0.76604444311897803520239265055542), s1 = T(0.64278760968653932632264340990726); // 2pi/9
    const T c2 = T(0.17364817766693034885171662676931), s2 = T(0.98480775301220805936674302458952); // 4pi/9
    const T c4 = T(-0.93969262078590838405410927732473), s4 = T(0.34202014332566873304409961468226); // 8pi/9
#pragma unroll
    for (int n1 = 0; n1 < 3; n1++)
        dft3(v[n1], v[n1 + 3], v[n1 + 6]);
    // y[n1][k2] lives in v[n1 + 3 k2]
    v[4] = v[4] * mk(c1, -s1); // n1 = 1, k2 = 1: W9^1
    v[7] = v[7] * mk(c2, -s2); // n1 = 1, k2 = 2: W9^2
    v[5] = v[5] * mk(c2, -s2); // n1 = 2, k2 = 1: W9^2
    v[8] = v[8] * mk(c4, -s4); // n1 = 2, k2 = 2: W9^4
#pragma unroll
    for (int k2 = 0; k2 < 3; k2++)
        dft3(v[3 * k2], v[3 * k2 + 1], v[3 * k2 + 2]);
}

// Register holding output r of codelet R (identity except for the transposed radix-16 and radix-9 codelets).
template <int R>
__device__ __forceinline__ constexpr int codelet_out(int r)
{
    return R == 16 ? (r & 3) * 4 + (r >> 2) : R == 9 ? (r % 3) * 3 + r / 3 : r;
}

template <typename T, int R>
__device__ __forceinline__ void dft_codelet(cpx<T>* v);

// Composite radices with coprime factors R = R1 * R2 (6, 10, 12, 14, 15, 18), by the Good-Thomas prime
// factor algorithm: no twiddles between the two stages, only index maps that fold to register moves.
//   input  n = (R2 n1 + R1 n2) mod R
//   output k = (R2 e2 k1 + R1 e1 k2) mod R,  e2 = R2^-1 mod R1, e1 = R1^-1 mod R2
template <int R1, int R2>
struct pfa_split
{
    static constexpr int inv_mod(int a, int m)
    {
        for (int x = 1; x < m; x++)
            if ((a * x) % m == 1)
                return x;
        return 1;
    }
    static constexpr int e2 = inv_mod(R2 % R1, R1);
    static constexpr int e1 = inv_mod(R1 % R2, R2);
};

template <typename T, int R1, int R2>
__device__ __forceinline__ void dft_pfa(cpx<T>* v)
{
    constexpr int R = R1 * R2;
    using S         = pfa_split<R1, R2>;
    cpx<T> u[R1][R2];
#pragma unroll
    for (int n1 = 0; n1 < R1; n1++)
    {
#pragma unroll
        for (int n2 = 0; n2 < R2; n2++)
            u[n1][n2] = v[(R2 * n1 + R1 * n2) % R];
        dft_codelet<T, R2>(u[n1]);
    }
#pragma unroll
    for (int k2 = 0; k2 < R2; k2++)
    {
        cpx<T> w[R1];
#pragma unroll
        for (int n1 = 0; n1 < R1; n1++)
            w[n1] = u[n1][codelet_out<R2>(k2)];
        dft_codelet<T, R1>(w);
#pragma unroll
        for (int k1 = 0; k1 < R1; k1++)
            v[(R2 * S::e2 * k1 + R1 * S::e1 * k2) % R] = w[codelet_out<R1>(k1)];
    }
}

template <typename T, int R>
__device__ __forceinline__ void dft_codelet(cpx<T>* v)
{
    if constexpr (R == 2)
        dft2(v[0], v[1]);
    else if constexpr (R == 4)
        dft4(v[0], v[1], v[2], v[3]);
    else if constexpr (R == 8)
        dft8(v);
    else if constexpr (R == 16)
        dft16(v);
    else if constexpr (R == 9)
        dft9(v);
    else if constexpr (R == 6)
        dft_pfa<T, 2, 3>(v);
    else if constexpr (R == 10)
        dft_pfa<T, 2, 5>(v);
    else if constexpr (R == 12)
        dft_pfa<T, 4, 3>(v);
    else if constexpr (R == 14)
        dft_pfa<T, 2, 7>(v);
    else if constexpr (R == 15)
        dft_pfa<T, 3, 5>(v);
    else if constexpr (R == 18)
        dft_pfa<T, 2, 9>(v);
    else
        dft_odd<T, R>(v);
}

// --------------------------------------------------------------------------------------------------
// Block FFT descriptor (built on the host by the planner).
// --------------------------------------------------------------------------------------------------

__device__ __forceinline__ uint32_t fdiv(uint32_t x, const fast_div f)
{
    if (f.d == 1)
        return x;
    uint32_t hi = __umulhi(x, f.m);
    return (hi + ((x - hi) >> 1)) >> (f.s - 1);
}

// --------------------------------------------------------------------------------------------------
// One pass, split into a load half (gather butterflies, twiddle, DFT_R, all in the thread's register
// array v) and a store half (scatter to the self-sorted positions), with a barrier in between.  Every
// radix works on the same array v[EPT] so that the runtime radix switch keeps one register layout;
// threads lt in [0, ts) of a signal group own butterflies j = lt + b*ts.
// --------------------------------------------------------------------------------------------------

// v[r] *= W^{k r} from the one table value w1 = W^k by a binary powering tree, w_r = w_{r/2} w_{r - r/2}
// (at most ceil(log2 r) products deep): one load per butterfly instead of R - 1.  Both factors have index
// <= R/2 for every r < R, so only those powers stay live.
template <typename T, int R>
__device__ __forceinline__ void twiddle_powers(cpx<T> (&v)[R], const cpx<T> w1)
{
    cpx<T> w[R / 2 + 1];
    w[1] = w1;
    v[1] = v[1] * w1;
#pragma unroll
    for (int r = 2; r < R; r++)
    {
        const cpx<T> wr = w[r / 2] * w[r - r / 2];
        if (r <= R / 2)
            w[r] = wr;
        v[r] = v[r] * wr;
    }
}

template <typename T, int R, int EPT>
__device__ __forceinline__ void pass_load(cpx<T> (&v)[EPT], const cpx<T>* buf, const int n, const pass_desc& p,
                                          const cpx<T>* __restrict__ tw, const int lt, const int ts)
{
    constexpr int NB = EPT / R;
    const int nbf    = n / R;
    const int ns     = p.ns;
#pragma unroll
    for (int b = 0; b < NB; b++)
    {
        const int j = lt + b * ts;
        if (j < nbf)
        {
#pragma unroll
            for (int r = 0; r < R; r++)
                v[b * R + r] = buf[pidx<T>(j + r * nbf)];
            if (ns > 1)
            {
                const int k = j - int(fdiv(uint32_t(j), p.div_ns)) * ns;
                if constexpr (sizeof(T) == 4)
                {
                    // W^{k r} from the one table value W^k (the r = 1 entry) by the powering tree
                    twiddle_powers<T, R>(reinterpret_cast<cpx<T>(&)[R]>(v[b * R]), ldg(tw + p.tw_off + k));
                }
                else
                {
                    // double precision: table loads (FP64 products are slow on this part)
                    const cpx<T>* t = tw + p.tw_off + k;
#pragma unroll
                    for (int r = 1; r < R; r++)
                        v[b * R + r] = v[b * R + r] * ldg(t + (r - 1) * ns);
                }
            }
            dft_codelet<T, R>(&v[b * R]);
        }
    }
}

template <typename T, int R, int EPT>
__device__ __forceinline__ void pass_store(const cpx<T> (&v)[EPT], cpx<T>* buf, const int n, const pass_desc& p,
                                           const int lt, const int ts)
{
    constexpr int NB = EPT / R;
    const int nbf    = n / R;
    const int ns     = p.ns;
#pragma unroll
    for (int b = 0; b < NB; b++)
    {
        const int j = lt + b * ts;
        if (j < nbf)
        {
            const int k = ns > 1 ? j - int(fdiv(uint32_t(j), p.div_ns)) * ns : 0;
            const int d = (j - k) * R + k;
#pragma unroll
            for (int r = 0; r < R; r++)
                buf[pidx<T>(d + r * ns)] = v[b * R + codelet_out<R>(r)];
        }
    }
}

// Generic radix (any R, used for primes above 13): each thread computes up to EPT outputs
// o = lt + e*ts, each a length-R dot product of the twiddled inputs (read from shared memory) with the
// roots W_R^m.
template <typename T, int EPT>
__device__ __forceinline__ void pass_load_generic(cpx<T> (&v)[EPT], const cpx<T>* buf, const int n,
                                                  const pass_desc& p, const cpx<T>* __restrict__ tw, const int lt,
                                                  const int ts)
{
    const int R      = p.radix;
    const int nbf    = n / R;
    const int ns     = p.ns;
    const cpx<T>* wr = tw + p.wr_off;
#pragma unroll
    for (int e = 0; e < EPT; e++)
    {
        const int oi = lt + e * ts;
        if (oi < n)
        {
            const int q = oi / nbf;
            const int j = oi - q * nbf;
            const int k = ns > 1 ? j - int(fdiv(uint32_t(j), p.div_ns)) * ns : 0;
            cpx<T> acc  = buf[pidx<T>(j)];
            int widx    = 0;
#pragma unroll 1
            for (int r = 1; r < R; r++)
            {
                cpx<T> x = buf[pidx<T>(j + r * nbf)];
                if (ns > 1)
                    x = x * ldg(tw + p.tw_off + (r - 1) * ns + k);
                widx += q;
                if (widx >= R)
                    widx -= R;
                acc = acc + x * ldg(wr + widx);
            }
            v[e] = acc;
        }
    }
}

template <typename T, int EPT>
__device__ __forceinline__ void pass_store_generic(const cpx<T> (&v)[EPT], cpx<T>* buf, const int n,
                                                   const pass_desc& p, const int lt, const int ts)
{
    const int R   = p.radix;
    const int nbf = n / R;
    const int ns  = p.ns;
#pragma unroll
    for (int e = 0; e < EPT; e++)
    {
        const int oi = lt + e * ts;
        if (oi < n)
        {
            const int q = oi / nbf;
            const int j = oi - q * nbf;
            const int k = ns > 1 ? j - int(fdiv(uint32_t(j), p.div_ns)) * ns : 0;
            buf[pidx<T>((j - k) * R + k + q * ns)] = v[e];
        }
    }
}

// Runs every pass on the signal at buf.  The pass descriptors live in shared memory (staged by
// stage_passes) so that the runtime pass loop never indexes the kernel's parameter block.  Must be reached
// by all threads of the CTA (it synchronises); threads with lt >= ts only take part in the barriers.
template <typename T, int EPT>
__device__ __forceinline__ void block_fft(cpx<T>* buf, const pass_desc* sp, const int npass, const int n,
                                          const cpx<T>* __restrict__ tw, const int lt, const int ts)
{
    const int lta = lt < ts ? lt : n; // inactive threads own no butterflies
    cpx<T> v[EPT];
#pragma unroll 1
    for (int pi = 0; pi < npass; pi++)
    {
        const pass_desc p = sp[pi];
        switch (p.radix)
        {
#define KFR_GPU_LOAD_CASE(R)                                                                               \
    case R: pass_load<T, R, EPT>(v, buf, n, p, tw, lta, ts); break;
            KFR_GPU_LOAD_CASE(2)
            KFR_GPU_LOAD_CASE(3)
            KFR_GPU_LOAD_CASE(4)
            KFR_GPU_LOAD_CASE(5)
            KFR_GPU_LOAD_CASE(7)
            KFR_GPU_LOAD_CASE(8)
            KFR_GPU_LOAD_CASE(9)
            KFR_GPU_LOAD_CASE(11)
            KFR_GPU_LOAD_CASE(13)
            KFR_GPU_LOAD_CASE(16)
#undef KFR_GPU_LOAD_CASE
        default: pass_load_generic<T, EPT>(v, buf, n, p, tw, lta, ts); break;
        }
        __syncthreads();
        switch (p.radix)
        {
#define KFR_GPU_STORE_CASE(R)                                                                              \
    case R: pass_store<T, R, EPT>(v, buf, n, p, lta, ts); break;
            KFR_GPU_STORE_CASE(2)
            KFR_GPU_STORE_CASE(3)
            KFR_GPU_STORE_CASE(4)
            KFR_GPU_STORE_CASE(5)
            KFR_GPU_STORE_CASE(7)
            KFR_GPU_STORE_CASE(8)
            KFR_GPU_STORE_CASE(9)
            KFR_GPU_STORE_CASE(11)
            KFR_GPU_STORE_CASE(13)
            KFR_GPU_STORE_CASE(16)
#undef KFR_GPU_STORE_CASE
        default: pass_store_generic<T, EPT>(v, buf, n, p, lta, ts); break;
        }
        __syncthreads();
    }
}

// --------------------------------------------------------------------------------------------------
// Compile-time block FFT: the same Stockham passes for a length and radix sequence fixed at compile time,
// so every index, divisor and twiddle offset folds to a constant and each pass's butterfly loop unrolls.
// Used for the lengths listed in ct_table.hpp; the twiddle table layout matches block_program::build with
// the same radix order.
// --------------------------------------------------------------------------------------------------

template <typename T>
__host__ __device__ constexpr int ct_ps(int n, int ts)
{
    return sizeof(T) == 4 ? ct_pad_shift_f32(n, ts) : smem_pad<T>::shift;
}

template <int N, int TS, int R>
__host__ __device__ constexpr int ct_nb()
{
    return (N / R + TS - 1) / TS;
}
template <int N, int TS, int... Rs>
__host__ __device__ constexpr int ct_ept()
{
    int e = 1;
    ((e = (ct_nb<N, TS, Rs>() * Rs > e ? ct_nb<N, TS, Rs>() * Rs : e)), ...);
    return e;
}

template <typename T, int N, int TS, int EPT, int R, int NS, int TWOFF>
__device__ __forceinline__ void ct_pass(cpx<T> (&v)[EPT], cpx<T>* buf, const cpx<T>* __restrict__ tw, const int lt)
{
    constexpr int NBF = N / R;
    constexpr int NB  = (NBF + TS - 1) / TS;
    static_assert(NB * R <= EPT, "register array too small");
#pragma unroll
    for (int b = 0; b < NB; b++)
    {
        const int j = lt + b * TS;
        if (j < NBF)
        {
#pragma unroll
            for (int r = 0; r < R; r++)
                v[b * R + r] = buf[pidx_s<ct_ps<T>(N, TS)>(j + r * NBF)];
            if constexpr (NS > 1)
            {
                const int k     = j % NS;
                const cpx<T>* t = tw + TWOFF + k;
#pragma unroll
                for (int r = 1; r < R; r++)
                    v[b * R + r] = v[b * R + r] * ldg(t + (r - 1) * NS);
            }
            dft_codelet<T, R>(&v[b * R]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NB; b++)
    {
        const int j = lt + b * TS;
        if (j < NBF)
        {
            const int k = NS > 1 ? j % NS : 0;
            const int d = (j - k) * R + k;
#pragma unroll
            for (int r = 0; r < R; r++)
                buf[pidx_s<ct_ps<T>(N, TS)>(d + r * NS)] = v[b * R + codelet_out<R>(r)];
        }
    }
    __syncthreads();
}

template <typename T, int N, int TS, int EPT, int NS, int TWOFF, int R, int... Rest>
__device__ __forceinline__ void ct_passes(cpx<T> (&v)[EPT], cpx<T>* buf, const cpx<T>* __restrict__ tw, const int lt)
{
    ct_pass<T, N, TS, EPT, R, NS, TWOFF>(v, buf, tw, lt);
    if constexpr (sizeof...(Rest) > 0)
        ct_passes<T, N, TS, EPT, NS * R, TWOFF + (NS > 1 ? NS * (R - 1) : 0), Rest...>(v, buf, tw, lt);
}

template <typename T, int N, int TS, int... Rs>
__device__ __forceinline__ void ct_block_fft(cpx<T>* buf, const cpx<T>* __restrict__ tw, const int lt)
{
    constexpr int EPT = ct_ept<N, TS, Rs...>();
    const int lta     = lt < TS ? lt : N;
    cpx<T> v[EPT];
    ct_passes<T, N, TS, EPT, 1, 0, Rs...>(v, buf, tw, lta);
}

// no-op post(j, o): the last pass stores its outputs as computed
struct no_post
{
    template <class V>
    __device__ __forceinline__ void operator()(int, V&) const
    {
    }
};

// Ping-pong compile-time block FFT: pass i reads buffer A (i even) or B (i odd) and writes the other, so a
// pass needs one barrier and each butterfly's outputs are stored as soon as they are computed (no register
// array spans the pass).  ld(p) fetches input p of the first pass, st(q, x) stores output q of the last
// pass (which writes A when the number of passes is even, else B); the passes in between use the padded
// layouts of A and B.  hook() runs once, after the first pass's closing barrier.  Ends with a barrier.
// post(j, o) sees butterfly j's outputs o[r] (output j + r NS in the last pass) before they are stored
template <typename T, int N, int TS, int R, int NS, int TWOFF, class LD, class ST, class PO = no_post>
__device__ __forceinline__ void pp_pass(const LD& ld, const ST& st, const cpx<T>* __restrict__ tw, const int lt,
                                        const PO& post = PO())
{
    constexpr int NBF = N / R;
    constexpr int NB  = (NBF + TS - 1) / TS;
#pragma unroll
    for (int b = 0; b < NB; b++)
    {
        const int j = lt + b * TS;
        if (j < NBF)
        {
            cpx<T> v[R];
#pragma unroll
            for (int r = 0; r < R; r++)
                v[r] = ld(j + r * NBF);
            const int k = NS > 1 ? j % NS : 0;
            if constexpr (NS > 1)
                twiddle_powers<T, R>(v, ldg(tw + TWOFF + k));
            dft_codelet<T, R>(v);
            const int d = (j - k) * R + k;
            if constexpr (std::is_same_v<PO, no_post>)
            {
#pragma unroll
                for (int r = 0; r < R; r++)
                    st(d + r * NS, v[codelet_out<R>(r)]);
            }
            else
            {
                cpx<T> o[R];
#pragma unroll
                for (int r = 0; r < R; r++)
                    o[r] = v[codelet_out<R>(r)];
                post(j, o);
#pragma unroll
                for (int r = 0; r < R; r++)
                    st(d + r * NS, o[r]);
            }
        }
    }
    __syncthreads();
}

template <typename T, int N, int TS, int NS, int TWOFF, int I, class LD, class ST, class H, class P, int R,
          int... Rest, class PO = no_post>
__device__ __forceinline__ void pp_chain(const LD& ld, const ST& st, const H& hook, const P& pre_last, cpx<T>* A,
                                         cpx<T>* B, const cpx<T>* __restrict__ tw, const int lt,
                                         const PO& post = PO())
{
    if constexpr (sizeof...(Rest) == 0)
    {
        pre_last();
        pp_pass<T, N, TS, R, NS, TWOFF>(ld, st, tw, lt, post);
        if constexpr (NS == 1)
            hook();
    }
    else
    {
        cpx<T>* dst      = (I % 2 == 0) ? B : A;
        const auto d_st  = [dst](int q, cpx<T> x) { dst[pidx_s<ct_ps<T>(N, TS)>(q)] = x; };
        const auto d_ld  = [dst](int p) { return dst[pidx_s<ct_ps<T>(N, TS)>(p)]; };
        constexpr int TN = TWOFF + (NS > 1 ? NS * (R - 1) : 0);
        pp_pass<T, N, TS, R, NS, TWOFF>(ld, d_st, tw, lt);
        if constexpr (NS == 1)
            hook();
        pp_chain<T, N, TS, NS * R, TN, I + 1, decltype(d_ld), ST, H, P, Rest...>(d_ld, st, hook, pre_last, A, B, tw,
                                                                                lt, post);
    }
}

// hook() runs after the first pass, pre_last() before the last pass (all threads, uniformly); post(j, o) as
// in pp_pass, on the last pass's outputs.
template <typename T, int N, int TS, int... Rs, class LD, class ST, class H, class P, class PO = no_post>
__device__ __forceinline__ void ct_block_fft_pp(const LD& ld, const ST& st, const H& hook, const P& pre_last,
                                                cpx<T>* A, cpx<T>* B, const cpx<T>* __restrict__ tw, const int lt,
                                                const PO& post = PO())
{
    const int lta = lt < TS ? lt : N;
    pp_chain<T, N, TS, 1, 0, 0, LD, ST, H, P, Rs...>(ld, st, hook, pre_last, A, B, tw, lta, post);
}


// In-place compile-time block FFT with the signal in registers between the passes (EPT values per thread)
// and its loads and stores given as functors: the first pass reads ld(p), the passes exchange through the
// padded buffer, the last pass writes st(q, x).  Each pass loads (and transforms) all of its butterflies,
// then runs mid() for the last pass or a barrier otherwise, then stores; a barrier follows each store phase
// except the last pass's.  mid() must contain a barrier (after it the buffer is no longer read).  The chains
// below take a hook() that runs after the first pass.
template <typename T, int N, int TS, int EPT, int R, int NS, int TWOFF, class LD, class MID, class ST>
__device__ __forceinline__ void io_pass(cpx<T> (&v)[EPT], const LD& ld, const MID& mid, const ST& st,
                                        const cpx<T>* __restrict__ tw, const int lt)
{
    constexpr int NBF = N / R;
    constexpr int NB  = (NBF + TS - 1) / TS;
    static_assert(NB * R <= EPT, "register array too small");
#pragma unroll
    for (int b = 0; b < NB; b++)
    {
        const int j = lt + b * TS;
        if (j < NBF)
        {
            cpx<T> u[R];
#pragma unroll
            for (int r = 0; r < R; r++)
                u[r] = ld(j + r * NBF);
            if constexpr (NS > 1)
                twiddle_powers<T, R>(u, ldg(tw + TWOFF + j % NS));
            dft_codelet<T, R>(u);
#pragma unroll
            for (int r = 0; r < R; r++)
                v[b * R + r] = u[codelet_out<R>(r)];
        }
    }
    mid();
#pragma unroll
    for (int b = 0; b < NB; b++)
    {
        const int j = lt + b * TS;
        if (j < NBF)
        {
            const int k = NS > 1 ? j % NS : 0;
            const int d = (j - k) * R + k;
#pragma unroll
            for (int r = 0; r < R; r++)
                st(d + r * NS, v[b * R + r]);
        }
    }
}

// hook() runs once, after the first pass's closing barrier (the first pass's sources are no longer read).
template <typename T, int N, int TS, int EPT, int NS, int TWOFF, class LD, class MID, class ST, class H, int R,
          int... Rest>
__device__ __forceinline__ void io_chain(cpx<T> (&v)[EPT], const LD& ld, const MID& mid, const ST& st, const H& hook,
                                         cpx<T>* buf, const cpx<T>* __restrict__ tw, const int lt)
{
    if constexpr (sizeof...(Rest) == 0)
        io_pass<T, N, TS, EPT, R, NS, TWOFF>(v, ld, mid, st, tw, lt);
    else
    {
        const auto sync = []() { __syncthreads(); };
        const auto b_st = [buf](int q, cpx<T> x) { buf[pidx_s<ct_ps<T>(N, TS)>(q)] = x; };
        const auto b_ld = [buf](int p) { return buf[pidx_s<ct_ps<T>(N, TS)>(p)]; };
        io_pass<T, N, TS, EPT, R, NS, TWOFF>(v, ld, sync, b_st, tw, lt);
        __syncthreads();
        if constexpr (NS == 1)
            hook();
        constexpr int TN = TWOFF + (NS > 1 ? NS * (R - 1) : 0);
        io_chain<T, N, TS, EPT, NS * R, TN, decltype(b_ld), MID, ST, H, Rest...>(v, b_ld, mid, st, hook, buf, tw,
                                                                                 lt);
    }
}

template <typename T, int N, int TS, int... Rs, class LD, class MID, class ST, class H>
__device__ __forceinline__ void ct_block_fft_io(const LD& ld, const MID& mid, const ST& st, const H& hook,
                                                cpx<T>* buf, const cpx<T>* __restrict__ tw, const int lt)
{
    constexpr int EPT = ct_ept<N, TS, Rs...>();
    const int lta     = lt < TS ? lt : N;
    cpx<T> v[EPT];
    io_chain<T, N, TS, EPT, 1, 0, LD, MID, ST, H, Rs...>(v, ld, mid, st, hook, buf, tw, lta);
}

// Copies the descriptor's passes into shared memory with compile-time parameter offsets.  Ends with a
// barrier.
__device__ __forceinline__ void stage_passes(pass_desc* sp, const fft_desc& d)
{
#pragma unroll
    for (int i = 0; i < kMaxPasses; i++)
        if (int(threadIdx.x) == i)
            sp[i] = d.pass[i];
    __syncthreads();
}

} // namespace kfr_gpu
