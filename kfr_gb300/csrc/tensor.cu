// Radix-16 passes as tensor-core contractions (warp-level mma.sync, m16n8k16, FP32 accumulation) with split
// operands, for N = 16^2, 16^3 in one CTA and N = 2^16, 2^20, 2^24 as a four-step of 256- and 4096-point
// column and row FFTs.
//
// One radix-16 butterfly is y = F16 u (u: the 16 twiddled inputs, F16[k][r] = e^{-2 pi i k r / 16}).  In real
// arithmetic, with F16 = C - iS:
//     [Re y]   [ C  S ] [Re u]
//     [Im y] = [-S  C ] [Im u]          (32 x 32 times 32 x 8 for eight butterflies)
// computed as 16 x 16 x 8 tiles.  FP32 values do not fit one 16-bit operand, so each is split into a sum of
// 16-bit parts and the contraction keeps the partial products down to about FP32's rounding:
//
//   TC_FP16: x = hi + lo, hi = fp16(x), lo = fp16(x - hi): 22 significant bits.  FP16's exponent range is
//     narrow, so each butterfly's 16 inputs are first scaled by a power of two that puts their largest
//     magnitude in [2^14, 2^15) (exact; undone on the outputs, which the FP32 accumulator holds): no part
//     overflows, and no low part of a value within 2^-17 of the butterfly's largest one falls into FP16's
//     subnormal range.  Products kept: hi*hi + hi*lo + lo*hi (three contractions per tile; lo*lo, below
//     2^-22 of the product, is dropped).
//   TC_BF16: x = hi + mid + lo, each the BF16 rounding of what the previous parts leave: 24 significant bits
//     and FP32's exponent range, so no scaling.  Products kept: every pair whose weight is at least 2^-16:
//     hi*hi, hi*mid, mid*hi, hi*lo, lo*hi, mid*mid (six contractions per tile).
//
// The smaller products are accumulated first.  Twiddles are applied in FP32 before the split.
#include "kernels.cuh"
#include "tensor.hpp"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace kfr_gpu
{

namespace
{

constexpr unsigned kFull = 0xffffffffu;

// number of 16-bit parts per operand
template <int MODE>
constexpr int kParts = MODE == TC_BF16 ? 3 : 2;

template <int MODE>
__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    if constexpr (MODE == TC_BF16)
    {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<const uint32_t*>(&h);
    }
    else
    {
        const __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<const uint32_t*>(&h);
    }
}

template <int MODE>
__device__ __forceinline__ float2 unpack2(uint32_t v)
{
    if constexpr (MODE == TC_BF16)
        return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&v));
    else
        return __half22float2(*reinterpret_cast<const __half2*>(&v));
}

// splits (a, b) into kParts<MODE> pairs of 16-bit values, largest first
template <int MODE>
__device__ __forceinline__ void split_pair(float a, float b, uint32_t (&p)[kParts<MODE>])
{
#pragma unroll
    for (int i = 0; i < kParts<MODE>; i++)
    {
        p[i]           = pack2<MODE>(a, b);
        const float2 f = unpack2<MODE>(p[i]);
        a -= f.x;
        b -= f.y;
    }
}

template <int MODE>
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    if constexpr (MODE == TC_BF16)
        asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                     "{%0,%1,%2,%3};"
                     : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                     : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
    else
        asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                     "{%0,%1,%2,%3};"
                     : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                     : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// negation of both 16-bit values of a pair (sign bits), exact in either format
__device__ __forceinline__ uint32_t neg_pair(uint32_t x) { return x ^ 0x80008000u; }

// A fragments of the DFT-16 matrix: C (cos), S (sin) and -S, each split into kParts parts.  Row k = output,
// column r = input; a lane holds rows g, g + 8 and columns 2q, 2q + 1, 2q + 8, 2q + 9.
template <int MODE>
struct tc_frags
{
    uint32_t C[kParts<MODE>][4], S[kParts<MODE>][4], nS[kParts<MODE>][4];

    __device__ explicit tc_frags(const float* __restrict__ cs)
    {
        const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
        const int rows[4] = { g, g + 8, g, g + 8 };
        const int cols[4] = { 2 * q, 2 * q, 2 * q + 8, 2 * q + 8 };
#pragma unroll
        for (int i = 0; i < 4; i++)
        {
            uint32_t c[kParts<MODE>], s[kParts<MODE>];
            split_pair<MODE>(cs[rows[i] * 16 + cols[i]], cs[rows[i] * 16 + cols[i] + 1], c);
            split_pair<MODE>(cs[256 + rows[i] * 16 + cols[i]], cs[256 + rows[i] * 16 + cols[i] + 1], s);
#pragma unroll
            for (int p = 0; p < kParts<MODE>; p++)
            {
                C[p][i]  = c[p];
                S[p][i]  = s[p];
                nS[p][i] = neg_pair(s[p]);
            }
        }
    }
};

// acc += M * u over the kept partial products, smallest weights first (bx: the B pairs of u's parts, x0 for
// rows 2q, 2q+1 and x1 for rows 2q+8, 2q+9)
template <int MODE>
__device__ __forceinline__ void contract(float (&acc)[4], const uint32_t (&M)[kParts<MODE>][4],
                                         const uint32_t (&x0)[kParts<MODE>], const uint32_t (&x1)[kParts<MODE>])
{
    if constexpr (MODE == TC_BF16)
    {
        mma16816<MODE>(acc, M[2], x0[0], x1[0]); // lo * hi   (2^-16)
        mma16816<MODE>(acc, M[0], x0[2], x1[2]); // hi * lo   (2^-16)
        mma16816<MODE>(acc, M[1], x0[1], x1[1]); // mid * mid (2^-16)
        mma16816<MODE>(acc, M[1], x0[0], x1[0]); // mid * hi  (2^-8)
        mma16816<MODE>(acc, M[0], x0[1], x1[1]); // hi * mid  (2^-8)
        mma16816<MODE>(acc, M[0], x0[0], x1[0]); // hi * hi
    }
    else
    {
        mma16816<MODE>(acc, M[1], x0[0], x1[0]); // lo * hi (2^-11)
        mma16816<MODE>(acc, M[0], x0[1], x1[1]); // hi * lo (2^-11)
        mma16816<MODE>(acc, M[0], x0[0], x1[0]); // hi * hi
    }
}

// 2^k as a float for |k| <= 126 (exact)
__device__ __forceinline__ float pow2f(int k) { return __int_as_float((127 + k) << 23); }

// One radix-16 pass over nsig signals of length L in shared memory (signal s at src + s * stride, element e
// at pidx(e)), Stockham order: butterfly j (j < L / 16, k = j mod ns) reads elements j + r L / 16 (r < 16),
// multiplies input r by tw[(r - 1) ns + k] (ns > 1) and writes output m to (j - k) 16 + k + m ns of dst.
// Warp-uniform loop over tiles of eight butterflies.
template <int MODE, int L>
__device__ __forceinline__ void tc_pass(const cpx<float>* src, cpx<float>* dst, const int nsig, const int stride,
                                        const int ns, const cpx<float>* __restrict__ tw, const tc_frags<MODE>& F)
{
    constexpr int NBF   = L / 16;
    constexpr int TILES = NBF / 8;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int g = lane >> 2, q = lane & 3;
    for (int t = warp; t < nsig * TILES; t += nwarps)
    {
        const int s = t / TILES, j0 = (t - s * TILES) * 8;
        const cpx<float>* sb = src + s * stride;
        // B operands: butterfly j0 + g, inputs r in {2q, 2q+1, 2q+8, 2q+9}
        const int j = j0 + g, k = j % ns;
        const int rr[4] = { 2 * q, 2 * q + 1, 2 * q + 8, 2 * q + 9 };
        cpx<float> u[4];
#pragma unroll
        for (int i = 0; i < 4; i++)
        {
            cpx<float> v = sb[pidx<float>(j + rr[i] * NBF)];
            if (ns > 1 && rr[i] > 0)
                v = v * ldg(tw + (rr[i] - 1) * ns + k);
            u[i] = v;
        }
        float unscale0 = 1.0f, unscale1 = 1.0f;
        if constexpr (MODE == TC_FP16)
        {
            // per-butterfly power of two: the largest magnitude of the 16 inputs into [2^14, 2^15)
            float mx = 0.0f;
#pragma unroll
            for (int i = 0; i < 4; i++)
                mx = fmaxf(mx, fmaxf(fabsf(u[i].x), fabsf(u[i].y)));
            mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, 1));
            mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, 2));
            int e = 0;
            frexpf(mx, &e); // mx < 2^e (e = 0 for mx = 0)
            e              = e < -100 ? -100 : (e > 100 ? 100 : e);
            const float sc = pow2f(15 - e);
#pragma unroll
            for (int i = 0; i < 4; i++)
                u[i] = scale(u[i], sc);
            // output columns 2q and 2q + 1 are the butterflies whose inputs lanes 4 (2q) and 4 (2q + 1) hold
            const int ee = e;
            unscale0     = pow2f(__shfl_sync(kFull, ee, 8 * q) - 15);
            unscale1     = pow2f(__shfl_sync(kFull, ee, 8 * q + 4) - 15);
        }
        uint32_t re0[kParts<MODE>], re1[kParts<MODE>], im0[kParts<MODE>], im1[kParts<MODE>];
        split_pair<MODE>(u[0].x, u[1].x, re0);
        split_pair<MODE>(u[2].x, u[3].x, re1);
        split_pair<MODE>(u[0].y, u[1].y, im0);
        split_pair<MODE>(u[2].y, u[3].y, im1);
        float top[4] = { 0, 0, 0, 0 }, bot[4] = { 0, 0, 0, 0 };
        contract<MODE>(top, F.S, im0, im1); // Re y = C Re u + S Im u
        contract<MODE>(top, F.C, re0, re1);
        contract<MODE>(bot, F.nS, re0, re1); // Im y = -S Re u + C Im u
        contract<MODE>(bot, F.C, im0, im1);
        // D: outputs m = g (regs 0, 1) and g + 8 (regs 2, 3) of butterflies j0 + 2q and j0 + 2q + 1
        cpx<float>* db = dst + s * stride;
#pragma unroll
        for (int c = 0; c < 2; c++)
        {
            const float us = c == 0 ? unscale0 : unscale1;
            const int bf = j0 + 2 * q + c, kk = bf % ns, d = (bf - kk) * 16 + kk;
            db[pidx<float>(d + g * ns)]       = mk<float>(top[c] * us, bot[c] * us);
            db[pidx<float>(d + (g + 8) * ns)] = mk<float>(top[2 + c] * us, bot[2 + c] * us);
        }
    }
}

// All log16(L) passes over nsig signals ping-ponging between a and b (tw: the passes' tables, pass with stride
// ns > 1 at the running offset); returns the buffer holding the result.
template <int MODE, int L>
__device__ __forceinline__ cpx<float>* tc_block_fft(cpx<float>* a, cpx<float>* b, const int nsig, const int stride,
                                                    const cpx<float>* __restrict__ tw, const tc_frags<MODE>& F)
{
    constexpr int P = L == 256 ? 2 : 3;
    static_assert(L == 256 || L == 4096, "lengths 16^2 and 16^3");
    cpx<float>* src = a;
    cpx<float>* dst = b;
    int ns = 1, twoff = 0;
#pragma unroll 1
    for (int p = 0; p < P; p++)
    {
        tc_pass<MODE, L>(src, dst, nsig, stride, ns, tw + twoff, F);
        __syncthreads();
        twoff += ns > 1 ? ns * 15 : 0;
        ns *= 16;
        cpx<float>* tmp = src;
        src             = dst;
        dst             = tmp;
    }
    return src;
}

// Signals that fit one CTA: spc signals of N = 256 or 4096 per CTA.
template <int MODE, int N>
__global__ void __launch_bounds__(512, 1) k_c2c_tc(const c2c_args a, const float* __restrict__ cs, const int spc)
{
    constexpr int STRIDE = padded_len<float>(N);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<float>* bufA = reinterpret_cast<cpx<float>*>(smem_raw);
    cpx<float>* bufB = bufA + spc * STRIDE;
    const long long s0 = (long long)blockIdx.x * spc;
    const cpx<float>* __restrict__ in = reinterpret_cast<const cpx<float>*>(a.in);
    cpx<float>* __restrict__ out      = reinterpret_cast<cpx<float>*>(a.out);
    const bool inv = a.inverse != 0;
    const int nsig = a.batch - s0 < spc ? int(a.batch - s0) : spc;
    const tc_frags<MODE> F(cs);
    for (int i = threadIdx.x; i < nsig * N; i += blockDim.x)
    {
        const int s = i / N, e = i - s * N;
        bufA[s * STRIDE + pidx<float>(e)] = conj_if(in[(s0 + s) * a.istride + e], inv);
    }
    __syncthreads();
    const cpx<float>* res = tc_block_fft<MODE, N>(bufA, bufB, nsig, STRIDE, reinterpret_cast<const cpx<float>*>(a.tw), F);
    for (int i = threadIdx.x; i < nsig * N; i += blockDim.x)
    {
        const int s = i / N, e = i - s * N;
        out[(s0 + s) * a.ostride + e] = conj_if(res[s * STRIDE + pidx<float>(e)], inv);
    }
}

// Four-step N = N1 x N2 (x as N1 rows of N2): column pass.  A CTA takes S consecutive columns c0.. of signal
// blockIdx.y, runs FFT_N1 down each, multiplies output k1 of column c by W_N^(c k1) and stores column c
// contiguously at out[c N1 + k1].
template <int MODE, int N1, int S>
__global__ void __launch_bounds__(512, 1) k_tc_cols(const tc_fs_args a)
{
    constexpr int STRIDE = padded_len<float>(N1);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<float>* bufA = reinterpret_cast<cpx<float>*>(smem_raw);
    cpx<float>* bufB = bufA + S * STRIDE;
    const int n2 = a.n2;
    const long long n = (long long)N1 * n2;
    const int c0       = blockIdx.x * S;
    const cpx<float>* __restrict__ in = reinterpret_cast<const cpx<float>*>(a.in) + blockIdx.y * n;
    cpx<float>* __restrict__ out      = reinterpret_cast<cpx<float>*>(a.out) + blockIdx.y * n;
    const cpx<float>* twA = reinterpret_cast<const cpx<float>*>(a.twA);
    const cpx<float>* twB = reinterpret_cast<const cpx<float>*>(a.twB);
    const bool inv = a.inverse != 0;
    const tc_frags<MODE> F(a.cs);
    for (int i = threadIdx.x; i < N1 * S; i += blockDim.x)
    {
        const int r = i / S, c = i - r * S;
        bufA[c * STRIDE + pidx<float>(r)] = conj_if(in[(long long)r * n2 + c0 + c], inv);
    }
    __syncthreads();
    const cpx<float>* res = tc_block_fft<MODE, N1>(bufA, bufB, S, STRIDE, reinterpret_cast<const cpx<float>*>(a.tw1), F);
    for (int i = threadIdx.x; i < S * N1; i += blockDim.x)
    {
        const int c = i / N1, k1 = i - c * N1;
        const cpx<float> v = res[c * STRIDE + pidx<float>(k1)] * twiddle_2level(twA, twB, (long long)(c0 + c) * k1, a.lbits);
        out[(long long)(c0 + c) * N1 + k1] = v;
    }
}

// Four-step row pass: a CTA takes S consecutive k1 of signal blockIdx.y, reads element col of row k1 at
// in[col N1 + k1] (the column pass's output), runs FFT_N2 and stores X[k1 + N1 k2].
template <int MODE, int N2, int S>
__global__ void __launch_bounds__(512, 1) k_tc_rows(const tc_fs_args a)
{
    constexpr int STRIDE = padded_len<float>(N2);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<float>* bufA = reinterpret_cast<cpx<float>*>(smem_raw);
    cpx<float>* bufB = bufA + S * STRIDE;
    const int n1 = a.n1;
    const long long n = (long long)n1 * N2;
    const int k0       = blockIdx.x * S;
    const cpx<float>* __restrict__ in = reinterpret_cast<const cpx<float>*>(a.in) + blockIdx.y * n;
    cpx<float>* __restrict__ out      = reinterpret_cast<cpx<float>*>(a.out) + blockIdx.y * n;
    const bool inv = a.inverse != 0;
    const tc_frags<MODE> F(a.cs);
    for (int i = threadIdx.x; i < N2 * S; i += blockDim.x)
    {
        const int col = i / S, j = i - col * S;
        bufA[j * STRIDE + pidx<float>(col)] = in[(long long)col * n1 + k0 + j];
    }
    __syncthreads();
    const cpx<float>* res = tc_block_fft<MODE, N2>(bufA, bufB, S, STRIDE, reinterpret_cast<const cpx<float>*>(a.tw2), F);
    for (int i = threadIdx.x; i < N2 * S; i += blockDim.x)
    {
        const int k2 = i / S, j = i - k2 * S;
        out[k0 + j + (long long)n1 * k2] = conj_if(res[j * STRIDE + pidx<float>(k2)], inv);
    }
}

// columns (rows) per CTA of a pass of length L: two ping-pong buffers in at most 160 KB
constexpr int tc_tile(int L) { return L == 256 ? 16 : 2; }

template <class K>
cudaError_t go_tc(K kernel, dim3 grid, int smem, cudaStream_t st, const tc_fs_args& a)
{
    const cudaError_t e = prepare_launch(reinterpret_cast<const void*>(kernel), 512, smem);
    if (e != cudaSuccess)
        return e;
    kernel<<<grid, 512, smem, st>>>(a);
    return cudaGetLastError();
}

template <int MODE>
cudaError_t launch_tc_pass(const tc_fs_args& a, bool cols, cudaStream_t st)
{
    const int L = cols ? a.n1 : a.n2;
    const int other = cols ? a.n2 : a.n1;
    if ((L != 256 && L != 4096) || a.batch > 65535)
        return cudaErrorInvalidValue;
    const int S = tc_tile(L);
    if (other % S)
        return cudaErrorInvalidValue;
    const dim3 grid(unsigned(other / S), unsigned(a.batch));
    const int smem = 2 * S * padded_len<float>(L) * 8;
    if (cols)
        return L == 256 ? go_tc(k_tc_cols<MODE, 256, tc_tile(256)>, grid, smem, st, a)
                        : go_tc(k_tc_cols<MODE, 4096, tc_tile(4096)>, grid, smem, st, a);
    return L == 256 ? go_tc(k_tc_rows<MODE, 256, tc_tile(256)>, grid, smem, st, a)
                    : go_tc(k_tc_rows<MODE, 4096, tc_tile(4096)>, grid, smem, st, a);
}

} // namespace

cudaError_t launch_c2c_tc_f32(const c2c_args& a, int n, int mode, const float* cs, cudaStream_t st)
{
    const int stride = padded_len<float>(n);
    const int spc    = n == 256 ? 8 : 2;
    const int smem   = 2 * spc * stride * 8;
    const unsigned grid = unsigned((a.batch + spc - 1) / spc);
    auto go = [&](auto kernel) -> cudaError_t
    {
        const cudaError_t e = prepare_launch(reinterpret_cast<const void*>(kernel), 512, smem);
        if (e != cudaSuccess)
            return e;
        kernel<<<grid, 512, smem, st>>>(a, cs, spc);
        return cudaGetLastError();
    };
    if (mode == TC_BF16)
        return n == 256 ? go(k_c2c_tc<TC_BF16, 256>) : go(k_c2c_tc<TC_BF16, 4096>);
    return n == 256 ? go(k_c2c_tc<TC_FP16, 256>) : go(k_c2c_tc<TC_FP16, 4096>);
}

cudaError_t launch_tc_fourstep_pass_f32(const tc_fs_args& a, bool cols, int mode, cudaStream_t st)
{
    return mode == TC_BF16 ? launch_tc_pass<TC_BF16>(a, cols, st) : launch_tc_pass<TC_FP16>(a, cols, st);
}

} // namespace kfr_gpu
