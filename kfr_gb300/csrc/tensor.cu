// Radix-16 passes as tensor-core contractions (warp-level mma.sync, m16n8k16, FP32 accumulation) with split
// hi + lo operands, for lengths 16^k that fit one CTA.
//
// One radix-16 butterfly is y = F16 u (u: the 16 twiddled inputs, F16[k][r] = e^{-2 pi i k r / 16}).  In real
// arithmetic, with F16 = C - iS:
//     [Re y]   [ C  S ] [Re u]
//     [Im y] = [-S  C ] [Im u]          (32 x 32 times 32 x 8 for eight butterflies)
// computed as four 16 x 16 x 8 tiles.  Each operand is split into a high and a low part in the 16-bit format
// (BF16 or FP16): x = hi + lo, hi = round(x), lo = round(x - hi); the product keeps hi*hi + hi*lo + lo*hi
// (three tensor-core products per tile, accumulated in FP32) and drops lo*lo.  Inputs are scaled by 1/16 per
// pass (exact) so that FP16 operands stay in range; the final store undoes it (x 16^passes, exact).
#include "kernels.cuh"
#include "tensor.hpp"

#include <cuda_bf16.h>
#include <cuda_fp16.h>

namespace kfr_gpu
{

template <int MODE>
__device__ __forceinline__ void split_pair(float a, float b, uint32_t& hi, uint32_t& lo)
{
    if constexpr (MODE == TC_BF16)
    {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        const float2 hf        = __bfloat1622float2(h);
        const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
        hi                     = *reinterpret_cast<const uint32_t*>(&h);
        lo                     = *reinterpret_cast<const uint32_t*>(&l);
    }
    else
    {
        const __half2 h  = __floats2half2_rn(a, b);
        const float2 hf  = __half22float2(h);
        const __half2 l  = __floats2half2_rn(a - hf.x, b - hf.y);
        hi               = *reinterpret_cast<const uint32_t*>(&h);
        lo               = *reinterpret_cast<const uint32_t*>(&l);
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

template <int MODE, int N>
__global__ void __launch_bounds__(512, 1) k_c2c_tc(const c2c_args a, const float* __restrict__ cs, const int spc)
{
    constexpr int R      = 16;
    constexpr int NBF    = N / R;
    constexpr int TILES  = NBF / 8; // tiles of eight butterflies per signal and pass
    constexpr int STRIDE = padded_len<float>(N);
    constexpr int P      = N == 256 ? 2 : N == 4096 ? 3 : 1;
    static_assert(N == 256 || N == 4096, "lengths 16^2 and 16^3");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<float>* bufA = reinterpret_cast<cpx<float>*>(smem_raw);
    cpx<float>* bufB = bufA + spc * STRIDE;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int g = lane >> 2, q = lane & 3;
    const long long s0 = (long long)blockIdx.x * spc;
    const cpx<float>* __restrict__ in = reinterpret_cast<const cpx<float>*>(a.in);
    cpx<float>* __restrict__ out      = reinterpret_cast<cpx<float>*>(a.out);
    const cpx<float>* __restrict__ tw = reinterpret_cast<const cpx<float>*>(a.tw);
    const bool inv = a.inverse != 0;
    const int nsig = a.batch - s0 < spc ? int(a.batch - s0) : spc;
    // A fragments of C (cos) and S (sin), row k = output, column r = input: rows g, g+8; columns 2q.., 2q+8..
    uint32_t Ch[4], Cl[4], Sh[4], Sl[4];
    {
        const int rows[4] = { g, g + 8, g, g + 8 };
        const int cols[4] = { 2 * q, 2 * q, 2 * q + 8, 2 * q + 8 };
#pragma unroll
        for (int i = 0; i < 4; i++)
        {
            split_pair<MODE>(cs[rows[i] * 16 + cols[i]], cs[rows[i] * 16 + cols[i] + 1], Ch[i], Cl[i]);
            split_pair<MODE>(cs[256 + rows[i] * 16 + cols[i]], cs[256 + rows[i] * 16 + cols[i] + 1], Sh[i], Sl[i]);
        }
    }
    uint32_t nSh[4], nSl[4];
#pragma unroll
    for (int i = 0; i < 4; i++)
    {
        nSh[i] = neg_pair(Sh[i]);
        nSl[i] = neg_pair(Sl[i]);
    }
    for (int i = threadIdx.x; i < nsig * N; i += blockDim.x)
    {
        const int s = i / N, e = i - s * N;
        bufA[s * STRIDE + pidx<float>(e)] = conj_if(in[(s0 + s) * a.istride + e], inv);
    }
    __syncthreads();
    cpx<float>* src = bufA;
    cpx<float>* dst = bufB;
    int ns = 1, twoff = 0;
#pragma unroll 1
    for (int p = 0; p < P; p++)
    {
        for (int t = warp; t < nsig * TILES; t += nwarps)
        {
            const int s = t / TILES, j0 = (t - s * TILES) * 8;
            const cpx<float>* sb = src + s * STRIDE;
            // B operands: butterfly j0 + g, inputs r in {2q, 2q+1, 2q+8, 2q+9}, twiddled and scaled by 1/16
            const int j = j0 + g, k = j % ns;
            cpx<float> u[4];
            const int rr[4] = { 2 * q, 2 * q + 1, 2 * q + 8, 2 * q + 9 };
#pragma unroll
            for (int i = 0; i < 4; i++)
            {
                cpx<float> v = sb[pidx<float>(j + rr[i] * NBF)];
                if (ns > 1 && rr[i] > 0)
                    v = v * ldg(tw + twoff + (rr[i] - 1) * ns + k);
                u[i] = scale(v, 0.0625f);
            }
            uint32_t bth0, btl0, bth1, btl1, bbh0, bbl0, bbh1, bbl1;
            split_pair<MODE>(u[0].x, u[1].x, bth0, btl0);
            split_pair<MODE>(u[2].x, u[3].x, bth1, btl1);
            split_pair<MODE>(u[0].y, u[1].y, bbh0, bbl0);
            split_pair<MODE>(u[2].y, u[3].y, bbh1, bbl1);
            float top[4] = { 0, 0, 0, 0 }, bot[4] = { 0, 0, 0, 0 };
            // Re y = C Re u + S Im u
            mma16816<MODE>(top, Ch, bth0, bth1);
            mma16816<MODE>(top, Ch, btl0, btl1);
            mma16816<MODE>(top, Cl, bth0, bth1);
            mma16816<MODE>(top, Sh, bbh0, bbh1);
            mma16816<MODE>(top, Sh, bbl0, bbl1);
            mma16816<MODE>(top, Sl, bbh0, bbh1);
            // Im y = -S Re u + C Im u
            mma16816<MODE>(bot, nSh, bth0, bth1);
            mma16816<MODE>(bot, nSh, btl0, btl1);
            mma16816<MODE>(bot, nSl, bth0, bth1);
            mma16816<MODE>(bot, Ch, bbh0, bbh1);
            mma16816<MODE>(bot, Ch, bbl0, bbl1);
            mma16816<MODE>(bot, Cl, bbh0, bbh1);
            // D: outputs k = g (regs 0, 1) and g + 8 (regs 2, 3) of butterflies j0 + 2q and j0 + 2q + 1
            cpx<float>* db = dst + s * STRIDE;
#pragma unroll
            for (int c = 0; c < 2; c++)
            {
                const int bf = j0 + 2 * q + c, kk = bf % ns, d = (bf - kk) * R + kk;
                db[pidx<float>(d + g * ns)]       = mk<float>(top[c], bot[c]);
                db[pidx<float>(d + (g + 8) * ns)] = mk<float>(top[2 + c], bot[2 + c]);
            }
        }
        __syncthreads();
        twoff += ns > 1 ? ns * (R - 1) : 0;
        ns *= R;
        cpx<float>* tmp = src;
        src             = dst;
        dst             = tmp;
    }
    const float unscale = P == 2 ? 256.0f : 4096.0f;
    for (int i = threadIdx.x; i < nsig * N; i += blockDim.x)
    {
        const int s = i / N, e = i - s * N;
        out[(s0 + s) * a.ostride + e] = conj_if(scale(src[s * STRIDE + pidx<float>(e)], unscale), inv);
    }
}

cudaError_t launch_c2c_tc_f32(const c2c_args& a, int n, int mode, const float* cs, cudaStream_t st)
{
    const int stride = padded_len<float>(n);
    const int spc    = n == 256 ? 8 : 2;
    const int smem   = 2 * spc * stride * 8;
    const unsigned grid = unsigned((a.batch + spc - 1) / spc);
    auto go_tc = [&](auto kernel) -> cudaError_t
    {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess)
            return e;
        kernel<<<grid, 512, smem, st>>>(a, cs, spc);
        return cudaGetLastError();
    };
    if (mode == TC_BF16)
        return n == 256 ? go_tc(k_c2c_tc<TC_BF16, 256>) : go_tc(k_c2c_tc<TC_BF16, 4096>);
    return n == 256 ? go_tc(k_c2c_tc<TC_FP16, 256>) : go_tc(k_c2c_tc<TC_FP16, 4096>);
}

} // namespace kfr_gpu
