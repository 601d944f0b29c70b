// Lengths with compile-time specialised block FFTs (single precision).  Each entry is
//   X(N, TS, radices...)   N = product of the radices, TS = threads per signal
// chosen so that no thread holds more than 18 complex values in any pass.  The planner uses an entry when
// the kernel kind and length match (block_program::build then lays the twiddles out in this radix order);
// every other length runs the runtime-radix kernel.  Lists are per kernel kind to bound compile time:
// they cover the parity and benchmark configurations and the power-of-two lengths up to 16384.
#pragma once

// complex DFT of one-CTA lengths (dft_plan<float>)
#define KFR_CT_C2C_F32(X)                                                                                   \
    X(64, 4, 16, 4)                                                                                          \
    X(128, 8, 16, 8)                                                                                         \
    X(256, 16, 16, 16)                                                                                       \
    X(512, 64, 8, 8, 8)                                                                                      \
    X(1000, 100, 10, 10, 10)                                                                                 \
    X(1024, 64, 16, 16, 4)                                                                                   \
    X(1536, 96, 16, 16, 6)                                                                                   \
    X(2048, 128, 16, 16, 8)                                                                                  \
    X(2187, 243, 9, 9, 9, 3)                                                                                 \
    X(4096, 256, 16, 16, 16)                                                                                 \
    X(8192, 512, 16, 16, 16, 2)                                                                              \
    X(16384, 1024, 16, 16, 16, 4)

// convolution lengths M = next_pow2(2N - 1) of the one-CTA Bluestein kernel (any N with that M)
#define KFR_CT_BLUESTEIN_F32(X)                                                                             \
    X(256, 16, 16, 16)                                                                                       \
    X(512, 64, 8, 8, 8)                                                                                      \
    X(1024, 64, 16, 16, 4)                                                                                   \
    X(2048, 128, 16, 16, 8)                                                                                  \
    X(4096, 256, 16, 16, 16)                                                                                 \
    X(8192, 512, 16, 16, 16, 2)                                                                              \
    X(16384, 1024, 16, 16, 16, 4)

// convolution lengths L = n - 1 of the one-CTA Rader kernels for prime n (127, 8191); 14 and 10 are the
// Good-Thomas composite codelets
#define KFR_CT_RADER_F32(X)                                                                                 \
    X(126, 9, 14, 9)                                                                                         \
    X(8190, 1024, 13, 9, 14, 5)

// four-step pass lengths (columns and rows): the factors of 30720 = 160 x 192, of the power-of-two lengths
// 2^15 .. 2^24, of the real-DFT half lengths 22050 = 147 x 150 and 24000 = 150 x 160 (N = 44100, 48000) and
// of 30,720,000 = 5120 x 6000
#define KFR_CT_FOURSTEP_F32(X)                                                                              \
    X(147, 21, 7, 7, 3)                                                                                      \
    X(150, 15, 10, 15)                                                                                       \
    X(5120, 512, 16, 16, 4, 5)                                                                               \
    X(6000, 400, 16, 15, 5, 5)                                                                               \
    X(128, 8, 16, 8)                                                                                         \
    X(160, 16, 16, 10)                                                                                       \
    X(192, 16, 16, 12)                                                                                       \
    X(256, 16, 16, 16)                                                                                       \
    X(512, 64, 8, 8, 8)                                                                                      \
    X(1024, 64, 16, 16, 4)                                                                                   \
    X(2048, 128, 16, 16, 8)                                                                                  \
    X(4096, 256, 16, 16, 16)

// half lengths c = N/2 of the fused real DFT (dft_plan_real<float>): N = 1920, 2048, 4096, 8192
#define KFR_CT_REAL_F32(X)                                                                                  \
    X(960, 96, 16, 6, 10)                                                                                    \
    X(1024, 64, 16, 16, 4)                                                                                   \
    X(2048, 128, 16, 16, 8)                                                                                  \
    X(4096, 256, 16, 16, 16)

// DCT lengths (dct_plan<float>)
#define KFR_CT_DCT_F32(X)                                                                                   \
    X(512, 64, 8, 8, 8)                                                                                      \
    X(1024, 64, 16, 16, 4)                                                                                   \
    X(4096, 256, 16, 16, 16)

// half FFT lengths c = F/2 of the overlap-save convolution kernel (F = 2048, 4096, 8192)
#define KFR_CT_CONV_F32(X)                                                                                  \
    X(1024, 64, 16, 16, 4)                                                                                   \
    X(2048, 128, 16, 16, 8)                                                                                  \
    X(4096, 256, 16, 16, 16)

// four-step splits whose two passes run as fully compile-time kernels (both lengths, the tiles and the
// twiddle table split fold to constants): X(n1, n2), each a KFR_CT_FOURSTEP length
#define KFR_CT_FSPAIR_F32(X)                                                                                \
    X(160, 192)                                                                                              \
    X(256, 256)                                                                                              \
    X(512, 512)                                                                                              \
    X(1024, 1024)                                                                                            \
    X(147, 150)                                                                                              \
    X(150, 160)                                                                                              \
    X(2048, 2048)                                                                                            \
    X(4096, 4096)

// Shared-memory layout of a compile-time length (single precision): X(N, TS, pad shift, extra group stride).
// Element i of a signal sits at i + (i >> shift) (shift 0: unpadded), signals of a CTA lie `stride` elements
// apart, stride = N + (N >> shift) + 1 + extra.  The default (shift 4, extra 0) suits power-of-two strides;
// these entries were chosen with a wavefront model of every pass's accesses (odd radices do best unpadded).
#define KFR_CT_LAYOUT_F32(X)                                                                                \
    X(126, 9, 0, 10)                                                                                         \
    X(1000, 100, 0, 11)                                                                                      \
    X(2187, 243, 0, 7)                                                                                       \
    X(8190, 1024, 0, 0)

#if defined(__CUDACC__)
#define KFR_CT_HD __host__ __device__
#else
#define KFR_CT_HD
#endif

namespace kfr_gpu
{
// b^e mod m (m < 2^31)
KFR_CT_HD constexpr long long powmod_ll(long long b, long long e, long long m)
{
    long long r = 1;
    b %= m;
    while (e > 0)
    {
        if (e & 1)
            r = r * b % m;
        b = b * b % m;
        e >>= 1;
    }
    return r;
}

// smallest primitive root of the prime n (the generator of Rader's permutation, shared by the planner and
// the compile-time kernels)
KFR_CT_HD constexpr long long primitive_root(long long n)
{
    const long long L = n - 1;
    for (long long g = 2; g < n; g++)
    {
        bool ok = true;
        long long x = L;
        for (long long p = 2; p * p <= x && ok; p++)
            if (x % p == 0)
            {
                if (powmod_ll(g, L / p, n) == 1)
                    ok = false;
                while (x % p == 0)
                    x /= p;
            }
        if (ok && x > 1 && powmod_ll(g, L / x, n) == 1)
            ok = false;
        if (ok)
            return g;
    }
    return 1;
}
} // namespace kfr_gpu

namespace kfr_gpu
{
KFR_CT_HD constexpr int ct_pad_shift_f32(int n, int ts)
{
#define KFR_CT_LAYOUT_SHIFT(N, TS, S, E)                                                                   \
    if (n == N && ts == TS)                                                                                \
        return S;
    KFR_CT_LAYOUT_F32(KFR_CT_LAYOUT_SHIFT)
#undef KFR_CT_LAYOUT_SHIFT
    return 4;
}
KFR_CT_HD constexpr int ct_group_stride_f32(int n, int ts)
{
#define KFR_CT_LAYOUT_STRIDE(N, TS, S, E)                                                                  \
    if (n == N && ts == TS)                                                                                \
        return n + (S ? (n >> S) : 0) + 1 + E;
    KFR_CT_LAYOUT_F32(KFR_CT_LAYOUT_STRIDE)
#undef KFR_CT_LAYOUT_STRIDE
    return n + (n >> 4) + 1;
}
} // namespace kfr_gpu

namespace kfr_gpu
{
// Tile (signals per CTA) of a compile-time four-step pass run ping-pong: the largest power of two <= 16 whose
// threads fit 1024 and whose two buffers fit `smem` bytes; 0 if fewer than 8 fit (the strided passes then
// take the in-place kernels).
KFR_CT_HD constexpr int fsp_tile(int n, int ts, int smem)
{
    int s = 16;
    while (s > 1 && (s * ts > 1024 || 2 * s * ct_group_stride_f32(n, ts) * 8 > smem))
        s /= 2;
    return s >= 8 ? s : 0;
}
// Shared memory the compile-time pair kernels are built for (the sm_103a per-block opt-in maximum less the
// static reserve).
constexpr int kFspSmem = 227 * 1024 - 2048;
} // namespace kfr_gpu
