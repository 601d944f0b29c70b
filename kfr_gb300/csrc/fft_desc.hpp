// Plain descriptors shared by the host planner (g++) and the device kernels (nvcc).
#pragma once

#include <cstdint>

namespace kfr_gpu
{

constexpr int kMaxPasses = 24;

// floor(x / d) for 0 <= x < 2^31 by a 32-bit multiply-high ("round-up" magic number method).
struct fast_div
{
    uint32_t d, m, s;
};

inline fast_div make_fast_div(uint32_t d)
{
    fast_div f;
    f.d = d;
    if (d <= 1)
    {
        f.d = 1;
        f.m = 0;
        f.s = 0;
        return f;
    }
    uint32_t s = 0;
    while ((uint64_t(1) << s) < d)
        s++;
    const uint64_t m = ((uint64_t(1) << (32 + s)) + d - 1) / d;
    f.m              = uint32_t(m - (uint64_t(1) << 32));
    f.s              = s;
    return f;
}

inline uint32_t host_fdiv(uint32_t x, const fast_div& f)
{
    if (f.d == 1)
        return x;
    const uint32_t hi = uint32_t((uint64_t(x) * f.m) >> 32);
    return (hi + ((x - hi) >> 1)) >> (f.s - 1);
}

// Shared-memory slots for an n-point signal of real type T: one spare slot every 16 (8-byte complex) or
// 8 (16-byte complex) slots, plus one.  Must match padded_len / pidx in fft_device.cuh.
template <typename T>
inline int padded_len_host(int n)
{
    return n + (n >> (sizeof(T) == 4 ? 4 : 3)) + 1;
}

// Elements of one stage buffer of the pipelined kernels: the enclosing 16-byte range of a tile of spc
// signals of n elements, or the padded layout of spc work signals (`gstride` apart), whichever is larger,
// rounded up to 128 bytes so that the next buffer stays aligned for bulk copies.
#if defined(__CUDACC__)
__host__ __device__
#endif
    inline constexpr int pipe_stage_len(int spc, int n, int gstride)
{
    return ((((spc * n + 3) / 2 * 2) > spc * gstride ? ((spc * n + 3) / 2 * 2) : spc * gstride) + 15) / 16 * 16;
}

struct pass_desc
{
    int radix;
    int ns;     // product of the radices of earlier passes
    int tw_off; // this pass's twiddles: tw[tw_off + (r-1)*ns + k] = W_{ns*R}^{k*r}
    int wr_off; // generic radix only: tw[wr_off + m] = W_R^m
    fast_div div_ns;
};

struct fft_desc
{
    int n;
    int npass;
    pass_desc pass[kMaxPasses];
};

} // namespace kfr_gpu
