// Compile-time specialised single-precision kernels: complex DFT and one-CTA Bluestein (ct_table.hpp).
#include "kernels.cuh"

#include <algorithm>

namespace kfr_gpu
{

cudaError_t launch_ct_c2c_f32(const c2c_args& a, const block_cfg& c, cudaStream_t st)
{
#define CT_KERNEL k_c2c
#define CT_GRID KFR_GPU_GRID1
#define CT_ARGS a, c.ts, c.spc
    switch (c.ct)
    {
        KFR_CT_C2C_F32(KFR_GPU_CT_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef CT_KERNEL
#undef CT_GRID
#undef CT_ARGS
}

cudaError_t launch_ct_bluestein_f32(const bluestein_args& a, const block_cfg& c, cudaStream_t st)
{
#define CT_KERNEL k_bluestein
#define CT_GRID KFR_GPU_GRID1
#define CT_ARGS a, c.ts, c.spc
    switch (c.ct)
    {
        KFR_CT_BLUESTEIN_F32(KFR_GPU_CT_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef CT_KERNEL
#undef CT_GRID
#undef CT_ARGS
}

cudaError_t launch_ct_rader_f32(const rader_args& a, const block_cfg& c, cudaStream_t st)
{
#define CT_KERNEL k_rader
#define CT_GRID KFR_GPU_GRID1
#define CT_ARGS a, c.ts, c.spc
    switch (c.ct)
    {
        KFR_CT_RADER_F32(KFR_GPU_CT_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef CT_KERNEL
#undef CT_GRID
#undef CT_ARGS
}

// Persistent launch: as many CTAs as fit on the device at once, capped by the number of tiles.
template <typename K, typename... Args>
static cudaError_t go_persistent(K kernel, const block_cfg& c, long long ntiles, cudaStream_t st, Args... args)
{
    int per_sm    = 0;
    cudaError_t e = prepare_launch(reinterpret_cast<const void*>(kernel), c.threads, c.smem, &per_sm);
    if (e != cudaSuccess)
        return e;
    const int sms = device_sm_count();
    if (per_sm < 1 || sms < 1)
        return cudaErrorInvalidConfiguration;
    const long long grid = std::min<long long>(ntiles, (long long)per_sm * sms);
    kernel<<<unsigned(grid), c.threads, c.smem, st>>>(args...);
    return cudaGetLastError();
}

cudaError_t launch_ct_c2c_pipe_f32(const c2c_args& a0, const block_cfg& c, long long ntiles, int* err, cudaStream_t st)
{
    c2c_args a   = a0;
    a.wait_spins = wait_limit();
#define KFR_GPU_PIPE_CASE(N, TS, ...)                                                                      \
    case N:                                                                                                \
        return go_persistent(k_c2c_pipe<float, ct_fft<float, N, TS, __VA_ARGS__>>, c, ntiles, st, a, ntiles, c.spc, err);
    switch (c.ct)
    {
        KFR_CT_C2C_F32(KFR_GPU_PIPE_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef KFR_GPU_PIPE_CASE
}

// one signal per CTA, persistent: built for the lengths whose three-tile pipeline does not fit (8192 and up)
template <class F>
static cudaError_t go_reg(const c2c_args& a, const block_cfg& c, long long nsig, int* err, cudaStream_t st)
{
    if constexpr (F::n >= 8192)
        return go_persistent(k_c2c_reg<float, F>, c, nsig, st, a, nsig, err);
    else
        return cudaErrorInvalidValue;
}

cudaError_t launch_ct_c2c_reg_f32(const c2c_args& a0, const block_cfg& c, long long nsig, int* err, cudaStream_t st)
{
    c2c_args a   = a0;
    a.wait_spins = wait_limit();
#define KFR_GPU_REG_CASE(N, TS, ...)                                                                       \
    case N: return go_reg<ct_fft<float, N, TS, __VA_ARGS__>>(a, c, nsig, err, st);
    switch (c.ct)
    {
        KFR_CT_C2C_F32(KFR_GPU_REG_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef KFR_GPU_REG_CASE
}

cudaError_t launch_ct_r2c_pipe_f32(const real_args& a0, const block_cfg& c, long long ntiles, int* err, cudaStream_t st)
{
    real_args a  = a0;
    a.wait_spins = wait_limit();
#define KFR_GPU_R2C_PIPE_CASE(N, TS, ...)                                                                  \
    case N:                                                                                                \
        return go_persistent(k_r2c_pipe<float, ct_fft<float, N, TS, __VA_ARGS__>>, c, ntiles, st, a, ntiles, c.spc, err);
    switch (c.ct)
    {
        KFR_CT_REAL_F32(KFR_GPU_R2C_PIPE_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef KFR_GPU_R2C_PIPE_CASE
}

cudaError_t launch_ct_c2r_pipe_f32(const real_args& a0, const block_cfg& c, long long ntiles, int* err, cudaStream_t st)
{
    real_args a  = a0;
    a.wait_spins = wait_limit();
#define KFR_GPU_C2R_PIPE_CASE(N, TS, ...)                                                                  \
    case N:                                                                                                \
        return go_persistent(k_c2r_pipe<float, ct_fft<float, N, TS, __VA_ARGS__>>, c, ntiles, st, a, ntiles, c.spc, err);
    switch (c.ct)
    {
        KFR_CT_REAL_F32(KFR_GPU_C2R_PIPE_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef KFR_GPU_C2R_PIPE_CASE
}

cudaError_t launch_ct_dct_pipe_f32(const dct_args& a0, const block_cfg& c, long long ntiles, int* err, bool inverse,
                                   cudaStream_t st)
{
    dct_args a   = a0;
    a.wait_spins = wait_limit();
#define KFR_GPU_DCT_PIPE_CASE(N, TS, ...)                                                                  \
    case N:                                                                                                \
        return inverse ? go_persistent(k_dct_pipe<float, ct_fft<float, N, TS, __VA_ARGS__>, true>, c, ntiles, st, a, \
                                       ntiles, c.spc, err)                                                 \
                       : go_persistent(k_dct_pipe<float, ct_fft<float, N, TS, __VA_ARGS__>, false>, c, ntiles, st, a, \
                                       ntiles, c.spc, err);
    switch (c.ct)
    {
        KFR_CT_DCT_F32(KFR_GPU_DCT_PIPE_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef KFR_GPU_DCT_PIPE_CASE
}


} // namespace kfr_gpu
