// Compile-time specialised single-precision kernels: fused real DFT and DCT (ct_table.hpp).
#include "kernels.cuh"

namespace kfr_gpu
{

#define CT_GRID KFR_GPU_GRID1
#define CT_ARGS a, c.ts, c.spc

cudaError_t launch_ct_r2c_f32(const real_args& a, const block_cfg& c, cudaStream_t st)
{
#define CT_KERNEL k_r2c
    switch (c.ct)
    {
        KFR_CT_REAL_F32(KFR_GPU_CT_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef CT_KERNEL
}

cudaError_t launch_ct_c2r_f32(const real_args& a, const block_cfg& c, cudaStream_t st)
{
#define CT_KERNEL k_c2r
    switch (c.ct)
    {
        KFR_CT_REAL_F32(KFR_GPU_CT_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef CT_KERNEL
}

cudaError_t launch_ct_dct2_f32(const dct_args& a, const block_cfg& c, cudaStream_t st)
{
#define CT_KERNEL k_dct2
    switch (c.ct)
    {
        KFR_CT_DCT_F32(KFR_GPU_CT_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef CT_KERNEL
}

cudaError_t launch_ct_dct3_f32(const dct_args& a, const block_cfg& c, cudaStream_t st)
{
#define CT_KERNEL k_dct3
    switch (c.ct)
    {
        KFR_CT_DCT_F32(KFR_GPU_CT_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef CT_KERNEL
}

#undef CT_GRID
#undef CT_ARGS

} // namespace kfr_gpu
