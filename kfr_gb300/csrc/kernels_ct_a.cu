// Compile-time specialised single-precision kernels: complex DFT and one-CTA Bluestein (ct_table.hpp).
#include "kernels.cuh"

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

} // namespace kfr_gpu
