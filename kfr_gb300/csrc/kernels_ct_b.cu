// Compile-time specialised single-precision kernels: four-step column and row passes (ct_table.hpp).
#include "kernels.cuh"

namespace kfr_gpu
{

cudaError_t launch_ct_fs_cols_f32(const fourstep_args& a, const block_cfg& c, cudaStream_t st)
{
#define CT_KERNEL k_fs_cols
#define CT_GRID KFR_GPU_GRID2
#define CT_ARGS a, c.ts
    switch (c.ct)
    {
        KFR_CT_FOURSTEP_F32(KFR_GPU_CT_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef CT_KERNEL
#undef CT_GRID
#undef CT_ARGS
}

cudaError_t launch_ct_fs_rows_f32(const fourstep_args& a, const block_cfg& c, cudaStream_t st)
{
#define CT_KERNEL k_fs_rows
#define CT_GRID KFR_GPU_GRID2
#define CT_ARGS a, c.ts
    switch (c.ct)
    {
        KFR_CT_FOURSTEP_F32(KFR_GPU_CT_CASE)
    default: return cudaErrorInvalidValue;
    }
#undef CT_KERNEL
#undef CT_GRID
#undef CT_ARGS
}

} // namespace kfr_gpu
