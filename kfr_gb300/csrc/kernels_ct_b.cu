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

template <int N>
struct fs_len;
#define KFR_GPU_FS_LEN(N, TS, ...)                                                                         \
    template <>                                                                                            \
    struct fs_len<N>                                                                                       \
    {                                                                                                      \
        using type = ct_fft<float, N, TS, __VA_ARGS__>;                                                     \
    };
KFR_CT_FOURSTEP_F32(KFR_GPU_FS_LEN)
#undef KFR_GPU_FS_LEN

bool has_ct_fsp_f32(int n1, int n2)
{
#define KFR_GPU_FSP_HAS(A, B)                                                                              \
    if (n1 == A && n2 == B)                                                                                \
        return true;
    KFR_CT_FSPAIR_F32(KFR_GPU_FSP_HAS)
#undef KFR_GPU_FSP_HAS
    return false;
}

template <class K>
static cudaError_t go_fsp(K kernel, dim3 grid, int threads, int smem, cudaStream_t st, const fourstep_args& a)
{
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess)
        return e;
    kernel<<<grid, threads, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_ct_fsp_f32(const fourstep_args& a, bool cols, cudaStream_t st)
{
#define KFR_GPU_FSP_CASE(A, B)                                                                             \
    if (a.n1 == A && a.n2 == B)                                                                            \
    {                                                                                                      \
        using FA = fs_len<A>::type;                                                                        \
        using FB = fs_len<B>::type;                                                                        \
        if (cols)                                                                                          \
        {                                                                                                  \
            constexpr int S = fsp_tile(A, FA::ts, kFspSmem);                                               \
            return go_fsp(k_fsp_cols<float, FA, B>, dim3((B + S - 1) / S, unsigned(a.batch)),              \
                          (S * FA::ts + 31) / 32 * 32, 2 * S * FA::gstride() * 8, st, a);                  \
        }                                                                                                  \
        constexpr int S = fsp_tile(B, FB::ts, kFspSmem);                                                   \
        return go_fsp(k_fsp_rows<float, FB, A>, dim3((A + S - 1) / S, unsigned(a.batch)),                  \
                      (S * FB::ts + 31) / 32 * 32, 2 * S * FB::gstride() * 8, st, a);                      \
    }
    KFR_CT_FSPAIR_F32(KFR_GPU_FSP_CASE)
#undef KFR_GPU_FSP_CASE
    return cudaErrorInvalidValue;
}

} // namespace kfr_gpu
