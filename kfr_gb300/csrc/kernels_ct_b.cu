// Compile-time specialised single-precision kernels: four-step column and row passes (ct_table.hpp).
#include <algorithm>

#include <cuda.h>
#include <cudaTypedefs.h>

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
    const cudaError_t e = prepare_launch(reinterpret_cast<const void*>(kernel), threads, smem);
    if (e != cudaSuccess)
        return e;
    kernel<<<grid, threads, smem, st>>>(a);
    return cudaGetLastError();
}

// cuTensorMapEncodeTiled, looked up once through the runtime's driver entry-point query (no link-time
// dependency on the CUDA driver library)
static PFN_cuTensorMapEncodeTiled_v12000 tensor_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

static_assert(sizeof(tensor_map) == sizeof(CUtensorMap) && alignof(tensor_map) == alignof(CUtensorMap),
              "tensor_map mirrors CUtensorMap");

// 2-D map over `rows` rows of `row_elems` complex single-precision values (as 2 row_elems floats), box of
// S values (S = 16, 8, 4: 128, 64, 32 bytes with the swizzle of that width; 2: 16 bytes, no swizzle) x
// box_rows rows, zero fill out of range.  False when the base address or the row pitch is not a multiple of
// 16 bytes, or the encoder refuses.
static bool map_rows(tensor_map& m, const void* base, long long row_elems, long long rows, int box_rows, int S)
{
    const auto fn = tensor_encoder();
    if (!fn || reinterpret_cast<uintptr_t>(base) % 16 || (row_elems * 8) % 16 || box_rows > 256 || rows < 1 ||
        (S != 16 && S != 8 && S != 4 && S != 2))
        return false;
    const cuuint64_t dims[2]    = { cuuint64_t(2 * row_elems), cuuint64_t(rows) };
    const cuuint64_t strides[1] = { cuuint64_t(row_elems * 8) };
    const cuuint32_t box[2]     = { cuuint32_t(2 * S), cuuint32_t(box_rows) };
    const cuuint32_t estr[2]    = { 1, 1 };
    return fn(reinterpret_cast<CUtensorMap*>(&m), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims,
              strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              S == 16  ? CU_TENSOR_MAP_SWIZZLE_128B
              : S == 8 ? CU_TENSOR_MAP_SWIZZLE_64B
              : S == 4 ? CU_TENSOR_MAP_SWIZZLE_32B
                       : CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <class K, class... Args>
static cudaError_t go_fspt(K kernel, int threads, int smem, long long ntiles, cudaStream_t st, Args... args)
{
    int per_sm    = 0;
    cudaError_t e = prepare_launch(reinterpret_cast<const void*>(kernel), threads, smem, &per_sm);
    if (e != cudaSuccess)
        return e;
    const int sms = device_sm_count();
    if (per_sm < 1 || sms < 1)
        return cudaErrorInvalidConfiguration;
    const long long grid = std::min<long long>(ntiles, (long long)per_sm * sms);
    kernel<<<unsigned(grid), threads, smem, st>>>(args...);
    return cudaGetLastError();
}

// The persistent tensor-copy pair kernels where the length and the buffers allow them; done = false
// otherwise (the caller then launches k_fsp_cols / k_fsp_rows).
template <class FA, int N2, bool RP = false>
static cudaError_t try_fspt_cols(const fourstep_args& a, cudaStream_t st, bool& done)
{
    done = false;
    if constexpr (fspt_ok<FA>())
    {
        constexpr int N1 = FA::n, S = fspt_tile<FA>();
        tensor_map m;
        if (!a.err || a.sig_stride != (long long)N1 * N2 || reinterpret_cast<uintptr_t>(a.out) % 16 ||
            !map_rows(m, a.in, N2, N1 * a.batch, N1 < 256 ? N1 : 256, S))
            return cudaSuccess;
        done = true;
        const long long ntiles = a.batch * ((N2 + S - 1) / S);
        return go_fspt(k_fspt_cols<float, FA, N2, RP>, fspt_threads<FA>(), fspt_smem<FA>(), ntiles, st, a, m, ntiles,
                       a.err);
    }
    return cudaSuccess;
}

// The fused real row pass over the real-fused column layout (rows N1 rounded up to even values apart).
template <class FB, int N1>
static cudaError_t try_fspt_rows_r2c(const fourstep_args& a, cudaStream_t st, bool& done)
{
    done = false;
    if constexpr (fspt_ok<FB>() && FB::npass == 2 && fspt_tile<FB>() % 2 == 0)
    {
        constexpr int N2 = FB::n, S = fspt_tile<FB>(), BR = N2 < 256 ? N2 : 256, P1 = N1 + (N1 & 1);
        tensor_map mi;
        if (!a.err || !a.rtw || !map_rows(mi, a.in, P1, N2 * a.batch, BR, S))
            return cudaSuccess;
        done = true;
        const long long ntiles = a.batch * ((P1 + S - 1) / S);
        return go_fspt(k_fspt_rows_r2c<float, FB, N1>, fspt_threads<FB>(), fspt_smem<FB>(), ntiles, st, a, mi, ntiles,
                       a.err);
    }
    return cudaSuccess;
}

template <class FB, int N1>
static cudaError_t try_fspt_rows(const fourstep_args& a, cudaStream_t st, bool& done)
{
    done = false;
    if constexpr (fspt_ok<FB>())
    {
        constexpr int N2 = FB::n, S = fspt_tile<FB>(), BR = N2 < 256 ? N2 : 256;
        // the three-pass kernel stores from its last pass: no output map (the input map fills the slot)
        tensor_map mi, mo;
        if (!a.err || a.sig_stride != (long long)N1 * N2 || !map_rows(mi, a.in, N1, N2 * a.batch, BR, S))
            return cudaSuccess;
        if (FB::npass == 3)
            mo = mi;
        else if (!map_rows(mo, a.out, N1, N2 * a.batch, BR, S))
            return cudaSuccess;
        done = true;
        const long long ntiles = a.batch * ((N1 + S - 1) / S);
        return go_fspt(k_fspt_rows<float, FB, N1>, fspt_threads<FB>(), fspt_smem<FB>(), ntiles, st, a, mi, mo, ntiles,
                       a.err);
    }
    return cudaSuccess;
}

// The per-tile pair kernels where their tiles (at least 8 signals) fit; cudaErrorNotSupported otherwise (the
// caller then runs the generic four-step kernels).
template <class FA, class FB, int A, int B>
static cudaError_t go_fsp_pair(const fourstep_args& a, bool cols, cudaStream_t st)
{
    constexpr int SA = fsp_tile(A, FA::ts, kFspSmem), SB = fsp_tile(B, FB::ts, kFspSmem);
    if (cols)
    {
        if constexpr (SA >= 8)
            return go_fsp(k_fsp_cols<float, FA, B>, dim3((B + SA - 1) / SA, unsigned(a.batch)),
                          (SA * FA::ts + 31) / 32 * 32, 2 * SA * FA::gstride() * 8, st, a);
        else
            return cudaErrorNotSupported;
    }
    if constexpr (SB >= 8)
        return go_fsp(k_fsp_rows<float, FB, A>, dim3((A + SB - 1) / SB, unsigned(a.batch)),
                      (SB * FB::ts + 31) / 32 * 32, 2 * SB * FB::gstride() * 8, st, a);
    else
        return cudaErrorNotSupported;
}

bool has_ct_fsp_r2c_f32(int n1, int n2)
{
#define KFR_GPU_FSP_R2C_HAS(A, B)                                                                          \
    if (n1 == A && n2 == B)                                                                                \
        return fspt_ok<fs_len<A>::type>() && fspt_ok<fs_len<B>::type>() && fs_len<B>::type::npass == 2 &&    \
               fspt_tile<fs_len<B>::type>() % 2 == 0 && (B * 8) % 16 == 0;
    KFR_CT_FSPAIR_F32(KFR_GPU_FSP_R2C_HAS)
#undef KFR_GPU_FSP_R2C_HAS
    return false;
}

cudaError_t launch_ct_fsp_r2c_f32(const fourstep_args& a0, bool cols, cudaStream_t st)
{
    fourstep_args a = a0;
    a.wait_spins    = wait_limit();
#define KFR_GPU_FSP_R2C_CASE(A, B)                                                                         \
    if (a.n1 == A && a.n2 == B)                                                                            \
    {                                                                                                      \
        bool done = false;                                                                                 \
        const cudaError_t te = cols ? try_fspt_cols<fs_len<A>::type, B, true>(a, st, done)                   \
                                    : try_fspt_rows_r2c<fs_len<B>::type, A>(a, st, done);                    \
        return te != cudaSuccess ? te : (done ? cudaSuccess : cudaErrorNotSupported);                     \
    }
    KFR_CT_FSPAIR_F32(KFR_GPU_FSP_R2C_CASE)
#undef KFR_GPU_FSP_R2C_CASE
    return cudaErrorNotSupported;
}

cudaError_t launch_ct_fsp_f32(const fourstep_args& a0, bool cols, cudaStream_t st)
{
    fourstep_args a = a0;
    a.wait_spins    = wait_limit();
#define KFR_GPU_FSP_CASE(A, B)                                                                             \
    if (a.n1 == A && a.n2 == B)                                                                            \
    {                                                                                                      \
        using FA = fs_len<A>::type;                                                                        \
        using FB = fs_len<B>::type;                                                                        \
        bool done = false;                                                                                 \
        const cudaError_t te = cols ? try_fspt_cols<FA, B>(a, st, done) : try_fspt_rows<FB, A>(a, st, done);   \
        if (done || te != cudaSuccess)                                                                     \
            return te;                                                                                     \
        return go_fsp_pair<FA, FB, A, B>(a, cols, st);                                                     \
    }
    KFR_CT_FSPAIR_F32(KFR_GPU_FSP_CASE)
#undef KFR_GPU_FSP_CASE
    return cudaErrorInvalidValue;
}

} // namespace kfr_gpu
