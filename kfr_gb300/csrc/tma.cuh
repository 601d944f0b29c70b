// Bulk asynchronous copies (TMA, cp.async.bulk) and mbarriers, as inline PTX for sm_103a.
//
// Every wait is bounded: mbar_wait gives up after a given number of try_wait rounds (each of which itself
// suspends for a bounded, hardware-defined time; kMbarSpins by default) and reports failure, so a kernel can
// record an error, let its own copies in flight land and return instead of spinning forever.
#pragma once

#include <cstdint>

namespace kfr_gpu
{

constexpr uint32_t kMbarSpins = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes initialised mbarriers visible to the async proxy (TMA).
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Bounded wait for the phase with the given parity to complete (at most `spins` try_wait rounds).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t spins = kMbarSpins)
{
    for (uint32_t i = 0; i < spins; i++)
        if (mbar_try_wait(bar, parity))
            return true;
    return false;
}

// Orders this thread's generic-proxy shared-memory accesses before later async-proxy (TMA) accesses.
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Global -> shared bulk copy completing on `bar` (bytes and both addresses multiples of 16).
__device__ __forceinline__ void bulk_g2s(void* dst_smem, const void* src_gmem, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst_smem)),
                 "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Opaque 128-byte tensor map (the CUDA driver API's CUtensorMap layout), passed to kernels as a __grid_constant__
// parameter.
struct alignas(128) tensor_map
{
    unsigned long long opaque[16];
};

// Global -> shared tiled copy of the 2-D box at element coordinates (x, y) of the tensor map, completing on
// `bar`.  x * element size must be a multiple of 16 bytes; out-of-range elements read as zero.
__device__ __forceinline__ void tensor_g2s_2d(void* dst_smem, const tensor_map* tm, int x, int y, uint64_t* bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                 "[%4];" ::"r"(smem_u32(dst_smem)),
                 "l"(tm), "r"(x), "r"(y), "r"(smem_u32(bar))
                 : "memory");
}

// Shared -> global tiled copy of a 2-D box in this thread's bulk async-group (x, y >= 0; x * element size a
// multiple of 16 bytes).  The writes to the source must be ordered before it by fence_proxy_async_smem() and
// a barrier.
__device__ __forceinline__ void tensor_s2g_2d(const tensor_map* tm, int x, int y, const void* src_smem)
{
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(tm), "r"(x),
                 "r"(y), "r"(smem_u32(src_smem))
                 : "memory");
}

// Element (row, col) of a box whose rows hold S 8-byte elements (S = 16, 8 or 4: 128-, 64- or 32-byte rows), as
// laid out in shared memory by the matching swizzle of 16-byte chunks: chunk c / 2 of row `row` lands at chunk
// (c / 2) ^ (row % 8) (128-byte swizzle), ^ ((row / 2) % 4) (64-byte) or ^ ((row / 4) % 2) (32-byte).  The box
// must start on a 1024-byte boundary.
// S = 2 (16-byte rows) is not swizzled.
template <int S>
__device__ __forceinline__ int swz_8b(int row, int col)
{
    static_assert(S == 16 || S == 8 || S == 4 || S == 2, "16, 8, 4 or 2 elements per row");
    if constexpr (S == 16)
        return row * 16 + (col ^ ((row & 7) << 1));
    else if constexpr (S == 8)
        return row * 8 + (col ^ (((row >> 1) & 3) << 1));
    else if constexpr (S == 4)
        return row * 4 + (col ^ (((row >> 2) & 1) << 1));
    else
        return row * 2 + col;
}

// Shared -> global bulk copy in this thread's bulk async-group (bytes and both addresses multiples of 16).
// The writes to the source must be ordered before it by fence_proxy_async_smem() and a barrier.
__device__ __forceinline__ void bulk_s2g(void* dst_gmem, const void* src_smem, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst_gmem), "r"(smem_u32(src_smem)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Waits until this thread's committed bulk stores have finished reading shared memory (the source may be
// overwritten afterwards).
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// Waits until this thread's committed bulk stores have completed.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

} // namespace kfr_gpu
