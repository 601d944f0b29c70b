// kfr_dft_execute_static_scratch_f32: complex c32 DFT execution that allocates nothing.
//
// Who needs it: callers that may not allocate GPU memory while they run, such as real-time audio or control
// threads, code recorded inside CUDA stream capture, and hosts that reserve all device memory at start-up.
// The regular entry points allocate plan-owned scratch the first time a long (two-pass) or multi-kernel
// Bluestein plan runs, and staging buffers for host pointers.  This entry point instead takes the scratch
// from one fixed device array defined below, which every GPU that runs this library keeps until the process
// exits, so its size is a modest, stated maximum (KFR_STATIC_SCRATCH_BYTES in include/kfr_capi.h).
//
// The array's name is only a host-side stand-in in host code: its device address comes from
// cudaGetSymbolAddress, looked up once per device (with that device current) on the first call there,
// whatever the plan.  The CUDA driver loads device code lazily, one compiled module at a time, on a kernel's
// first launch, and loading takes device memory: so run each plan once through this entry point, with the
// batch it will use, before stream capture or real-time use.  All calls share the array; none needs it
// zeroed (each pass writes every scratch element it later reads), and calls that overlap on the GPU race
// on it.
#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>

#include "kfr_capi.h"
#include "plan.hpp"

namespace kfr_gpu
{
void run_static_scratch_f32(void* plan, size_t batch, void* out, const void* in, bool inverse, void* stream,
                            void* (*scratch_of)(), size_t scratch_limit);
} // namespace kfr_gpu

namespace
{

static __device__ __align__(256) unsigned char g_static_scratch[KFR_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device (set-up on first use per device).
void* static_scratch_address()
{
    int dev = 0;
    kfr_gpu::check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        throw std::invalid_argument("device ordinal " + std::to_string(dev) + " is out of range for the static scratch");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_addr[dev])
    {
        void* p = nullptr;
        kfr_gpu::check(cudaGetSymbolAddress(&p, g_static_scratch), "cudaGetSymbolAddress(static scratch)");
        g_scratch_addr[dev] = p;
    }
    return g_scratch_addr[dev];
}

} // namespace

extern "C" KFR_API_SPEC void kfr_dft_execute_static_scratch_f32(KFR_DFT_PLAN_F32* plan, size_t batch, kfr_c32* out,
                                                                const kfr_c32* in, kfr_bool inverse, void* stream)
{
    kfr_gpu::run_static_scratch_f32(plan, batch, out, in, inverse, stream, &static_scratch_address,
                                    KFR_STATIC_SCRATCH_BYTES);
}
