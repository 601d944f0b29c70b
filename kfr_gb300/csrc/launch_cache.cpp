// Per-process cache of the launch bookkeeping that the persistent kernels need on every launch (see
// prepare_launch in launch.hpp).
#include "launch.hpp"

#include <map>
#include <mutex>
#include <tuple>
#include <utility>

namespace kfr_gpu
{

namespace
{
std::mutex g_mu;
// (device, kernel) -> the dynamic shared-memory limit set so far
std::map<std::pair<int, const void*>, int> g_limit;
// (device, kernel, threads, smem) -> blocks per SM
std::map<std::tuple<int, const void*, int, int>, int> g_occupancy;
} // namespace

cudaError_t prepare_launch(const void* kernel, int threads, int smem, int* per_sm)
{
    int dev       = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    std::lock_guard<std::mutex> lock(g_mu);
    if (smem > 48 * 1024)
    {
        const auto lk = std::make_pair(dev, kernel);
        const auto it = g_limit.find(lk);
        if (it == g_limit.end() || it->second < smem)
        {
            if ((e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)) != cudaSuccess)
                return e;
            g_limit[lk] = smem;
        }
    }
    if (per_sm)
    {
        const auto key = std::make_tuple(dev, kernel, threads, smem);
        auto it        = g_occupancy.find(key);
        if (it == g_occupancy.end())
        {
            int n = 0;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, size_t(smem))) != cudaSuccess)
                return e;
            it = g_occupancy.emplace(key, n).first;
        }
        *per_sm = it->second;
    }
    return cudaSuccess;
}

int device_sm_count()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return 0;
    std::lock_guard<std::mutex> lock(g_mu);
    static std::map<int, int> counts;
    auto it = counts.find(dev);
    if (it == counts.end())
    {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
            return 0;
        it = counts.emplace(dev, v).first;
    }
    return it->second;
}

} // namespace kfr_gpu
