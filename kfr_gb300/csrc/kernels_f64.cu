// Double-precision (c64) instantiation of the transform kernels.
#include "kernels.cuh"

namespace kfr_gpu
{
KFR_GPU_INSTANTIATE(double)

int max_threads_for(int elem_bytes, int ept) { return (elem_bytes == 4 ? 1024 : 512) / (ept / 16); }

int max_smem_bytes()
{
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return 227 * 1024;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0)
        return 227 * 1024;
    return v;
}
} // namespace kfr_gpu
