// Single-precision (c32) instantiation of the transform kernels.
#include "kernels.cuh"

namespace kfr_gpu
{
KFR_GPU_INSTANTIATE(float)
} // namespace kfr_gpu
