// Tensor-core radix-16 passes with split hi + lo 16-bit operands (tensor.cu).
#pragma once

#include "launch.hpp"

namespace kfr_gpu
{

enum tc_mode
{
    TC_NONE = 0,
    TC_BF16 = 1, // operands split into BF16 hi + lo
    TC_FP16 = 2, // operands split into FP16 hi + lo
};

// Complex DFT of n = 256 or 4096 (all radix-16 passes on the tensor cores); a.tw: the passes' twiddles in the
// block-program layout of radices {16, ...}; cs: 16 x 16 cos then 16 x 16 sin of 2 pi k r / 16 (device).
cudaError_t launch_c2c_tc_f32(const c2c_args& a, int n, int mode, const float* cs, cudaStream_t st);

} // namespace kfr_gpu
