// Tensor-core radix-16 passes with split hi + lo 16-bit operands (tensor.cu).
#pragma once

#include "launch.hpp"

namespace kfr_gpu
{

enum tc_mode
{
    TC_NONE = 0,
    TC_BF16 = 1, // operands split into three BF16 parts (hi + mid + lo)
    TC_FP16 = 2, // operands split into FP16 hi + lo after a per-butterfly power-of-two scaling
};

// Complex DFT of n = 256 or 4096 (all radix-16 passes on the tensor cores); a.tw: the passes' twiddles, pass
// with stride ns > 1 at the running offset, entry (r - 1) ns + k = W_{16 ns}^{r k}; cs: 16 x 16 cos then
// 16 x 16 sin of 2 pi k r / 16 (device).
cudaError_t launch_c2c_tc_f32(const c2c_args& a, int n, int mode, const float* cs, cudaStream_t st);

// One pass of the tensor-core four-step N = n1 x n2 (n1, n2 in {256, 4096}), over `batch` contiguous signals:
//   column pass: FFT_n1 down each column, times W_N^(col k1), stored column-contiguous at out[col n1 + k1]
//   row pass:    FFT_n2 along each k1 of the column pass's output, stored at out[k1 + n1 k2]
// inverse: conjugate on the column pass's load and the row pass's store.
struct tc_fs_args
{
    const void* in;
    void* out;
    long long batch;
    int n1, n2;
    int inverse;
    const void* tw1; // twiddles of the n1-point passes (layout as for launch_c2c_tc_f32)
    const void* tw2; // twiddles of the n2-point passes
    const void* twA; // two-level table of W_N^m = twA[m >> lbits] twB[m & (2^lbits - 1)]
    const void* twB;
    int lbits;
    const float* cs; // the DFT-16 matrix as for launch_c2c_tc_f32
};
cudaError_t launch_tc_fourstep_pass_f32(const tc_fs_args& a, bool cols, int mode, cudaStream_t st);

} // namespace kfr_gpu
