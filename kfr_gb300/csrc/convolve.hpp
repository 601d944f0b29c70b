// Whole-signal convolution, correlation and autocorrelation (include/kfr/dft/convolution.hpp:53-76,
// src/dft/convolution-impl.cpp:106-128) and the plan cache they use (dft_cache, include/kfr/dft/cache.hpp).
//
// The reference pads both inputs to size = next_pow2(n1 + n2 - 1) as complex values, runs two complex DFTs, a
// product and an inverse complex DFT, and keeps the real part scaled by 1/size (for complex inputs too: the
// result is truncate(real(...)) at src/dft/convolution-impl.cpp:127).  Here real inputs go through real DFTs
// of the same size (half the work, the same result to rounding); complex inputs take the complex path and keep
// the reference's real-part-only result.
#pragma once

#include <memory>
#include <mutex>

#include "plan.hpp"

namespace kfr_gpu
{

// Process-wide plan cache keyed by (precision, kind, size), guarded by a mutex like dft_cache
// (include/kfr/dft/cache.hpp:54-83).  Plans live until clear() or process exit.
class plan_cache
{
public:
    static plan_cache& instance();
    template <typename T>
    std::shared_ptr<complex_engine<T>> complex(long long n);
    template <typename T>
    std::shared_ptr<real_engine<T>> real(long long n);
    void clear();
    size_t size() const;

private:
    struct entry;
    mutable std::mutex mu_;
    std::vector<std::shared_ptr<entry>> entries_;
};

// out: n1 + n2 - 1 values (complex inputs: complex values whose imaginary parts are zero).  All pointers are
// device pointers; work is enqueued on st.  is_complex: interleaved complex inputs.  mode: 0 convolve,
// 1 correlate (second input reversed, not conjugated, as the reference does).
template <typename T>
void convolve_device(void* out, const void* a, long long na, const void* b, long long nb, bool is_complex, int mode,
                     cudaStream_t st);

// Device scratch bytes convolve_device needs.
template <typename T>
size_t convolve_scratch_bytes(long long na, long long nb, bool is_complex);

} // namespace kfr_gpu
