// FFT convolution filter: the GPU counterpart of convolve_filter<T> (include/kfr/dft/convolution.hpp:98-148,
// src/dft/convolution-impl.cpp:37-84, 134-228).
//
// The reference streams a uniformly partitioned overlap-add, one block at a time, keeping the FFTs of past
// blocks and the overlap as state.  Its output is the causal FIR convolution of everything passed since
// the last reset(): y[n] = sum_{k<M} h[k] x[n-k].  Here every output block of a process() call is computed
// at once by a batched overlap-save: CTA b takes input samples [b*B - (M-1), b*B + B) (the part before the
// call comes from a device history of the last M-1 samples), runs a real FFT of F = B + M - 1 rounded up to
// a power of two, multiplies by the taps' spectrum (scaled by 1/F, as set_data does), runs the inverse,
// and writes its B valid samples.  State is the M-1 sample history per channel, so results do not depend
// on how the input is split into calls.
#pragma once

#include "plan.hpp"

namespace kfr_gpu
{

struct conv_args
{
    const void* in;    // channels x n samples
    void* out;
    const void* hist;  // channels x (M-1) previous samples
    long long n;       // samples per channel in this call
    long long m1;      // M - 1
    long long bo;      // valid outputs per block
    int channels;
    const void* hspec; // c+1 complex: FFT_F(taps) / F
    const void* rtw;   // W_F^k, k = 0..c
    const void* tw;
    fast_div div_c;
    fft_desc d;        // c = F/2 point complex FFT
};

template <typename T>
cudaError_t launch_conv_os(const conv_args& a, const block_cfg& c, long long nblocks, cudaStream_t st);
template <typename T>
cudaError_t launch_hist_update(const void* hist_old, void* hist_new, const void* in, long long n, long long m1,
                               int channels, cudaStream_t st);

template <typename T>
class conv_filter
{
public:
    // taps: host or device pointer to `ntaps` values; block_size is the reference's partition size and
    // only bounds the FFT length from below here (outputs do not depend on it).  Taps too long for one
    // overlap-save FFT per CTA (M - 1 >= F / 2 at the largest one-CTA F) take the long mode: each call
    // convolves [history, input] with the taps through one real-FFT convolution per channel.
    conv_filter(const T* taps, size_t ntaps, size_t block_size, int channels = 1);
    // in / out: device pointers to channels x n samples (channel-major).  out must not alias in.
    void process(T* out, const T* in, size_t n, cudaStream_t st);
    void reset();
    size_t taps() const { return m_; }
    size_t fft_size() const { return f_; }
    int channels() const { return channels_; }
    bool long_mode() const { return long_; }
    int launches(size_t n) const;

private:
    size_t m_, f_, c_, bo_;
    int channels_;
    bool long_ = false;
    block_program<T> prog_;
    dbuf hspec_, rtw_, hist_[2];
    dbuf htaps_, lin_, lout_; // long mode: taps, [history, input] and the full convolution of one channel
    int cur_ = 0;
};

} // namespace kfr_gpu
