// FFT convolution filter kernels and host class (see conv.hpp).
#include "conv.hpp"
#include "convolve.hpp"
#include "kernels.cuh"

#include <algorithm>
#include <vector>

namespace kfr_gpu
{

// Real-DFT split of bins (k, c-k) from the c-point complex spectrum of the packed reals.
template <typename T>
__device__ __forceinline__ cpx<T> rsplit(cpx<T> zk, cpx<T> zkk, cpx<T> w)
{
    const cpx<T> znk = conj(zkk);
    return scale(zk + znk, T(0.5)) + w * scale(mul_mi(zk - znk), T(0.5));
}
// Real-DFT merge (inverse of rsplit, times 2) of bins (k, c-k).
template <typename T>
__device__ __forceinline__ cpx<T> rmerge(cpx<T> yk, cpx<T> ykk, cpx<T> w)
{
    const cpx<T> ynk = conj(ykk);
    return (yk + ynk) + mul_pi(conj(w) * (yk - ynk));
}

// One overlap-save block per CTA: blockIdx.x = output block, blockIdx.y = channel.
template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1) k_conv_os(const conv_args a, const int ts)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ pass_desc sp[kMaxPasses];
    const F fft(sp, a.d, ts);
    cpx<T>* sm       = reinterpret_cast<cpx<T>*>(smem_raw);
    const int c      = fft.n;
    const long long b = blockIdx.x;
    const int ch     = blockIdx.y;
    const T* in      = reinterpret_cast<const T*>(a.in) + (long long)ch * a.n;
    const T* hist    = reinterpret_cast<const T*>(a.hist) + (long long)ch * a.m1;
    T* out           = reinterpret_cast<T*>(a.out) + (long long)ch * a.n;
    const long long base  = b * a.bo;
    const long long limit = a.m1 + a.n;
    // pairs (x[i0], x[i0 + 1]) with i0 - m1 even come from `in` as one 8-byte load when it is 8-byte aligned
    const bool in_pairs = ((a.m1 | base) & 1) == 0 && (reinterpret_cast<uintptr_t>(in) & (2 * sizeof(T) - 1)) == 0;
#pragma unroll 4
    for (int m = threadIdx.x; m < c; m += blockDim.x)
    {
        const long long i0 = base + 2 * m;
        cpx<T> v;
        if (in_pairs && i0 >= a.m1 && i0 + 1 < limit)
            v = *reinterpret_cast<const cpx<T>*>(in + (i0 - a.m1));
        else
        {
            T v0 = T(0), v1 = T(0);
            if (i0 < limit)
                v0 = i0 < a.m1 ? hist[i0] : in[i0 - a.m1];
            if (i0 + 1 < limit)
                v1 = i0 + 1 < a.m1 ? hist[i0 + 1] : in[i0 + 1 - a.m1];
            v = mk(v0, v1);
        }
        sm[F::pi(m)] = v;
    }
    __syncthreads();
    const cpx<T>* tw = reinterpret_cast<const cpx<T>*>(a.tw);
    const int lt     = int(threadIdx.x) < ts ? int(threadIdx.x) : ts;
    fft.run(sm, tw, lt);
    const cpx<T>* H   = reinterpret_cast<const cpx<T>*>(a.hspec);
    const cpx<T>* rtw = reinterpret_cast<const cpx<T>*>(a.rtw);
    for (int k = threadIdx.x; k <= c / 2; k += blockDim.x)
    {
        if (k == 0)
        {
            const cpx<T> z0 = sm[0];
            const T y0      = (z0.x + z0.y) * ldg(H).x;
            const T yc      = (z0.x - z0.y) * ldg(H + c).x;
            sm[0]           = conj(mk(y0 + yc, y0 - yc));
        }
        else
        {
            const int kk      = c - k;
            const cpx<T> zk   = sm[F::pi(k)];
            const cpx<T> zkk  = sm[F::pi(kk)];
            const cpx<T> wk   = ldg(rtw + k);
            const cpx<T> wkk  = ldg(rtw + kk);
            const cpx<T> yk   = rsplit(zk, zkk, wk) * ldg(H + k);
            const cpx<T> ykk  = rsplit(zkk, zk, wkk) * ldg(H + kk);
            sm[F::pi(k)]    = conj(rmerge(yk, ykk, wk));
            if (kk != k)
                sm[F::pi(kk)] = conj(rmerge(ykk, yk, wkk));
        }
    }
    __syncthreads();
    fft.run(sm, tw, lt);
    // outputs j = m1 + t, t < bo: element j / 2 holds (y[j even], -y[j + 1]); with m1, base and bo even and
    // `out` 8-byte aligned, each pair goes out as one 8-byte store
    if (((a.m1 | base | a.bo) & 1) == 0 && (reinterpret_cast<uintptr_t>(out) & (2 * sizeof(T) - 1)) == 0)
    {
        for (long long u = threadIdx.x; 2 * u < a.bo; u += blockDim.x)
        {
            const long long no = base + 2 * u;
            const cpx<T> v     = sm[F::pi(int((a.m1 >> 1) + u))];
            if (no + 1 < a.n)
                *reinterpret_cast<cpx<T>*>(out + no) = mk(v.x, -v.y);
            else if (no < a.n)
                out[no] = v.x;
        }
    }
    else
    {
        for (long long t = threadIdx.x; t < a.bo; t += blockDim.x)
        {
            const long long no = base + t;
            if (no < a.n)
            {
                const long long j = a.m1 + t;
                const cpx<T> v    = sm[F::pi(int(j >> 1))];
                out[no]           = (j & 1) ? -v.y : v.x;
            }
        }
    }
}

// new_hist[i] = i + n < m1 ? old_hist[i + n] : in[i + n - m1]
template <typename T>
__global__ void k_hist_update(const T* __restrict__ hold, T* __restrict__ hnew, const T* __restrict__ in, long long n,
                              long long m1, int channels)
{
    const long long total = m1 * channels;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
    {
        const long long ch = i / m1, e = i - ch * m1;
        const long long s  = e + n;
        hnew[i]            = s < m1 ? hold[ch * m1 + s] : in[ch * n + (s - m1)];
    }
}

template <typename T>
cudaError_t launch_conv_os(const conv_args& a, const block_cfg& c, long long nblocks, cudaStream_t st)
{
    const dim3 grid(unsigned(nblocks), unsigned(a.channels));
    if (c.ct)
    {
        if constexpr (std::is_same<T, float>::value)
        {
#define CT_KERNEL k_conv_os
#define CT_GRID grid
#define CT_ARGS a, c.ts
            switch (c.ct)
            {
                KFR_CT_CONV_F32(KFR_GPU_CT_CASE)
            default: return cudaErrorInvalidValue;
            }
#undef CT_KERNEL
#undef CT_GRID
#undef CT_ARGS
        }
        return cudaErrorInvalidValue;
    }
    KFR_GPU_RUNTIME_DISPATCH(k_conv_os, grid, a, c.ts)
}

template <typename T>
cudaError_t launch_hist_update(const void* hold, void* hnew, const void* in, long long n, long long m1, int channels,
                               cudaStream_t st)
{
    const long long total = m1 * channels;
    if (total <= 0)
        return cudaSuccess;
    const long long blocks = std::min<long long>((total + 255) / 256, 4096);
    k_hist_update<T><<<unsigned(blocks), 256, 0, st>>>(static_cast<const T*>(hold), static_cast<T*>(hnew),
                                                        static_cast<const T*>(in), n, m1, channels);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------------------
// conv_filter
// ------------------------------------------------------------------------------------------------------

static size_t next_pow2(size_t x)
{
    size_t p = 1;
    while (p < x)
        p <<= 1;
    return p;
}

template <typename T>
conv_filter<T>::conv_filter(const T* taps, size_t ntaps, size_t block_size, int channels)
    : m_(ntaps), channels_(channels)
{
    if (channels < 1)
        throw std::invalid_argument("convolution filter needs at least one channel");
    std::vector<T> h(ntaps);
    if (ntaps)
    {
        if (!taps)
            throw std::invalid_argument("taps pointer is NULL");
        cudaPointerAttributes pa;
        const bool dev = cudaPointerGetAttributes(&pa, taps) == cudaSuccess &&
                         (pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged);
        cudaGetLastError();
        check(cudaMemcpy(h.data(), taps, ntaps * sizeof(T), dev ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost),
              "copy taps");
    }
    const size_t m1 = ntaps ? ntaps - 1 : 0;
    // largest one-CTA complex length (power of two) for this precision
    size_t cmax = 1;
    while (block_program<T>::feasible((long long)(cmax * 2)))
        cmax *= 2;
    const size_t fmax = 2 * cmax;
    // the FFT is at least 8x the taps (at most 1/8 of each block re-reads the overlap; measured 0.390 ->
    // 0.374 ms against 4x for 64 channels of 2^20 samples and 1023 taps) and twice the block
    size_t f          = std::max(next_pow2(8 * m1), 2 * next_pow2(block_size ? block_size : 1024));
    f                 = std::max<size_t>(f, 64);
    if (f > fmax)
        f = fmax;
    const size_t hb = std::max<size_t>(1, m1 * size_t(channels)) * sizeof(T);
    hist_[0].alloc(hb);
    hist_[1].alloc(hb);
    if (m1 >= f / 2)
    {
        // long mode: the taps stay on the device for whole-call convolutions
        long_ = true;
        f_ = c_ = bo_ = 0;
        htaps_.upload(h.data(), ntaps * sizeof(T));
        reset();
        return;
    }
    f_  = f;
    c_  = f / 2;
    bo_ = f - m1;
    prog_.build(int(c_), CT_CONV);
    // taps spectrum FFT_F(h padded) / F, bins 0..c (set_data, src/dft/convolution-impl.cpp:53-71)
    std::vector<std::complex<double>> a(f, { 0.0, 0.0 });
    for (size_t i = 0; i < ntaps; i++)
        a[i] = double(h[i]);
    host_fft_pow2(a);
    std::vector<std::complex<T>> hs(c_ + 1), rt(c_ + 1);
    for (size_t k = 0; k <= c_; k++)
    {
        hs[k]        = std::complex<T>(T(a[k].real() / double(f)), T(a[k].imag() / double(f)));
        const auto w = twiddle((long long)k, (long long)f);
        rt[k]        = std::complex<T>(T(w.real()), T(w.imag()));
    }
    hspec_.upload(hs.data(), hs.size() * sizeof(std::complex<T>));
    rtw_.upload(rt.data(), rt.size() * sizeof(std::complex<T>));
    reset();
}

template <typename T>
void conv_filter<T>::reset()
{
    check(cudaMemset(hist_[0].get(), 0, hist_[0].size()), "reset filter state");
    check(cudaMemset(hist_[1].get(), 0, hist_[1].size()), "reset filter state");
    cur_ = 0;
}

template <typename T>
int conv_filter<T>::launches(size_t n) const
{
    if (long_ && n)
        return 2 + 8 * channels_; // per channel: two pads, two forward and one inverse real FFT, the product
    return (n && m_) ? (m_ > 1 ? 2 : 1) : (n ? 1 : 0);
}

template <typename T>
void conv_filter<T>::process(T* out, const T* in, size_t n, cudaStream_t st)
{
    if (n == 0)
        return;
    if (m_ == 0)
    {
        check(cudaMemsetAsync(out, 0, n * channels_ * sizeof(T), st), "zero output");
        return;
    }
    const long long m1 = (long long)m_ - 1;
    if (long_)
    {
        // y = ([history, input] * taps)[m1 + t], t < n, one real-FFT convolution per channel
        const long long ulen = m1 + (long long)n;
        lin_.ensure(size_t(ulen) * sizeof(T));
        lout_.ensure(size_t(ulen + (long long)m_ - 1) * sizeof(T));
        T* u = static_cast<T*>(lin_.get());
        T* y = static_cast<T*>(lout_.get());
        for (int ch = 0; ch < channels_; ch++)
        {
            check(cudaMemcpyAsync(u, static_cast<const T*>(hist_[cur_].get()) + ch * m1, size_t(m1) * sizeof(T),
                                  cudaMemcpyDeviceToDevice, st),
                  "copy filter history");
            check(cudaMemcpyAsync(u + m1, in + ch * (long long)n, n * sizeof(T), cudaMemcpyDeviceToDevice, st),
                  "copy filter input");
            convolve_device<T>(y, u, ulen, htaps_.get(), (long long)m_, false, 0, st);
            check(cudaMemcpyAsync(out + ch * (long long)n, y + m1, n * sizeof(T), cudaMemcpyDeviceToDevice, st),
                  "copy filter output");
        }
        check(launch_hist_update<T>(hist_[cur_].get(), hist_[1 - cur_].get(), in, (long long)n, m1, channels_, st),
              "launch history update");
        cur_ = 1 - cur_;
        return;
    }
    conv_args a;
    a.in       = in;
    a.out      = out;
    a.hist     = hist_[cur_].get();
    a.n        = (long long)n;
    a.m1       = m1;
    a.bo       = (long long)bo_;
    a.channels = channels_;
    a.hspec    = hspec_.get();
    a.rtw      = rtw_.get();
    a.tw       = prog_.tw.get();
    a.div_c    = make_fast_div(uint32_t(c_));
    a.d        = prog_.desc;
    block_cfg cfg       = prog_.cfg_tile(1);
    const long long nbl = ((long long)n + (long long)bo_ - 1) / (long long)bo_;
    check(launch_conv_os<T>(a, cfg, nbl, st), "launch convolution");
    if (m1 > 0)
    {
        check(launch_hist_update<T>(hist_[cur_].get(), hist_[1 - cur_].get(), in, (long long)n, m1, channels_, st),
              "launch history update");
        cur_ = 1 - cur_;
    }
}

template class conv_filter<float>;
template class conv_filter<double>;
template cudaError_t launch_conv_os<float>(const conv_args&, const block_cfg&, long long, cudaStream_t);
template cudaError_t launch_conv_os<double>(const conv_args&, const block_cfg&, long long, cudaStream_t);

} // namespace kfr_gpu
