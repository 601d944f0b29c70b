// Elementwise kernels of the adjoints and the FIR filter backward pass (adjoint.hpp).
#include "adjoint.hpp"
#include "conv.hpp"
#include "convolve.hpp"
#include "fft_device.cuh"

#include <algorithm>

namespace kfr_gpu
{

static unsigned grid_for(long long n)
{
    return unsigned(std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 32)));
}

template <typename T>
__global__ void k_spectrum_weight(cpx<T>* out, const cpx<T>* in, long long batch, long long bins, int ccs, T w)
{
    const long long total = batch * bins;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
    {
        const long long k = i % bins;
        const bool edge   = k == 0 || (ccs && k == bins - 1);
        out[i]            = edge ? in[i] : scale(in[i], w);
    }
}

template <typename T>
__global__ void k_scale_first(T* out, const T* in, long long batch, long long n, T f)
{
    const long long total = batch * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
        out[i] = (i % n == 0) ? in[i] * f : in[i];
}

template <typename T>
__global__ void k_reverse(T* out, const T* in, long long channels, long long n)
{
    const long long total = channels * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
    {
        const long long c = i / n, t = i - c * n;
        out[i]            = in[c * n + (n - 1 - t)];
    }
}

template <typename T>
__global__ void k_pad_real(T* out, const T* in, long long channels, long long n, long long size)
{
    const long long total = channels * size;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x)
    {
        const long long c = i / size, t = i - c * size;
        out[i]            = t < n ? in[c * n + t] : T(0);
    }
}

template <typename T>
__global__ void k_scale(T* out, const T* in, long long n, T f)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = in[i] * f;
}

template <typename T>
__global__ void k_cmac_conj(cpx<T>* acc, const cpx<T>* a, const cpx<T>* b, long long channels, long long bins, int first)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < bins; k += (long long)gridDim.x * blockDim.x)
    {
        cpx<T> s = first ? mk<T>(0, 0) : acc[k];
        for (long long c = 0; c < channels; c++)
            s = s + a[c * bins + k] * conj(b[c * bins + k]);
        acc[k] = s;
    }
}

template <typename T>
cudaError_t launch_spectrum_weight(void* out, const void* in, long long batch, long long bins, bool ccs, T interior,
                                   cudaStream_t st)
{
    if (batch * bins <= 0)
        return cudaSuccess;
    k_spectrum_weight<T><<<grid_for(batch * bins), 256, 0, st>>>(static_cast<cpx<T>*>(out),
                                                                  static_cast<const cpx<T>*>(in), batch, bins, ccs, interior);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_scale_first(T* out, const T* in, long long batch, long long n, T f, cudaStream_t st)
{
    if (batch * n <= 0)
        return cudaSuccess;
    k_scale_first<T><<<grid_for(batch * n), 256, 0, st>>>(out, in, batch, n, f);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_reverse(T* out, const T* in, long long channels, long long n, cudaStream_t st)
{
    if (channels * n <= 0)
        return cudaSuccess;
    k_reverse<T><<<grid_for(channels * n), 256, 0, st>>>(out, in, channels, n);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_pad(T* out, const T* in, long long channels, long long n, long long size, cudaStream_t st)
{
    if (channels * size <= 0)
        return cudaSuccess;
    k_pad_real<T><<<grid_for(channels * size), 256, 0, st>>>(out, in, channels, n, size);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_cmac_conj(void* acc, const void* a, const void* b, long long channels, long long bins, bool first,
                             cudaStream_t st)
{
    if (bins <= 0)
        return cudaSuccess;
    k_cmac_conj<T><<<grid_for(bins), 256, 0, st>>>(static_cast<cpx<T>*>(acc), static_cast<const cpx<T>*>(a),
                                                    static_cast<const cpx<T>*>(b), channels, bins, first);
    return cudaGetLastError();
}

template <typename T>
void fir_backward(const T* taps, long long ntaps, long long channels, long long n, const T* x, const T* grad_y,
                  T* grad_x, T* grad_h, cudaStream_t st)
{
    if (ntaps <= 0 || channels <= 0 || n <= 0)
        throw std::invalid_argument("FIR backward needs taps, channels and samples");
    if (grad_x)
    {
        // grad_x = reverse(FIR_h(reverse(grad_y))): the same filter run backwards in time
        dbuf rev, fout;
        rev.alloc(size_t(channels * n) * sizeof(T));
        fout.alloc(size_t(channels * n) * sizeof(T));
        check(launch_reverse<T>(static_cast<T*>(rev.get()), grad_y, channels, n, st), "reverse");
        conv_filter<T> f(taps, size_t(ntaps), 1024, int(channels));
        f.process(static_cast<T*>(fout.get()), static_cast<const T*>(rev.get()), size_t(n), st);
        check(launch_reverse<T>(grad_x, static_cast<const T*>(fout.get()), channels, n, st), "reverse");
        check(cudaStreamSynchronize(st), "FIR backward (signal)");
    }
    if (grad_h)
    {
        // grad_h[m] = sum_c sum_t g_c[t] x_c[t-m]: real DFTs of size P >= n + M - 1 (no wrap-around for lags
        // 0..M-1), sum over channels of G_c conj(X_c), one inverse, the first M values scaled by 1/P
        long long P = 2;
        while (P < n + ntaps - 1)
            P <<= 1;
        auto eng              = plan_cache::instance().real<T>(P);
        const long long bins  = P / 2 + 1;
        const long long chunk = std::max<long long>(1, std::min<long long>(channels, (256LL << 20) / (P * (long long)sizeof(T))));
        dbuf pg, px, G, X, acc, scr, r;
        pg.alloc(size_t(chunk * P) * sizeof(T));
        px.alloc(size_t(chunk * P) * sizeof(T));
        G.alloc(size_t(chunk * bins) * 2 * sizeof(T));
        X.alloc(size_t(chunk * bins) * 2 * sizeof(T));
        acc.alloc(size_t(bins) * 2 * sizeof(T));
        r.alloc(size_t(P) * sizeof(T));
        const size_t sb = size_t(eng->scratch_elems(chunk)) * 2 * sizeof(T);
        if (sb)
            scr.alloc(sb);
        for (long long c0 = 0; c0 < channels; c0 += chunk)
        {
            const long long nc = std::min(chunk, channels - c0);
            check(launch_pad<T>(static_cast<T*>(pg.get()), grad_y + c0 * n, nc, n, P, st), "pad");
            check(launch_pad<T>(static_cast<T*>(px.get()), x + c0 * n, nc, n, P, st), "pad");
            eng->forward(G.get(), pg.get(), nc, true, scr.get(), st);
            eng->forward(X.get(), px.get(), nc, true, scr.get(), st);
            check(launch_cmac_conj<T>(acc.get(), G.get(), X.get(), nc, bins, c0 == 0, st), "accumulate");
        }
        eng->inverse(r.get(), acc.get(), 1, true, scr.get(), st);
        // grad_h = r[0 .. M-1] / P
        k_scale<T><<<grid_for(ntaps), 256, 0, st>>>(grad_h, static_cast<const T*>(r.get()), ntaps, T(1) / T(P));
        check(cudaGetLastError(), "scale taps gradient");
        check(cudaStreamSynchronize(st), "FIR backward (taps)");
    }
}

#define KFR_GPU_ADJ(T)                                                                                     \
    template cudaError_t launch_spectrum_weight<T>(void*, const void*, long long, long long, bool, T, cudaStream_t); \
    template cudaError_t launch_scale_first<T>(T*, const T*, long long, long long, T, cudaStream_t);       \
    template cudaError_t launch_reverse<T>(T*, const T*, long long, long long, cudaStream_t);              \
    template cudaError_t launch_pad<T>(T*, const T*, long long, long long, long long, cudaStream_t);       \
    template cudaError_t launch_cmac_conj<T>(void*, const void*, const void*, long long, long long, bool, cudaStream_t); \
    template void fir_backward<T>(const T*, long long, long long, long long, const T*, const T*, T*, T*, cudaStream_t);
KFR_GPU_ADJ(float)
KFR_GPU_ADJ(double)

} // namespace kfr_gpu
