// Elementwise kernels of the multi-kernel paths (see launch.hpp: ew_op).
#include <algorithm>

#include "fft_device.cuh"
#include "launch.hpp"

namespace kfr_gpu
{

template <typename T>
__global__ void __launch_bounds__(256) k_elementwise(const int op, const ew_args a)
{
    const long long total = a.batch * a.n;
    const cpx<T>* in      = reinterpret_cast<const cpx<T>*>(a.in);
    cpx<T>* out           = reinterpret_cast<cpx<T>*>(a.out);
    const cpx<T>* t0      = reinterpret_cast<const cpx<T>*>(a.t0);
    const T* inr          = reinterpret_cast<const T*>(a.in);
    T* outr               = reinterpret_cast<T*>(a.out);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x)
    {
        const long long s = i / a.n;
        const long long e = i - s * a.n;
        switch (op)
        {
        case EW_BS_PRE:
        {
            cpx<T> v = mk<T>(0, 0);
            if (e < a.n_src)
                v = conj_if(in[s * a.istride + e], a.flag != 0) * ldg(t0 + e);
            out[s * a.ostride + e] = v;
            break;
        }
        case EW_BS_MID:
            out[s * a.ostride + e] = conj(in[s * a.istride + e] * ldg(t0 + e));
            break;
        case EW_BS_POST:
            out[s * a.ostride + e] = conj_if(conj(in[s * a.istride + e]) * ldg(t0 + e), a.flag != 0);
            break;
        case EW_DCT2_PRE:
        {
            // e is the source index; write its mirrored position
            const long long n   = a.n;
            const long long pos = (e & 1) ? n - 1 - (e >> 1) : (e >> 1);
            out[s * a.ostride + pos] = mk<T>(inr[s * a.istride + e], T(0));
            break;
        }
        case EW_DCT2_POST:
        {
            const cpx<T> y = in[s * a.istride + e];
            const cpx<T> w = ldg(t0 + e);
            outr[s * a.ostride + e] = y.x * w.x + y.y * w.y;
            break;
        }
        case EW_DCT3_PRE:
        {
            const T x      = inr[s * a.istride + e];
            const cpx<T> w = ldg(t0 + e);
            cpx<T> v       = mk<T>(x * w.x, -(x * w.y));
            if (e == 0)
                v = scale(v, T(0.5));
            out[s * a.ostride + e] = v;
            break;
        }
        case EW_DCT3_POST:
        {
            const long long n   = a.n;
            const long long pos = (e & 1) ? n - 1 - (e >> 1) : (e >> 1);
            outr[s * a.ostride + e] = in[s * a.istride + pos].x;
            break;
        }
        default: break;
        }
    }
}

template <typename T>
cudaError_t launch_elementwise(int op, const ew_args& a, cudaStream_t st)
{
    const long long total = a.batch * a.n;
    if (total <= 0)
        return cudaSuccess;
    long long blocks = (total + 255) / 256;
    if (blocks > 152LL * 32)
        blocks = 152LL * 32;
    k_elementwise<T><<<unsigned(blocks), 256, 0, st>>>(op, a);
    return cudaGetLastError();
}

// Real-DFT split / merge over mirror pairs: thread e of a signal (e = 0 .. c/2) reads Z[e] and Z[c - e] (or
// X[e] and X[c - e]) once and writes both outputs; e == c - e (c even) writes one.  grid.y walks the signals.
template <typename T, bool INV>
__global__ void __launch_bounds__(256) k_real_pairs(const ew_args a)
{
    const long long c = a.n_src;
    const cpx<T>* t0  = reinterpret_cast<const cpx<T>*>(a.t0);
    const bool ccs    = a.flag != 0;
    for (long long s = blockIdx.y; s < a.batch; s += gridDim.y)
    {
        const cpx<T>* in = reinterpret_cast<const cpx<T>*>(a.in) + s * a.istride;
        cpx<T>* out      = reinterpret_cast<cpx<T>*>(a.out) + s * a.ostride;
        for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e <= c / 2;
             e += (long long)gridDim.x * blockDim.x)
        {
            if (e == 0)
            {
                const cpx<T> z0 = in[0];
                if constexpr (!INV)
                {
                    out[0] = ccs ? mk<T>(z0.x + z0.y, 0) : mk<T>(z0.x + z0.y, z0.x - z0.y);
                    if (ccs)
                        out[c] = mk<T>(z0.x - z0.y, 0);
                }
                else
                {
                    const T xn = ccs ? in[c].x : z0.y;
                    out[0]     = mk<T>(z0.x + xn, z0.x - xn);
                }
                continue;
            }
            const long long m = c - e;
            const cpx<T> u    = in[e];
            const cpx<T> v    = in[m];
            if constexpr (!INV)
            {
                // X[k] = (Z[k] + conj Z[c-k]) / 2 - i W_2c^k (Z[k] - conj Z[c-k]) / 2
                out[e] = scale(u + conj(v), T(0.5)) + ldg(t0 + e) * scale(mul_mi(u - conj(v)), T(0.5));
                if (m != e)
                    out[m] = scale(v + conj(u), T(0.5)) + ldg(t0 + m) * scale(mul_mi(v - conj(u)), T(0.5));
            }
            else
            {
                // Z[k] = (X[k] + conj X[c-k]) + i conj(W_2c^k) (X[k] - conj X[c-k])
                out[e] = (u + conj(v)) + mul_pi(conj(ldg(t0 + e)) * (u - conj(v)));
                if (m != e)
                    out[m] = (v + conj(u)) + mul_pi(conj(ldg(t0 + m)) * (v - conj(u)));
            }
        }
    }
}

template <typename T>
cudaError_t launch_real_pairs(const ew_args& a, bool inverse, cudaStream_t st)
{
    const long long pairs = a.n_src / 2 + 1;
    if (a.batch <= 0 || a.n_src < 1)
        return cudaSuccess;
    const unsigned bx = unsigned(std::min<long long>((pairs + 255) / 256, 1024));
    const unsigned by = unsigned(std::min<long long>(a.batch, std::max<long long>(1, 152LL * 16 / bx)));
    if (inverse)
        k_real_pairs<T, true><<<dim3(bx, by), 256, 0, st>>>(a);
    else
        k_real_pairs<T, false><<<dim3(bx, by), 256, 0, st>>>(a);
    return cudaGetLastError();
}
template cudaError_t launch_real_pairs<float>(const ew_args&, bool, cudaStream_t);
template cudaError_t launch_real_pairs<double>(const ew_args&, bool, cudaStream_t);

// Spectral product of include/kfr/dft/fft.hpp:983-1020 over a batch: one thread per element, grid-stride.
// The Perm format stores the DC and Nyquist bins, both real, as the real and imaginary parts of element 0, so
// that element is multiplied part by part instead of as a complex number.
template <typename T, bool ACC>
__global__ void __launch_bounds__(256) k_fft_multiply(cpx<T>* dest, const cpx<T>* acc, const cpx<T>* src1,
                                                      const cpx<T>* src2, const long long size,
                                                      const long long total, const long long src2_stride,
                                                      const int perm)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x)
    {
        const long long s = i / size;
        const long long e = i - s * size;
        const cpx<T> a    = src1[i];
        const cpx<T> b    = src2[s * src2_stride + e];
        cpx<T> v          = (perm && e == 0) ? mk<T>(a.x * b.x, a.y * b.y) : a * b;
        if constexpr (ACC)
            v = acc[i] + v;
        dest[i] = v;
    }
}

template <typename T>
cudaError_t launch_fft_multiply(void* dest, const void* acc, const void* src1, const void* src2, long long size,
                                long long batch, long long src2_stride, bool perm, cudaStream_t st)
{
    const long long total = size * batch;
    if (total <= 0)
        return cudaSuccess;
    long long blocks = (total + 255) / 256;
    if (blocks > 152LL * 16)
        blocks = 152LL * 16;
    auto* d        = static_cast<cpx<T>*>(dest);
    const auto* a  = static_cast<const cpx<T>*>(acc);
    const auto* s1 = static_cast<const cpx<T>*>(src1);
    const auto* s2 = static_cast<const cpx<T>*>(src2);
    if (acc)
        k_fft_multiply<T, true><<<unsigned(blocks), 256, 0, st>>>(d, a, s1, s2, size, total, src2_stride, perm);
    else
        k_fft_multiply<T, false><<<unsigned(blocks), 256, 0, st>>>(d, a, s1, s2, size, total, src2_stride, perm);
    return cudaGetLastError();
}

template cudaError_t launch_fft_multiply<float>(void*, const void*, const void*, const void*, long long, long long,
                                                long long, bool, cudaStream_t);
template cudaError_t launch_fft_multiply<double>(void*, const void*, const void*, const void*, long long,
                                                 long long, long long, bool, cudaStream_t);

// Batched complex transpose through a 32 x 32 shared-memory tile (one padding column, so the column reads
// of the tile fall into distinct banks); each thread moves 4 elements per direction.  blockIdx.y walks the
// batch (more than 65535 matrices take several launches).
template <typename T>
__global__ void __launch_bounds__(256) k_transpose(cpx<T>* out, const cpx<T>* in, const long long rows,
                                                   const long long cols, const long long b0)
{
    __shared__ cpx<T> tile[32][33];
    const long long b  = b0 + blockIdx.y;
    const long long gx = (cols + 31) / 32; // tiles along a row; blockIdx.x = row tile * gx + column tile
    const long long c0 = ((long long)blockIdx.x % gx) * 32, r0 = ((long long)blockIdx.x / gx) * 32;
    const cpx<T>* src  = in + b * rows * cols;
    cpx<T>* dst        = out + b * rows * cols;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < 32; i += 8)
    {
        const long long r = r0 + ty + i, c = c0 + tx;
        if (r < rows && c < cols)
            tile[ty + i][tx] = src[r * cols + c];
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 32; i += 8)
    {
        const long long c = c0 + ty + i, r = r0 + tx;
        if (r < rows && c < cols)
            dst[c * rows + r] = tile[tx][ty + i];
    }
}

template <typename T>
cudaError_t launch_transpose(void* out, const void* in, long long batch, long long rows, long long cols,
                             cudaStream_t st)
{
    if (batch <= 0 || rows <= 0 || cols <= 0)
        return cudaSuccess;
    const long long tiles = ((cols + 31) / 32) * ((rows + 31) / 32);
    if (tiles > 2147483647LL)
        return cudaErrorInvalidValue;
    for (long long b0 = 0; b0 < batch; b0 += 65535)
    {
        const unsigned gb = unsigned(std::min<long long>(65535, batch - b0));
        k_transpose<T><<<dim3(unsigned(tiles), gb), 256, 0, st>>>(static_cast<cpx<T>*>(out),
                                                                   static_cast<const cpx<T>*>(in), rows, cols, b0);
    }
    return cudaGetLastError();
}

template cudaError_t launch_transpose<float>(void*, const void*, long long, long long, long long, cudaStream_t);
template cudaError_t launch_transpose<double>(void*, const void*, long long, long long, long long, cudaStream_t);

template cudaError_t launch_elementwise<float>(int, const ew_args&, cudaStream_t);
template cudaError_t launch_elementwise<double>(int, const ew_args&, cudaStream_t);

} // namespace kfr_gpu
