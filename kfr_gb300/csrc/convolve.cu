// Whole-signal convolution and the plan cache (see convolve.hpp).
#include "convolve.hpp"
#include "fft_device.cuh"

#include <algorithm>
#include <type_traits>

namespace kfr_gpu
{

// ------------------------------------------------------------------------------------------------------
// plan_cache
// ------------------------------------------------------------------------------------------------------

struct plan_cache::entry
{
    int kind;
    long long n;
    std::shared_ptr<void> plan;
};

plan_cache& plan_cache::instance()
{
    static plan_cache c;
    return c;
}

template <typename T>
static int kind_of(bool real)
{
    return (real ? 2 : 0) + (sizeof(T) == 8 ? 1 : 0);
}

template <typename T>
std::shared_ptr<complex_engine<T>> plan_cache::complex(long long n)
{
    std::lock_guard<std::mutex> lock(mu_);
    const int kd = kind_of<T>(false);
    for (auto& e : entries_)
        if (e->kind == kd && e->n == n)
            return std::static_pointer_cast<complex_engine<T>>(e->plan);
    auto p = std::make_shared<complex_engine<T>>(n);
    entries_.push_back(std::make_shared<entry>(entry{ kd, n, p }));
    return p;
}

template <typename T>
std::shared_ptr<real_engine<T>> plan_cache::real(long long n)
{
    std::lock_guard<std::mutex> lock(mu_);
    const int kd = kind_of<T>(true);
    for (auto& e : entries_)
        if (e->kind == kd && e->n == n)
            return std::static_pointer_cast<real_engine<T>>(e->plan);
    auto p = std::make_shared<real_engine<T>>(n);
    entries_.push_back(std::make_shared<entry>(entry{ kd, n, p }));
    return p;
}

void plan_cache::clear()
{
    std::lock_guard<std::mutex> lock(mu_);
    entries_.clear();
}

size_t plan_cache::size() const
{
    std::lock_guard<std::mutex> lock(mu_);
    return entries_.size();
}

template std::shared_ptr<complex_engine<float>> plan_cache::complex<float>(long long);
template std::shared_ptr<complex_engine<double>> plan_cache::complex<double>(long long);
template std::shared_ptr<real_engine<float>> plan_cache::real<float>(long long);
template std::shared_ptr<real_engine<double>> plan_cache::real<double>(long long);

// ------------------------------------------------------------------------------------------------------
// kernels
// ------------------------------------------------------------------------------------------------------

// out[i] = i < n ? in[reverse ? n-1-i : i] : 0 for i < size (E = T for reals, cpx<T> for complex)
template <typename E>
__global__ void k_pad(E* __restrict__ out, const E* __restrict__ in, long long n, long long size, int reverse)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < size; i += (long long)gridDim.x * blockDim.x)
    {
        E v{};
        if (i < n)
            v = in[reverse ? n - 1 - i : i];
        out[i] = v;
    }
}

template <typename T>
__global__ void k_cmul_scale(cpx<T>* __restrict__ a, const cpx<T>* __restrict__ b, long long n, T s)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        a[i] = scale(a[i] * b[i], s);
}

template <typename T>
__global__ void k_real_part(cpx<T>* __restrict__ out, const cpx<T>* __restrict__ in, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = mk(in[i].x, T(0));
}

static unsigned blocks_for(long long n) { return unsigned(std::max<long long>(1, std::min<long long>((n + 255) / 256, 4096))); }

template <typename T>
size_t convolve_scratch_bytes(long long na, long long nb, bool is_complex)
{
    const long long olen = na + nb - 1;
    long long size       = 1;
    while (size < olen)
        size <<= 1;
    if (!is_complex)
    {
        size = std::max<long long>(size, 2);
        return size_t(2 * size * sizeof(T) + 2 * (size / 2 + 1) * 2 * sizeof(T));
    }
    return size_t(2 * size * 2 * sizeof(T));
}

template <typename T>
void convolve_device(void* out, const void* a, long long na, const void* b, long long nb, bool is_complex, int mode,
                     cudaStream_t st)
{
    if (na <= 0 || nb <= 0)
        return;
    const long long olen = na + nb - 1;
    long long size       = 1;
    while (size < olen)
        size <<= 1;
    const int rev = mode == 1;
    void* work    = nullptr;
    check(cudaMallocAsync(&work, convolve_scratch_bytes<T>(na, nb, is_complex), st), "cudaMallocAsync");
    struct freer
    {
        void* p;
        cudaStream_t s;
        ~freer() { cudaFreeAsync(p, s); }
    } guard{ work, st };
    if (!is_complex)
    {
        size                 = std::max<long long>(size, 2);
        const long long c    = size / 2;
        auto eng             = plan_cache::instance().real<T>(size);
        T* pa                = static_cast<T*>(work);
        T* pb                = pa + size;
        cpx<T>* A            = reinterpret_cast<cpx<T>*>(pb + size);
        cpx<T>* B            = A + (c + 1);
        const size_t escr    = size_t(eng->scratch_elems(1)) * 2 * sizeof(T);
        void* escratch       = nullptr;
        if (escr)
            check(cudaMallocAsync(&escratch, escr, st), "cudaMallocAsync");
        k_pad<T><<<blocks_for(size), 256, 0, st>>>(pa, static_cast<const T*>(a), na, size, 0);
        k_pad<T><<<blocks_for(size), 256, 0, st>>>(pb, static_cast<const T*>(b), nb, size, rev);
        eng->forward(A, pa, 1, true, escratch, st);
        eng->forward(B, pb, 1, true, escratch, st);
        k_cmul_scale<T><<<blocks_for(c + 1), 256, 0, st>>>(A, B, c + 1, T(1) / T(size));
        eng->inverse(pa, A, 1, true, escratch, st);
        check(cudaMemcpyAsync(out, pa, olen * sizeof(T), cudaMemcpyDeviceToDevice, st), "copy result");
        if (escratch)
            cudaFreeAsync(escratch, st);
    }
    else
    {
        auto eng          = plan_cache::instance().complex<T>(size);
        cpx<T>* pa        = static_cast<cpx<T>*>(work);
        cpx<T>* pb        = pa + size;
        const size_t escr = size_t(eng->scratch_elems(1)) * 2 * sizeof(T);
        void* escratch    = nullptr;
        if (escr)
            check(cudaMallocAsync(&escratch, escr, st), "cudaMallocAsync");
        k_pad<cpx<T>><<<blocks_for(size), 256, 0, st>>>(pa, static_cast<const cpx<T>*>(a), na, size, 0);
        k_pad<cpx<T>><<<blocks_for(size), 256, 0, st>>>(pb, static_cast<const cpx<T>*>(b), nb, size, rev);
        eng->execute(pa, pa, 1, size, size, false, escratch, st);
        eng->execute(pb, pb, 1, size, size, false, escratch, st);
        k_cmul_scale<T><<<blocks_for(size), 256, 0, st>>>(pa, pb, size, T(1) / T(size));
        eng->execute(pa, pa, 1, size, size, true, escratch, st);
        k_real_part<T><<<blocks_for(olen), 256, 0, st>>>(static_cast<cpx<T>*>(out), pa, olen);
        if (escratch)
            cudaFreeAsync(escratch, st);
    }
    check(cudaGetLastError(), "launch convolution");
}

template void convolve_device<float>(void*, const void*, long long, const void*, long long, bool, int, cudaStream_t);
template void convolve_device<double>(void*, const void*, long long, const void*, long long, bool, int, cudaStream_t);
template size_t convolve_scratch_bytes<float>(long long, long long, bool);
template size_t convolve_scratch_bytes<double>(long long, long long, bool);

} // namespace kfr_gpu
