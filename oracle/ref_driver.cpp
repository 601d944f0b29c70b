// ref_driver: a thin extern "C" shim over KFR 7.0.1's own C++ DFT API.  TEST INFRASTRUCTURE ONLY.
//
// Built by oracle/Makefile against the reference's unmodified sources (src/dft/*.cpp) into
// oracle/_ref/libkfr_ref.so.  It is used in the build container to pin the C restatement in
// kfr_oracle.c to the reference itself, and to generate the golden fixtures under tests/golden/.  The
// entry points mirror kfr_oracle.c's so the same Python wrapper drives both.
//
// Calls made, with the reference lines they exercise:
//   dft_plan<T>::execute            include/kfr/dft/fft.hpp:265-272
//   dft_plan_real<T>::execute       include/kfr/dft/fft.hpp:512-535
//   dct_plan<T>::execute            include/kfr/dft/fft.hpp:932-970
//   convolve / correlate            include/kfr/dft/convolution.hpp:53-67
//   convolve_filter<T>              include/kfr/dft/convolution.hpp:98-148
//   fir_filter<T> (the fir expression over a fir_state, as its process_buffer does)
//                                   include/kfr/dsp/fir.hpp:64-113, src/dsp/fir.cpp:54-57
#include <kfr/dft.hpp>
#include <kfr/dft/convolution.hpp>
#include <kfr/dsp/fir.hpp>

#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

using namespace kfr;

namespace
{
template <typename Fn>
void parallel_for(size_t count, int threads, Fn&& fn)
{
    if (threads < 1)
        threads = 1;
    if (static_cast<size_t>(threads) > count)
        threads = static_cast<int>(count ? count : 1);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++)
    {
        size_t b0 = count * t / threads, b1 = count * (t + 1) / threads;
        pool.emplace_back([=, &fn] { fn(b0, b1); });
    }
    for (auto& th : pool)
        th.join();
}

template <typename T>
int run_dft(T* out, const T* in, size_t n, size_t batch, int inverse, int threads)
{
    if (n == 0)
        return 0;
    dft_plan<T> plan(n);
    parallel_for(batch, threads,
                 [&](size_t b0, size_t b1)
                 {
                     univector<u8> temp(plan.temp_size);
                     for (size_t b = b0; b < b1; b++)
                         plan.execute(reinterpret_cast<complex<T>*>(out) + b * n,
                                      reinterpret_cast<const complex<T>*>(in) + b * n, temp.data(),
                                      inverse != 0);
                 });
    return 0;
}

template <typename T>
int run_real(T* out, const T* in, size_t n, int ccs, size_t batch, int inverse, int threads)
{
    if (n == 0 || n % 2)
        return -1;
    const dft_pack_format fmt = ccs ? dft_pack_format::CCs : dft_pack_format::Perm;
    dft_plan_real<T> plan(n, fmt);
    const size_t cs = plan.complex_size();
    parallel_for(batch, threads,
                 [&](size_t b0, size_t b1)
                 {
                     univector<u8> temp(plan.temp_size);
                     for (size_t b = b0; b < b1; b++)
                     {
                         if (!inverse)
                             plan.execute(reinterpret_cast<complex<T>*>(out) + b * cs, in + b * n, temp.data());
                         else
                             plan.execute(out + b * n, reinterpret_cast<const complex<T>*>(in) + b * cs,
                                          temp.data());
                     }
                 });
    return 0;
}

template <typename T>
int run_dct(T* out, const T* in, size_t n, int inverse, size_t batch, int threads)
{
    if (n == 0)
        return 0;
    dct_plan<T> plan(n);
    parallel_for(batch, threads,
                 [&](size_t b0, size_t b1)
                 {
                     univector<u8> temp(plan.temp_size);
                     for (size_t b = b0; b < b1; b++)
                         plan.execute(out + b * n, in + b * n, temp.data(), inverse != 0);
                 });
    return 0;
}

template <typename T>
size_t run_convolve(T* out, const T* a, size_t na, const T* b, size_t nb, int correlate, int is_complex)
{
    if (na == 0 || nb == 0)
        return 0;
    if (is_complex)
    {
        univector<complex<T>> x(na), y(nb);
        std::memcpy(x.data(), a, na * sizeof(complex<T>));
        std::memcpy(y.data(), b, nb * sizeof(complex<T>));
        univector<complex<T>> r = correlate ? kfr::correlate(x, y) : kfr::convolve(x, y);
        std::memcpy(out, r.data(), r.size() * sizeof(complex<T>));
        return r.size();
    }
    univector<T> x(na), y(nb);
    std::memcpy(x.data(), a, na * sizeof(T));
    std::memcpy(y.data(), b, nb * sizeof(T));
    univector<T> r = correlate ? kfr::correlate(x, y) : kfr::convolve(x, y);
    std::memcpy(out, r.data(), r.size() * sizeof(T));
    return r.size();
}

template <typename T>
int run_md(T* out, const T* in, size_t dims, const unsigned* shp, int inverse)
{
    shape<dynamic_shape> sh(dims);
    for (size_t i = 0; i < dims; i++)
        sh[i] = shp[i];
    dft_plan_md<T, dynamic_shape> plan(sh);
    univector<u8> temp(plan.temp_size);
    plan.execute(reinterpret_cast<complex<T>*>(out), reinterpret_cast<const complex<T>*>(in), temp.data(),
                 inverse != 0);
    return 0;
}

template <typename T>
int run_md_real(T* out, const T* in, size_t dims, const unsigned* shp, int inverse, int real_out_is_enough)
{
    shape<dynamic_shape> sh(dims);
    for (size_t i = 0; i < dims; i++)
        sh[i] = shp[i];
    dft_plan_md_real<T, dynamic_shape> plan(sh, real_out_is_enough != 0);
    univector<u8> temp(plan.temp_size);
    if (!inverse)
        plan.execute(reinterpret_cast<complex<T>*>(out), in, temp.data(), cdirect_t{});
    else
        plan.execute(out, reinterpret_cast<const complex<T>*>(in), temp.data(), cinvert_t{});
    return 0;
}

struct any_filter
{
    int is_complex;
    void* f;
};

template <typename T>
void* filter_create(const T* taps, size_t ntaps, size_t block, int is_complex)
{
    any_filter* h  = new any_filter;
    h->is_complex = is_complex;
    if (is_complex)
    {
        univector<complex<T>> t(ntaps);
        std::memcpy(t.data(), taps, ntaps * sizeof(complex<T>));
        h->f = new convolve_filter<complex<T>>(t, block ? block : 1024);
    }
    else
    {
        univector<T> t(ntaps);
        std::memcpy(t.data(), taps, ntaps * sizeof(T));
        h->f = new convolve_filter<T>(t, block ? block : 1024);
    }
    return h;
}

template <typename T>
void filter_process(void* vh, T* out, const T* in, size_t n)
{
    any_filter* h = static_cast<any_filter*>(vh);
    if (h->is_complex)
        static_cast<convolve_filter<complex<T>>*>(h->f)->apply(reinterpret_cast<complex<T>*>(out),
                                                               reinterpret_cast<const complex<T>*>(in), n);
    else
        static_cast<convolve_filter<T>*>(h->f)->apply(out, in, n);
}

template <typename T>
void filter_reset(void* vh)
{
    any_filter* h = static_cast<any_filter*>(vh);
    if (h->is_complex)
        static_cast<convolve_filter<complex<T>>*>(h->f)->reset();
    else
        static_cast<convolve_filter<T>*>(h->f)->reset();
}

template <typename T>
void filter_delete(void* vh)
{
    any_filter* h = static_cast<any_filter*>(vh);
    if (!h)
        return;
    if (h->is_complex)
        delete static_cast<convolve_filter<complex<T>>*>(h->f);
    else
        delete static_cast<convolve_filter<T>*>(h->f);
    delete h;
}
} // namespace

#define REF_API(T, SFX)                                                                                   \
    extern "C" __attribute__((visibility("default"))) int ref_dft##SFX(T* out, const T* in, size_t n,    \
                                                                      size_t batch, int inverse,         \
                                                                      int threads)                       \
    {                                                                                                    \
        return run_dft<T>(out, in, n, batch, inverse, threads);                                          \
    }                                                                                                    \
    extern "C" __attribute__((visibility("default"))) int ref_dft_real##SFX(                             \
        T* out, const T* in, size_t n, int ccs, size_t batch, int threads)                               \
    {                                                                                                    \
        return run_real<T>(out, in, n, ccs, batch, 0, threads);                                          \
    }                                                                                                    \
    extern "C" __attribute__((visibility("default"))) int ref_dft_real_inverse##SFX(                     \
        T* out, const T* in, size_t n, int ccs, size_t batch, int threads)                               \
    {                                                                                                    \
        return run_real<T>(out, in, n, ccs, batch, 1, threads);                                          \
    }                                                                                                    \
    extern "C" __attribute__((visibility("default"))) int ref_dct##SFX(T* out, const T* in, size_t n,    \
                                                                      int inverse, size_t batch,         \
                                                                      int threads)                       \
    {                                                                                                    \
        return run_dct<T>(out, in, n, inverse, batch, threads);                                          \
    }                                                                                                    \
    extern "C" __attribute__((visibility("default"))) size_t ref_convolve##SFX(                          \
        T* out, const T* a, size_t na, const T* b, size_t nb, int correlate, int is_complex)             \
    {                                                                                                    \
        return run_convolve<T>(out, a, na, b, nb, correlate, is_complex);                                \
    }                                                                                                    \
    extern "C" __attribute__((visibility("default"))) void* ref_filter_create##SFX(                      \
        const T* taps, size_t ntaps, size_t block, int is_complex)                                       \
    {                                                                                                    \
        return filter_create<T>(taps, ntaps, block, is_complex);                                         \
    }                                                                                                    \
    extern "C" __attribute__((visibility("default"))) void ref_filter_process##SFX(void* f, T* out,      \
                                                                                  const T* in, size_t n) \
    {                                                                                                    \
        filter_process<T>(f, out, in, n);                                                                \
    }                                                                                                    \
    extern "C" __attribute__((visibility("default"))) void ref_filter_reset##SFX(void* f)                \
    {                                                                                                    \
        filter_reset<T>(f);                                                                              \
    }                                                                                                    \
    extern "C" __attribute__((visibility("default"))) void ref_filter_delete##SFX(void* f)               \
    {                                                                                                    \
        filter_delete<T>(f);                                                                             \
    }

REF_API(double, _f64)
REF_API(float, _f32)

extern "C" __attribute__((visibility("default"))) int ref_dft_md_f64(double* out, const double* in, size_t dims,
                                                                     const unsigned* shape, int inverse)
{
    return run_md<double>(out, in, dims, shape, inverse);
}
extern "C" __attribute__((visibility("default"))) int ref_dft_md_real_f64(double* out, const double* in, size_t dims,
                                                                          const unsigned* shape, int inverse,
                                                                          int real_out_is_enough)
{
    return run_md_real<double>(out, in, dims, shape, inverse, real_out_is_enough);
}

// Timed baseline: one dft_plan<float> built once (plan creation excluded), shared const across `threads`
// std::threads over the batch, each with its own temp (the CPU-baseline method: one shared plan, per-thread
// temp, best of `reps` runs).  Returns the best wall time of one pass over the batch, in seconds.
extern "C" __attribute__((visibility("default"))) double ref_dft_time_f32(float* out, const float* in, size_t n,
                                                                          size_t batch, int inverse, int threads,
                                                                          int reps)
{
    if (n == 0 || batch == 0)
        return 0.0;
    const dft_plan<float> plan(n);
    if (threads < 1)
        threads = 1;
    if (static_cast<size_t>(threads) > batch)
        threads = static_cast<int>(batch);
    std::vector<univector<u8>> temps(threads, univector<u8>(plan.temp_size));
    double best = 1e30;
    for (int r = 0; r < (reps < 1 ? 1 : reps); r++)
    {
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<std::thread> pool;
        for (int t = 0; t < threads; t++)
        {
            const size_t b0 = batch * t / threads, b1 = batch * (t + 1) / threads;
            pool.emplace_back(
                [&, t, b0, b1]
                {
                    for (size_t b = b0; b < b1; b++)
                        plan.execute(reinterpret_cast<complex<float>*>(out) + b * n,
                                     reinterpret_cast<const complex<float>*>(in) + b * n, temps[t].data(),
                                     inverse != 0);
                });
        }
        for (auto& th : pool)
            th.join();
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        best            = dt < best ? dt : best;
    }
    return best;
}

// kfr::fft_multiply (acc NULL) and the three-operand kfr::fft_multiply_accumulate over n complex values
// (include/kfr/dft/fft.hpp:983-1020).
template <typename T>
void run_fft_multiply(T* dst, const T* acc, const T* a, const T* b, size_t n, int perm)
{
    using C = complex<T>;
    univector<C> d(n), s1(reinterpret_cast<const C*>(a), reinterpret_cast<const C*>(a) + n),
        s2(reinterpret_cast<const C*>(b), reinterpret_cast<const C*>(b) + n);
    const dft_pack_format fmt = perm ? dft_pack_format::Perm : dft_pack_format::CCs;
    if (acc)
    {
        univector<C> s0(reinterpret_cast<const C*>(acc), reinterpret_cast<const C*>(acc) + n);
        fft_multiply_accumulate(d, s0, s1, s2, fmt);
    }
    else
        fft_multiply(d, s1, s2, fmt);
    std::memcpy(dst, d.data(), n * sizeof(C));
}
extern "C" __attribute__((visibility("default"))) void ref_fft_multiply_f32(float* dst, const float* acc,
                                                                           const float* a, const float* b,
                                                                           size_t n, int perm)
{
    run_fft_multiply<float>(dst, acc, a, b, n, perm);
}
extern "C" __attribute__((visibility("default"))) void ref_fft_multiply_f64(double* dst, const double* acc,
                                                                           const double* a, const double* b,
                                                                           size_t n, int perm)
{
    run_fft_multiply<double>(dst, acc, a, b, n, perm);
}

// fir_filter<T>::process_buffer is `dest = fir(src, std::ref(state))` (src/dsp/fir.cpp:54-57); the same
// expression over the same state type is evaluated here, header-only.
template <typename T>
void* fir_create(const T* taps, size_t ntaps)
{
    return new fir_state<T, T>(make_univector(taps, ntaps));
}
template <typename T>
void fir_process(void* f, T* out, const T* in, size_t n)
{
    make_univector(out, n) = fir(make_univector(in, n), std::ref(*static_cast<fir_state<T, T>*>(f)));
}
template <typename T>
void fir_reset(void* f)
{
    auto* s             = static_cast<fir_state<T, T>*>(f);
    s->delayline        = scalar(T(0));
    s->delayline_cursor = 0;
}
#define REF_FIR(T, SFX)                                                                                          \
    extern "C" __attribute__((visibility("default"))) void* ref_fir_create##SFX(const T* taps, size_t ntaps)     \
    {                                                                                                            \
        return fir_create<T>(taps, ntaps);                                                                       \
    }                                                                                                            \
    extern "C" __attribute__((visibility("default"))) void ref_fir_process##SFX(void* f, T* out, const T* in,    \
                                                                              size_t n)                          \
    {                                                                                                            \
        fir_process<T>(f, out, in, n);                                                                           \
    }                                                                                                            \
    extern "C" __attribute__((visibility("default"))) void ref_fir_reset##SFX(void* f) { fir_reset<T>(f); }      \
    extern "C" __attribute__((visibility("default"))) void ref_fir_delete##SFX(void* f)                          \
    {                                                                                                            \
        delete static_cast<fir_state<T, T>*>(f);                                                                 \
    }
REF_FIR(float, _f32)
REF_FIR(double, _f64)

extern "C" __attribute__((visibility("default"))) void ref_dft_dump_f32(size_t n)
{
    dft_plan<float> plan(n);
    plan.dump();
}
