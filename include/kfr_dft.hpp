// kfr_dft.hpp: KFR's C++ DFT interface (include/kfr/dft/fft.hpp, include/kfr/dft/convolution.hpp,
// include/kfr/dft/cache.hpp) over the GB300 library's C ABI (kfr_capi.h, libkfr_capi.so).
//
// Code written against KFR's dft_plan<T>, dft_plan_real<T>, dft_plan_md<T>, dft_plan_md_real<T>,
// dct_plan<T>, convolve_filter<T>, convolve / correlate / autocorrelate, dft_cache and the dft() / idft() /
// realdft() / irealdft() helpers compiles against this header unchanged for the members listed here: the
// names, argument order and meaning (unscaled inverses, CCs / Perm packing, temp may be NULL) are the
// reference's.  Buffers may be host or device memory.  Errors are thrown as kfr::logic_error (invalid use,
// like the reference's KFR_LOGIC_CHECK) or std::runtime_error (device errors).
#pragma once

#include <complex>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "kfr_capi.h"

namespace kfr
{

using u8 = std::uint8_t;
template <typename T>
using complex = std::complex<T>;
template <typename T>
using univector = std::vector<T>;

struct logic_error : std::logic_error
{
    using std::logic_error::logic_error;
};

enum class dft_pack_format
{
    Perm = 0,
    CCs  = 1
};

namespace gpu_detail
{
inline void check()
{
    const char* e = kfr_last_error();
    if (e && *e)
    {
        const std::string msg(e);
        if (msg.find("requires") != std::string::npos || msg.find("invalid") != std::string::npos ||
            msg.find("NULL") != std::string::npos || msg.find("not supported") != std::string::npos)
            throw logic_error(msg);
        throw std::runtime_error(msg);
    }
}

template <typename T>
struct api;

template <>
struct api<float>
{
    using plan_t  = KFR_DFT_PLAN_F32;
    using rplan_t = KFR_DFT_REAL_PLAN_F32;
    using dct_t   = KFR_DCT_PLAN_F32;
    using flt_t   = KFR_FILTER_F32;
    static plan_t* create(size_t n) { return kfr_dft_create_plan_f32(n); }
    static plan_t* create_md(size_t d, const unsigned* s) { return kfr_dft_create_md_plan_f32(d, s); }
    static void del(plan_t* p) { kfr_dft_delete_plan_f32(p); }
    static size_t temp(plan_t* p) { return kfr_dft_get_temp_size_f32(p); }
    static void exec(plan_t* p, complex<float>* o, const complex<float>* i, u8* t, bool inv, size_t batch)
    {
        kfr_dft_execute_batch_f32(p, batch, reinterpret_cast<kfr_c32*>(o), reinterpret_cast<const kfr_c32*>(i), t, inv,
                                  nullptr);
    }
    static void dump(plan_t* p) { kfr_dft_dump_f32(p); }
    static size_t prog_total(plan_t* p) { return kfr_dft_progressive_total_steps_f32(p); }
    static size_t prog_start(plan_t* p, complex<float>* o, const complex<float>* i, u8* t, bool inv)
    {
        return kfr_dft_progressive_start_f32(p, reinterpret_cast<kfr_c32*>(o), reinterpret_cast<const kfr_c32*>(i), t, inv);
    }
    static void prog_step(plan_t* p, size_t step) { kfr_dft_progressive_step_f32(p, step); }
    static rplan_t* rcreate(size_t n, dft_pack_format f)
    {
        return kfr_dft_real_create_plan_f32(n, static_cast<KFR_DFT_PACK_FORMAT>(f));
    }
    static rplan_t* rcreate_md(size_t d, const unsigned* s, bool roe) { return kfr_dft_real_create_md_plan_f32(d, s, roe); }
    static void rdel(rplan_t* p) { kfr_dft_real_delete_plan_f32(p); }
    static size_t rtemp(rplan_t* p) { return kfr_dft_real_get_temp_size_f32(p); }
    static void rfwd(rplan_t* p, complex<float>* o, const float* i, u8* t, size_t batch)
    {
        kfr_dft_real_execute_batch_f32(p, batch, reinterpret_cast<kfr_c32*>(o), i, t, nullptr);
    }
    static void rinv(rplan_t* p, float* o, const complex<float>* i, u8* t, size_t batch)
    {
        kfr_dft_real_execute_inverse_batch_f32(p, batch, o, reinterpret_cast<const kfr_c32*>(i), t, nullptr);
    }
    static void rdump(rplan_t* p) { kfr_dft_real_dump_f32(p); }
    static dct_t* dcreate(size_t n) { return kfr_dct_create_plan_f32(n); }
    static void ddel(dct_t* p) { kfr_dct_delete_plan_f32(p); }
    static size_t dtemp(dct_t* p) { return kfr_dct_get_temp_size_f32(p); }
    static void dexec(dct_t* p, float* o, const float* i, u8* t, bool inv, size_t batch)
    {
        kfr_dct_execute_batch_f32(p, batch, o, i, t, inv, nullptr);
    }
    static flt_t* fcreate(const float* taps, size_t n, size_t block) { return kfr_filter_create_convolution_plan_f32(taps, n, block); }
    static void fdel(flt_t* p) { kfr_filter_delete_plan_f32(p); }
    static void fproc(flt_t* p, float* o, const float* i, size_t n) { kfr_filter_process_f32(p, o, i, n); }
    static void freset(flt_t* p) { kfr_filter_reset_f32(p); }
    static size_t conv(float* o, const float* a, size_t na, const float* b, size_t nb) { return kfr_convolve_f32(o, a, na, b, nb); }
    static size_t corr(float* o, const float* a, size_t na, const float* b, size_t nb) { return kfr_correlate_f32(o, a, na, b, nb); }
    static size_t conv(complex<float>* o, const complex<float>* a, size_t na, const complex<float>* b, size_t nb)
    {
        return kfr_convolve_c32(reinterpret_cast<kfr_c32*>(o), reinterpret_cast<const kfr_c32*>(a), na,
                                reinterpret_cast<const kfr_c32*>(b), nb);
    }
    static size_t corr(complex<float>* o, const complex<float>* a, size_t na, const complex<float>* b, size_t nb)
    {
        return kfr_correlate_c32(reinterpret_cast<kfr_c32*>(o), reinterpret_cast<const kfr_c32*>(a), na,
                                 reinterpret_cast<const kfr_c32*>(b), nb);
    }
    static size_t acorr(float* o, const float* a, size_t n) { return kfr_autocorrelate_f32(o, a, n); }
};

template <>
struct api<double>
{
    using plan_t  = KFR_DFT_PLAN_F64;
    using rplan_t = KFR_DFT_REAL_PLAN_F64;
    using dct_t   = KFR_DCT_PLAN_F64;
    using flt_t   = KFR_FILTER_F64;
    static plan_t* create(size_t n) { return kfr_dft_create_plan_f64(n); }
    static plan_t* create_md(size_t d, const unsigned* s) { return kfr_dft_create_md_plan_f64(d, s); }
    static void del(plan_t* p) { kfr_dft_delete_plan_f64(p); }
    static size_t temp(plan_t* p) { return kfr_dft_get_temp_size_f64(p); }
    static void exec(plan_t* p, complex<double>* o, const complex<double>* i, u8* t, bool inv, size_t batch)
    {
        kfr_dft_execute_batch_f64(p, batch, reinterpret_cast<kfr_c64*>(o), reinterpret_cast<const kfr_c64*>(i), t, inv,
                                  nullptr);
    }
    static void dump(plan_t* p) { kfr_dft_dump_f64(p); }
    static size_t prog_total(plan_t* p) { return kfr_dft_progressive_total_steps_f64(p); }
    static size_t prog_start(plan_t* p, complex<double>* o, const complex<double>* i, u8* t, bool inv)
    {
        return kfr_dft_progressive_start_f64(p, reinterpret_cast<kfr_c64*>(o), reinterpret_cast<const kfr_c64*>(i), t, inv);
    }
    static void prog_step(plan_t* p, size_t step) { kfr_dft_progressive_step_f64(p, step); }
    static rplan_t* rcreate(size_t n, dft_pack_format f)
    {
        return kfr_dft_real_create_plan_f64(n, static_cast<KFR_DFT_PACK_FORMAT>(f));
    }
    static rplan_t* rcreate_md(size_t d, const unsigned* s, bool roe) { return kfr_dft_real_create_md_plan_f64(d, s, roe); }
    static void rdel(rplan_t* p) { kfr_dft_real_delete_plan_f64(p); }
    static size_t rtemp(rplan_t* p) { return kfr_dft_real_get_temp_size_f64(p); }
    static void rfwd(rplan_t* p, complex<double>* o, const double* i, u8* t, size_t batch)
    {
        kfr_dft_real_execute_batch_f64(p, batch, reinterpret_cast<kfr_c64*>(o), i, t, nullptr);
    }
    static void rinv(rplan_t* p, double* o, const complex<double>* i, u8* t, size_t batch)
    {
        kfr_dft_real_execute_inverse_batch_f64(p, batch, o, reinterpret_cast<const kfr_c64*>(i), t, nullptr);
    }
    static void rdump(rplan_t* p) { kfr_dft_real_dump_f64(p); }
    static dct_t* dcreate(size_t n) { return kfr_dct_create_plan_f64(n); }
    static void ddel(dct_t* p) { kfr_dct_delete_plan_f64(p); }
    static size_t dtemp(dct_t* p) { return kfr_dct_get_temp_size_f64(p); }
    static void dexec(dct_t* p, double* o, const double* i, u8* t, bool inv, size_t batch)
    {
        kfr_dct_execute_batch_f64(p, batch, o, i, t, inv, nullptr);
    }
    static flt_t* fcreate(const double* taps, size_t n, size_t block) { return kfr_filter_create_convolution_plan_f64(taps, n, block); }
    static void fdel(flt_t* p) { kfr_filter_delete_plan_f64(p); }
    static void fproc(flt_t* p, double* o, const double* i, size_t n) { kfr_filter_process_f64(p, o, i, n); }
    static void freset(flt_t* p) { kfr_filter_reset_f64(p); }
    static size_t conv(double* o, const double* a, size_t na, const double* b, size_t nb) { return kfr_convolve_f64(o, a, na, b, nb); }
    static size_t corr(double* o, const double* a, size_t na, const double* b, size_t nb) { return kfr_correlate_f64(o, a, na, b, nb); }
    static size_t conv(complex<double>* o, const complex<double>* a, size_t na, const complex<double>* b, size_t nb)
    {
        return kfr_convolve_c64(reinterpret_cast<kfr_c64*>(o), reinterpret_cast<const kfr_c64*>(a), na,
                                reinterpret_cast<const kfr_c64*>(b), nb);
    }
    static size_t corr(complex<double>* o, const complex<double>* a, size_t na, const complex<double>* b, size_t nb)
    {
        return kfr_correlate_c64(reinterpret_cast<kfr_c64*>(o), reinterpret_cast<const kfr_c64*>(a), na,
                                 reinterpret_cast<const kfr_c64*>(b), nb);
    }
    static size_t acorr(double* o, const double* a, size_t n) { return kfr_autocorrelate_f64(o, a, n); }
};

template <typename T>
struct scalar_of
{
    using type = T;
};
template <typename T>
struct scalar_of<complex<T>>
{
    using type = T;
};
} // namespace gpu_detail

/// Complex DFT of any length (include/kfr/dft/fft.hpp:183-456).  Movable, not copyable.
template <typename T>
struct dft_plan
{
    size_t size      = 0;
    size_t temp_size = 0;

    dft_plan() = default;
    explicit dft_plan(size_t size_) : size(size_), h_(gpu_detail::api<T>::create(size_))
    {
        if (!h_)
            gpu_detail::check();
        temp_size = gpu_detail::api<T>::temp(h_.get());
    }
    bool is_initialized() const { return size != 0; }
    void dump() const
    {
        gpu_detail::api<T>::dump(h_.get());
        gpu_detail::check();
    }
    /// No scaling on inverse; out may equal in; temp may be NULL.
    void execute(complex<T>* out, const complex<T>* in, u8* temp, bool inverse = false) const
    {
        gpu_detail::api<T>::exec(h_.get(), out, in, temp, inverse, 1);
        gpu_detail::check();
    }
    void execute(univector<complex<T>>& out, const univector<complex<T>>& in, univector<u8>& temp,
                 bool inverse = false) const
    {
        execute(out.data(), in.data(), temp.data(), inverse);
    }
    void execute(univector<complex<T>>& out, const univector<complex<T>>& in, u8* temp, bool inverse = false) const
    {
        execute(out.data(), in.data(), temp, inverse);
    }
    /// Extension: `batch` signals back to back.
    void execute_batch(complex<T>* out, const complex<T>* in, size_t batch, u8* temp = nullptr,
                       bool inverse = false) const
    {
        gpu_detail::api<T>::exec(h_.get(), out, in, temp, inverse, batch);
        gpu_detail::check();
    }

    /// Progressive execution (include/kfr/dft/fft.hpp:393-439): one step is one kernel launch of the plan
    /// (the reference runs one stage per step); `out` holds the result after the last step.  One
    /// progressive execution per plan at a time.
    struct progressive
    {
        bool inverse;
        complex<T>* out;
        const complex<T>* in;
        u8* temp;
        size_t step  = 0;
        size_t total = 0; // steps of this execution
    };
    size_t progressive_total_steps() const
    {
        const size_t n = gpu_detail::api<T>::prog_total(h_.get());
        gpu_detail::check();
        return n;
    }
    progressive progressive_start(bool inverse, complex<T>* out, const complex<T>* in, u8* temp) const
    {
        if (!is_initialized())
            throw logic_error("dft_plan is not initialized");
        progressive p{ inverse, out, in, temp, 0, 0 };
        p.total = gpu_detail::api<T>::prog_start(h_.get(), out, in, temp, inverse);
        gpu_detail::check();
        return p;
    }
    bool progressive_step(progressive& p) const
    {
        gpu_detail::api<T>::prog_step(h_.get(), p.step);
        gpu_detail::check();
        return ++p.step < p.total;
    }

protected:
    struct deleter
    {
        void operator()(typename gpu_detail::api<T>::plan_t* p) const { gpu_detail::api<T>::del(p); }
    };
    std::unique_ptr<typename gpu_detail::api<T>::plan_t, deleter> h_;
};

/// Multi-dimensional complex DFT over a row-major array (include/kfr/dft/fft.hpp:568-702).
template <typename T, typename Shape = std::vector<size_t>>
struct dft_plan_md
{
    std::vector<size_t> size;
    size_t temp_size = 0;
    explicit dft_plan_md(const Shape& shape) : size(shape.begin(), shape.end())
    {
        std::vector<unsigned> s(size.begin(), size.end());
        h_.reset(gpu_detail::api<T>::create_md(s.size(), s.data()));
        if (!h_)
            gpu_detail::check();
        temp_size = gpu_detail::api<T>::temp(h_.get());
    }
    void execute(complex<T>* out, const complex<T>* in, u8* temp, bool inverse = false) const
    {
        gpu_detail::api<T>::exec(h_.get(), out, in, temp, inverse, 1);
        gpu_detail::check();
    }

private:
    struct deleter
    {
        void operator()(typename gpu_detail::api<T>::plan_t* p) const { gpu_detail::api<T>::del(p); }
    };
    std::unique_ptr<typename gpu_detail::api<T>::plan_t, deleter> h_;
};

/// Real DFT of even length (include/kfr/dft/fft.hpp:458-566).
template <typename T>
struct dft_plan_real
{
    size_t size          = 0;
    size_t temp_size     = 0;
    dft_pack_format fmt  = dft_pack_format::CCs;

    dft_plan_real() = default;
    explicit dft_plan_real(size_t size_, dft_pack_format fmt_ = dft_pack_format::CCs) : size(size_), fmt(fmt_)
    {
        if (size_ % 2 != 0)
            throw logic_error("dft_plan_real requires size to be even");
        h_.reset(gpu_detail::api<T>::rcreate(size_, fmt_));
        if (!h_)
            gpu_detail::check();
        temp_size = gpu_detail::api<T>::rtemp(h_.get());
    }
    bool is_initialized() const { return size != 0; }
    size_t complex_size() const { return complex_size_for(size, fmt); }
    static constexpr size_t complex_size_for(size_t size, dft_pack_format fmt)
    {
        return fmt == dft_pack_format::CCs ? size / 2 + 1 : size / 2;
    }
    void dump() const
    {
        gpu_detail::api<T>::rdump(h_.get());
        gpu_detail::check();
    }
    /// forward: size reals -> complex_size() complex values
    void execute(complex<T>* out, const T* in, u8* temp) const
    {
        gpu_detail::api<T>::rfwd(h_.get(), out, in, temp, 1);
        gpu_detail::check();
    }
    /// inverse (unscaled): complex_size() complex values -> size reals
    void execute(T* out, const complex<T>* in, u8* temp) const
    {
        gpu_detail::api<T>::rinv(h_.get(), out, in, temp, 1);
        gpu_detail::check();
    }
    void execute(univector<complex<T>>& out, const univector<T>& in, univector<u8>& temp) const
    {
        execute(out.data(), in.data(), temp.data());
    }
    void execute(univector<T>& out, const univector<complex<T>>& in, univector<u8>& temp) const
    {
        execute(out.data(), in.data(), temp.data());
    }

private:
    struct deleter
    {
        void operator()(typename gpu_detail::api<T>::rplan_t* p) const { gpu_detail::api<T>::rdel(p); }
    };
    std::unique_ptr<typename gpu_detail::api<T>::rplan_t, deleter> h_;
};

/// Multi-dimensional real DFT (include/kfr/dft/fft.hpp:704-924): CCs along the last axis.
template <typename T, typename Shape = std::vector<size_t>>
struct dft_plan_md_real
{
    std::vector<size_t> size;
    size_t temp_size = 0;
    bool real_out_is_enough;
    explicit dft_plan_md_real(const Shape& shape, bool real_out_is_enough_ = false)
        : size(shape.begin(), shape.end()), real_out_is_enough(real_out_is_enough_)
    {
        std::vector<unsigned> s(size.begin(), size.end());
        h_.reset(gpu_detail::api<T>::rcreate_md(s.size(), s.data(), real_out_is_enough_));
        if (!h_)
            gpu_detail::check();
        temp_size = gpu_detail::api<T>::rtemp(h_.get());
    }
    std::vector<size_t> complex_size() const
    {
        std::vector<size_t> c = size;
        if (!c.empty())
            c.back() = c.back() / 2 + 1;
        return c;
    }
    void execute(complex<T>* out, const T* in, u8* temp) const
    {
        gpu_detail::api<T>::rfwd(h_.get(), out, in, temp, 1);
        gpu_detail::check();
    }
    void execute(T* out, const complex<T>* in, u8* temp) const
    {
        gpu_detail::api<T>::rinv(h_.get(), out, in, temp, 1);
        gpu_detail::check();
    }

private:
    struct deleter
    {
        void operator()(typename gpu_detail::api<T>::rplan_t* p) const { gpu_detail::api<T>::rdel(p); }
    };
    std::unique_ptr<typename gpu_detail::api<T>::rplan_t, deleter> h_;
};

/// DCT-II (forward) and DCT-III with X0 halved (inverse), unscaled (include/kfr/dft/fft.hpp:926-978).
template <typename T>
struct dct_plan
{
    size_t size      = 0;
    size_t temp_size = 0;
    explicit dct_plan(size_t size_) : size(size_), h_(gpu_detail::api<T>::dcreate(size_))
    {
        if (!h_)
            gpu_detail::check();
        temp_size = gpu_detail::api<T>::dtemp(h_.get());
    }
    void execute(T* out, const T* in, u8* temp, bool inverse = false) const
    {
        gpu_detail::api<T>::dexec(h_.get(), out, in, temp, inverse, 1);
        gpu_detail::check();
    }
    void execute(univector<T>& out, const univector<T>& in, univector<u8>& temp, bool inverse = false) const
    {
        execute(out.data(), in.data(), temp.data(), inverse);
    }

private:
    struct deleter
    {
        void operator()(typename gpu_detail::api<T>::dct_t* p) const { gpu_detail::api<T>::ddel(p); }
    };
    std::unique_ptr<typename gpu_detail::api<T>::dct_t, deleter> h_;
};

/// Streaming FFT convolution filter (include/kfr/dft/convolution.hpp:98-148): causal FIR output, state
/// kept across apply() calls until reset().  Real samples (the C API's filters).
template <typename T>
class convolve_filter
{
public:
    explicit convolve_filter(const univector<T>& taps, size_t block_size = 1024)
        : block_size_(block_size), h_(gpu_detail::api<T>::fcreate(taps.data(), taps.size(), block_size))
    {
        if (!h_)
            gpu_detail::check();
    }
    void apply(T* dest, const T* src, size_t size)
    {
        gpu_detail::api<T>::fproc(h_.get(), dest, src, size);
        gpu_detail::check();
    }
    void apply(univector<T>& dest, const univector<T>& src) { apply(dest.data(), src.data(), src.size()); }
    void apply(univector<T>& inout) { apply(inout.data(), inout.data(), inout.size()); }
    void reset()
    {
        gpu_detail::api<T>::freset(h_.get());
        gpu_detail::check();
    }
    size_t input_block_size() const { return block_size_; }

private:
    struct deleter
    {
        void operator()(typename gpu_detail::api<T>::flt_t* p) const { gpu_detail::api<T>::fdel(p); }
    };
    size_t block_size_;
    std::unique_ptr<typename gpu_detail::api<T>::flt_t, deleter> h_;
};

/// Linear convolution (include/kfr/dft/convolution.hpp:53-58): n1 + n2 - 1 values; complex inputs keep
/// only the real part, as the reference does.
template <typename T>
univector<T> convolve(const univector<T>& a, const univector<T>& b)
{
    univector<T> out(a.size() + b.size() - 1);
    gpu_detail::api<typename gpu_detail::scalar_of<T>::type>::conv(out.data(), a.data(), a.size(), b.data(), b.size());
    gpu_detail::check();
    return out;
}
/// Correlation: b reversed (include/kfr/dft/convolution.hpp:61-66).
template <typename T>
univector<T> correlate(const univector<T>& a, const univector<T>& b)
{
    univector<T> out(a.size() + b.size() - 1);
    gpu_detail::api<typename gpu_detail::scalar_of<T>::type>::corr(out.data(), a.data(), a.size(), b.data(), b.size());
    gpu_detail::check();
    return out;
}
/// Lags 0 .. n-1 of correlate(a, a) (include/kfr/dft/convolution.hpp:69-76).
template <typename T>
univector<T> autocorrelate(const univector<T>& a)
{
    univector<T> out(a.size());
    gpu_detail::api<T>::acorr(out.data(), a.data(), a.size());
    gpu_detail::check();
    return out;
}

/// Process-wide plan cache (include/kfr/dft/cache.hpp:45-171), mutex-guarded.
struct dft_cache
{
    static dft_cache& instance()
    {
        static dft_cache c;
        return c;
    }
    template <typename T>
    std::shared_ptr<const dft_plan<T>> get(size_t size)
    {
        std::lock_guard<std::mutex> lock(mu_);
        auto& list = plans<T>();
        for (auto& p : list)
            if (p->size == size)
                return p;
        list.push_back(std::make_shared<const dft_plan<T>>(size));
        return list.back();
    }
    template <typename T>
    std::shared_ptr<const dft_plan_real<T>> getreal(size_t size)
    {
        std::lock_guard<std::mutex> lock(mu_);
        auto& list = real_plans<T>();
        for (auto& p : list)
            if (p->size == size)
                return p;
        list.push_back(std::make_shared<const dft_plan_real<T>>(size));
        return list.back();
    }
    void clear()
    {
        std::lock_guard<std::mutex> lock(mu_);
        plans<float>().clear();
        plans<double>().clear();
        real_plans<float>().clear();
        real_plans<double>().clear();
        kfr_dft_cache_clear();
    }

private:
    template <typename T>
    std::vector<std::shared_ptr<const dft_plan<T>>>& plans()
    {
        static std::vector<std::shared_ptr<const dft_plan<T>>> v;
        return v;
    }
    template <typename T>
    std::vector<std::shared_ptr<const dft_plan_real<T>>>& real_plans()
    {
        static std::vector<std::shared_ptr<const dft_plan_real<T>>> v;
        return v;
    }
    std::mutex mu_;
};

/// dft / idft / realdft / irealdft helpers (include/kfr/dft/cache.hpp:94-171), through the cache.
template <typename T>
univector<complex<T>> dft(const univector<complex<T>>& input)
{
    univector<complex<T>> out(input.size());
    dft_cache::instance().get<T>(input.size())->execute(out.data(), input.data(), nullptr, false);
    return out;
}
template <typename T>
univector<complex<T>> idft(const univector<complex<T>>& input)
{
    univector<complex<T>> out(input.size());
    dft_cache::instance().get<T>(input.size())->execute(out.data(), input.data(), nullptr, true);
    return out;
}
template <typename T>
univector<complex<T>> realdft(const univector<T>& input)
{
    univector<complex<T>> out(input.size() / 2 + 1);
    dft_cache::instance().getreal<T>(input.size())->execute(out.data(), input.data(), nullptr);
    return out;
}
template <typename T>
univector<T> irealdft(const univector<complex<T>>& input)
{
    const size_t n = (input.size() - 1) * 2;
    univector<T> out(n);
    dft_cache::instance().getreal<T>(n)->execute(out.data(), input.data(), nullptr);
    return out;
}

/// fft_multiply / fft_multiply_accumulate (include/kfr/dft/fft.hpp:983-1020), host-side: spectral product
/// with the Perm format's DC / Nyquist special case.
template <typename T>
void fft_multiply(univector<complex<T>>& dest, const univector<complex<T>>& src1, const univector<complex<T>>& src2,
                  dft_pack_format fmt = dft_pack_format::CCs)
{
    const complex<T> f0(src1[0].real() * src2[0].real(), src1[0].imag() * src2[0].imag());
    dest.resize(src1.size());
    for (size_t i = 0; i < src1.size(); i++)
        dest[i] = src1[i] * src2[i];
    if (fmt == dft_pack_format::Perm)
        dest[0] = f0;
}
template <typename T>
void fft_multiply_accumulate(univector<complex<T>>& dest, const univector<complex<T>>& src1,
                             const univector<complex<T>>& src2, dft_pack_format fmt = dft_pack_format::CCs)
{
    const complex<T> f0(dest[0].real() + src1[0].real() * src2[0].real(),
                        dest[0].imag() + src1[0].imag() * src2[0].imag());
    for (size_t i = 0; i < src1.size(); i++)
        dest[i] += src1[i] * src2[i];
    if (fmt == dft_pack_format::Perm)
        dest[0] = f0;
}

} // namespace kfr
