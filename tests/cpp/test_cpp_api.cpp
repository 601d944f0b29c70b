// C++ drop-in check: code written against KFR's C++ DFT interface, compiled against include/kfr_dft.hpp and
// linked with libkfr_capi.so.  Known answers are the reference's own (tests/dft_test.cpp:107-167, 396-423);
// DFTs are compared with a direct double-precision DFT.  Prints "OK" and returns 0 on success.
#include "kfr_dft.hpp"

#include <cmath>
#include <cstdio>
#include <vector>

using namespace kfr;

static int failures = 0;
#define EXPECT(cond, what)                                                                                  \
    do                                                                                                      \
    {                                                                                                       \
        if (!(cond))                                                                                        \
        {                                                                                                   \
            std::printf("FAIL: %s (%s:%d)\n", what, __FILE__, __LINE__);                                   \
            failures++;                                                                                     \
        }                                                                                                   \
    } while (0)

template <typename V1, typename V2>
static double rms_diff(const V1& a, const V2& b)
{
    double s = 0;
    for (size_t i = 0; i < a.size(); i++)
        s += std::norm(std::complex<double>(a[i]) - std::complex<double>(b[i]));
    return std::sqrt(s / double(a.size()));
}

static std::vector<complex<double>> naive_dft(const std::vector<complex<float>>& x, bool inverse)
{
    const size_t n = x.size();
    std::vector<complex<double>> y(n);
    for (size_t k = 0; k < n; k++)
    {
        complex<double> acc = 0;
        for (size_t j = 0; j < n; j++)
        {
            const double a = (inverse ? 2.0 : -2.0) * M_PI * double((j * k) % n) / double(n);
            acc += complex<double>(x[j]) * complex<double>(std::cos(a), std::sin(a));
        }
        y[k] = acc;
    }
    return y;
}

int main()
{
    // dft_plan<float>: forward, inverse, in place, NULL temp
    for (size_t n : { 1u, 7u, 16u, 100u, 127u, 1000u })
    {
        std::vector<complex<float>> x(n), y(n);
        for (size_t i = 0; i < n; i++)
            x[i] = complex<float>(std::sin(0.37 * i), std::cos(0.11 * i * i));
        dft_plan<float> plan(n);
        EXPECT(plan.size == n, "size");
        plan.execute(y.data(), x.data(), nullptr);
        EXPECT(rms_diff(y, naive_dft(x, false)) < 1e-5 * std::sqrt(double(n)), "forward DFT");
        plan.execute(y.data(), x.data(), nullptr, true);
        EXPECT(rms_diff(y, naive_dft(x, true)) < 1e-5 * std::sqrt(double(n)), "inverse DFT");
        std::vector<complex<float>> z = x;
        plan.execute(z.data(), z.data(), nullptr);
        EXPECT(rms_diff(z, naive_dft(x, false)) < 1e-5 * std::sqrt(double(n)), "in-place DFT");
        // progressive execution ends with the result in out
        auto pr = plan.progressive_start(false, y.data(), x.data(), nullptr);
        while (plan.progressive_step(pr))
        {
        }
        EXPECT(rms_diff(y, naive_dft(x, false)) < 1e-5 * std::sqrt(double(n)), "progressive DFT");
    }
    // dft() / idft() helpers through the cache
    {
        std::vector<complex<float>> x(256);
        for (size_t i = 0; i < x.size(); i++)
            x[i] = complex<float>(float(i % 7) - 3.f, float(i % 3));
        auto X  = dft(x);
        auto xi = idft(X);
        for (auto& v : xi)
            v /= float(x.size());
        EXPECT(rms_diff(xi, x) < 1e-5, "dft/idft round trip");
        EXPECT(dft_cache::instance().get<float>(256).get() == dft_cache::instance().get<float>(256).get(), "cache");
    }
    // dft_plan_real (CCs and Perm) round trip
    for (auto fmt : { dft_pack_format::CCs, dft_pack_format::Perm })
    {
        const size_t n = 1920;
        std::vector<float> x(n), y(n);
        for (size_t i = 0; i < n; i++)
            x[i] = float(std::sin(0.01 * i * i));
        dft_plan_real<float> plan(n, fmt);
        std::vector<complex<float>> X(plan.complex_size());
        plan.execute(X.data(), x.data(), nullptr);
        plan.execute(y.data(), X.data(), nullptr);
        for (auto& v : y)
            v /= float(n);
        EXPECT(rms_diff(y, x) < 1e-5, "real DFT round trip");
    }
    try
    {
        dft_plan_real<float> bad(7);
        EXPECT(false, "odd real size must throw");
    }
    catch (const logic_error&)
    {
    }
    // DCT golden vector (tests/dft_test.cpp:396-423)
    {
        std::vector<float> in(16), out(16);
        for (int i = 0; i < 16; i++)
            in[i] = float(i);
        const double ref[16] = { 120.0, -51.79283109806667, 0.0, -5.6781471211595695, 0.0, -1.9843883778092053, 0.0,
                                 -0.9603691873838152, 0.0, -0.5308329190495176, 0.0, -0.3030379000702155, 0.0,
                                 -0.1584982220313824, 0.0, -0.0494839805703826 };
        dct_plan<float> plan(16);
        plan.execute(out.data(), in.data(), nullptr);
        double e = 0;
        for (int i = 0; i < 16; i++)
            e += (out[i] - ref[i]) * (out[i] - ref[i]);
        EXPECT(std::sqrt(e / 16) < 1e-5, "DCT-II golden");
    }
    // convolve / correlate / convolve_filter golden vectors (tests/dft_test.cpp:107-167)
    {
        std::vector<float> a{ 1, 2, 3, 4, 5 }, b{ 0.25f, 0.5f, 1.0f, -2.0f, 1.5f };
        const std::vector<float> conv{ 0.25f, 1.f, 2.75f, 2.5f, 3.75f, 3.5f, 1.5f, -4.f, 7.5f };
        const std::vector<float> corr{ 1.5f, 1.f, 1.5f, 2.5f, 3.75f, -4.f, 7.75f, 3.5f, 1.25f };
        EXPECT(rms_diff(convolve(a, b), conv) < 1e-4, "convolve");
        EXPECT(rms_diff(correlate(a, b), corr) < 1e-4, "correlate");
        std::vector<float> dest(5);
        convolve_filter<float> f(a);
        f.apply(dest, b);
        EXPECT(rms_diff(dest, std::vector<float>{ 0.25f, 1.f, 2.75f, 2.5f, 3.75f }) < 1e-4, "convolve_filter");
        f.apply(dest, b);
        EXPECT(rms_diff(dest, std::vector<float>{ 0.25f, 1.f, 2.75f, 2.5f, 3.75f }) > 1e-4, "filter state");
        f.reset();
        f.apply(dest, b);
        EXPECT(rms_diff(dest, std::vector<float>{ 0.25f, 1.f, 2.75f, 2.5f, 3.75f }) < 1e-4, "filter reset");
    }
    // dft_plan_md 2-D vs separable direct DFTs
    {
        const size_t r = 6, c = 10;
        std::vector<complex<float>> x(r * c), y(r * c);
        for (size_t i = 0; i < x.size(); i++)
            x[i] = complex<float>(float(std::cos(0.3 * i)), float(i % 5) - 2.f);
        dft_plan_md<float> plan(std::vector<size_t>{ r, c });
        plan.execute(y.data(), x.data(), nullptr);
        std::vector<complex<double>> want(r * c);
        for (size_t k1 = 0; k1 < r; k1++)
            for (size_t k2 = 0; k2 < c; k2++)
            {
                complex<double> acc = 0;
                for (size_t n1 = 0; n1 < r; n1++)
                    for (size_t n2 = 0; n2 < c; n2++)
                    {
                        const double a = -2.0 * M_PI * (double(n1 * k1) / r + double(n2 * k2) / c);
                        acc += complex<double>(x[n1 * c + n2]) * complex<double>(std::cos(a), std::sin(a));
                    }
                want[k1 * c + k2] = acc;
            }
        EXPECT(rms_diff(y, want) < 1e-4, "2-D DFT");
    }
    if (failures)
    {
        std::printf("%d failures\n", failures);
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
