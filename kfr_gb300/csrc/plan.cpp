// Host-side planner and executors (see plan.hpp).
#include "plan.hpp"
#include "tensor.hpp"

#include "ct_table.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <sstream>

namespace kfr_gpu
{

// Scratch regions after the first start on a 256-byte boundary (the bulk and tensor copies of the kernels
// that use them need 16-byte-aligned bases); each such boundary costs at most kAlignSlack elements.
template <typename T>
constexpr long long kAlignSlack = 256 / (2 * (long long)sizeof(T));
inline char* align_scratch(char* p)
{
    return reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(p) + 255) & ~uintptr_t(255));
}

namespace
{
std::atomic<unsigned> g_wait_spins{ kDefaultWaitSpins };
} // namespace

unsigned wait_limit() { return g_wait_spins.load(); }
unsigned set_wait_limit(unsigned spins) { return g_wait_spins.exchange(spins); }

void check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess)
    {
        cudaGetLastError(); // clear a sticky-free error so the next call starts clean
        throw cuda_error(std::string(what) + ": " + cudaGetErrorString(e));
    }
}

// ------------------------------------------------------------------------------------------------------
// dbuf
// ------------------------------------------------------------------------------------------------------

void dbuf::alloc(size_t bytes)
{
    release();
    if (bytes == 0)
        return;
    check(cudaMalloc(&p_, bytes), "cudaMalloc");
    bytes_ = bytes;
}

void dbuf::ensure(size_t bytes)
{
    if (bytes > bytes_)
        alloc(bytes);
}

void dbuf::release()
{
    if (p_)
        cudaFree(p_);
    p_     = nullptr;
    bytes_ = 0;
}

void dbuf::upload(const void* host, size_t bytes)
{
    alloc(bytes);
    if (bytes)
        check(cudaMemcpy(p_, host, bytes, cudaMemcpyHostToDevice), "cudaMemcpy (tables)");
}

// ------------------------------------------------------------------------------------------------------
// Twiddles and factorisation
// ------------------------------------------------------------------------------------------------------

std::complex<double> twiddle(long long k, long long n)
{
    k %= n;
    if (k < 0)
        k += n;
    int q = 0;
    if (n % 2 == 0 && k >= n / 2)
    {
        q += 2;
        k -= n / 2;
    }
    if (n % 4 == 0 && k >= n / 4)
    {
        q += 1;
        k -= n / 4;
    }
    double re = 1.0, im = 0.0;
    if (k != 0)
    {
        const double a = 2.0 * M_PI * (double(k) / double(n));
        re             = std::cos(a);
        im             = -std::sin(a);
    }
    if (q & 1)
    {
        const double t = re;
        re             = im;
        im             = -t;
    }
    if (q & 2)
    {
        re = -re;
        im = -im;
    }
    return { re, im };
}

void host_fft_pow2(std::vector<std::complex<double>>& b)
{
    const long long m = (long long)b.size();
    // iterative radix-2 decimation in time, bit-reversed input order
    for (long long i = 1, j = 0; i < m; i++)
    {
        long long bit = m >> 1;
        for (; j & bit; bit >>= 1)
            j ^= bit;
        j ^= bit;
        if (i < j)
            std::swap(b[i], b[j]);
    }
    for (long long len = 2; len <= m; len <<= 1)
        for (long long i = 0; i < m; i += len)
            for (long long k = 0; k < len / 2; k++)
            {
                const std::complex<double> w = twiddle(k, len);
                const std::complex<double> u = b[i + k], v = b[i + k + len / 2] * w;
                b[i + k]                     = u + v;
                b[i + k + len / 2]           = u - v;
            }
}

// Forward DFT of a[0..n) in place by decimation in time over the smallest prime factor, the roots W_n^k
// read from w (W_N^k, k < N) at stride N / n.
static void host_dft_rec(std::complex<double>* a, long long n, const std::vector<std::complex<double>>& w, long long N)
{
    if (n <= 1)
        return;
    long long p = 2;
    while (p * p <= n && n % p)
        p++;
    if (n % p)
        p = n;
    const long long m = n / p, st = N / n;
    std::vector<std::complex<double>> sub(n);
    for (long long r = 0; r < p; r++)
        for (long long j = 0; j < m; j++)
            sub[r * m + j] = a[j * p + r];
    if (m > 1)
        for (long long r = 0; r < p; r++)
            host_dft_rec(&sub[r * m], m, w, N);
    for (long long k = 0; k < n; k++)
    {
        std::complex<double> acc = 0;
        for (long long r = 0; r < p; r++)
            acc += sub[r * m + k % m] * w[((r * k) % n) * st];
        a[k] = acc;
    }
}

void host_dft_smooth(std::vector<std::complex<double>>& a)
{
    const long long n = (long long)a.size();
    std::vector<std::complex<double>> w(std::max<long long>(n, 1));
    for (long long k = 0; k < n; k++)
        w[k] = twiddle(k, n);
    host_dft_rec(a.data(), n, w, n);
}

void host_dft(std::vector<std::complex<double>>& a)
{
    const long long n = (long long)a.size();
    if (n <= 1)
        return;
    long long p = 2;
    while (p * p <= n && n % p)
        p++;
    if (n % p)
        p = n;
    if (p == n)
    {
        std::vector<std::complex<double>> r(n);
        for (long long k = 0; k < n; k++)
        {
            std::complex<double> acc = 0;
            for (long long j = 0; j < n; j++)
                acc += a[j] * twiddle((j * k) % n, n);
            r[k] = acc;
        }
        a.swap(r);
        return;
    }
    // decimation in time by p: sub-sequences a[p*m + r], m < n/p
    const long long m = n / p;
    std::vector<std::vector<std::complex<double>>> sub(p, std::vector<std::complex<double>>(m));
    for (long long r = 0; r < p; r++)
    {
        for (long long j = 0; j < m; j++)
            sub[r][j] = a[j * p + r];
        host_dft(sub[r]);
    }
    for (long long k = 0; k < n; k++)
    {
        std::complex<double> acc = 0;
        for (long long r = 0; r < p; r++)
            acc += sub[r][k % m] * twiddle((r * k) % n, n);
        a[k] = acc;
    }
}

std::vector<int> factor_radices(long long n)
{
    std::vector<int> r;
    if (n <= 1)
        return r;
    int a = 0;
    while (n % 2 == 0)
    {
        n /= 2;
        a++;
    }
    const int q = a / 4, rem = a % 4;
    if (rem == 1 && q >= 1)
    {
        for (int i = 0; i < q - 1; i++)
            r.push_back(16);
        r.push_back(8);
        r.push_back(4);
    }
    else
    {
        for (int i = 0; i < q; i++)
            r.push_back(16);
        if (rem == 1)
            r.push_back(2);
        else if (rem == 2)
            r.push_back(4);
        else if (rem == 3)
            r.push_back(8);
    }
    while (n % 9 == 0)
    {
        r.push_back(9);
        n /= 9;
    }
    for (int p : { 3, 5, 7, 11, 13 })
        while (n % p == 0)
        {
            r.push_back(p);
            n /= p;
        }
    for (long long p = 17; p * p <= n; p += 2)
        while (n % p == 0)
        {
            if (p > kGenericMax)
                return {};
            r.push_back(int(p));
            n /= p;
        }
    if (n > 1)
    {
        if (n > kGenericMax)
            return {};
        r.push_back(int(n));
    }
    return r;
}

static bool is_codelet(int r)
{
    switch (r)
    {
    case 2:
    case 3:
    case 4:
    case 5:
    case 7:
    case 8:
    case 9:
    case 11:
    case 13:
    case 16: return true;
    // Good-Thomas composites: only in compile-time radix lists (factor_radices never produces them)
    case 6:
    case 10:
    case 12:
    case 14:
    case 15:
    case 18: return true;
    default: return false;
    }
}

// Threads per signal needed by a radix sequence at `ept` elements per thread (0 = infeasible).
int threads_needed(long long n, const std::vector<int>& radices, int ept)
{
    long long ts = 1;
    for (int r : radices)
    {
        long long need;
        if (is_codelet(r))
        {
            if (ept < r)
                return 0;
            const long long per = ept / r;
            need                = (n / r + per - 1) / per;
        }
        else
            need = (n + ept - 1) / ept;
        ts = std::max(ts, need);
    }
    return int(std::min<long long>(ts, 1 << 20));
}

static int ilog2(int x)
{
    int s = 0;
    while ((1 << s) < x)
        s++;
    return s;
}

int smem_budget()
{
    // dynamic shared memory left after the static pass-descriptor array and a small reserve
    static const int budget = max_smem_bytes() - int(sizeof(pass_desc)) * kMaxPasses - 1024;
    return budget;
}

// ------------------------------------------------------------------------------------------------------
// Compile-time kernel registry
// ------------------------------------------------------------------------------------------------------

template <typename T>
bool ct_lookup(int kind, int n, int& ts, std::vector<int>& radices)
{
    if (!std::is_same<T, float>::value)
        return false;
#define KFR_CT_HOST(N, TS, ...)                                                                            \
    if (n == N)                                                                                            \
    {                                                                                                      \
        ts      = TS;                                                                                      \
        radices = { __VA_ARGS__ };                                                                         \
        return true;                                                                                       \
    }
    switch (kind)
    {
    case CT_C2C: KFR_CT_C2C_F32(KFR_CT_HOST) break;
    case CT_BLUESTEIN: KFR_CT_BLUESTEIN_F32(KFR_CT_HOST) break;
    case CT_RADER: KFR_CT_RADER_F32(KFR_CT_HOST) break;
    case CT_FOURSTEP: KFR_CT_FOURSTEP_F32(KFR_CT_HOST) break;
    case CT_REAL: KFR_CT_REAL_F32(KFR_CT_HOST) break;
    case CT_DCT: KFR_CT_DCT_F32(KFR_CT_HOST) break;
    case CT_CONV: KFR_CT_CONV_F32(KFR_CT_HOST) break;
    default: break;
    }
#undef KFR_CT_HOST
    return false;
}

template bool ct_lookup<float>(int, int, int&, std::vector<int>&);
template bool ct_lookup<double>(int, int, int&, std::vector<int>&);

// ------------------------------------------------------------------------------------------------------
// block_program
// ------------------------------------------------------------------------------------------------------

template <typename T>
bool block_program<T>::feasible(long long n)
{
    if (n < 2 || n > (1 << 20))
        return false;
    const auto rad = factor_radices(n);
    if (rad.empty() || int(rad.size()) > kMaxPasses)
        return false;
    if (static_cast<long long>(padded_len_host<T>(int(n))) * static_cast<long long>(2 * sizeof(T)) > smem_budget())
        return false;
    for (int ept : { 16, 32 })
    {
        const int ts = threads_needed(n, rad, ept);
        if (ts > 0 && ts <= max_threads_for(int(sizeof(T)), ept))
            return true;
    }
    return false;
}

template <typename T>
void block_program<T>::build(int n_, int kind, const std::vector<int>* order, int ept_only)
{
    n  = n_;
    ct = 0;
    int cts = 0;
    std::vector<int> ctr;
    if (!order && kind != CT_NONE && ct_lookup<T>(kind, n, cts, ctr))
    {
        radices = ctr;
        ts      = cts;
        ept     = 16;
        ct      = n;
    }
    else
    {
        radices = order ? *order : factor_radices(n);
        if (radices.empty() || int(radices.size()) > kMaxPasses)
            throw std::invalid_argument("internal: length has no one-CTA radix plan");
        long long prod = 1;
        for (int r : radices)
            prod *= r;
        if (prod != n)
            throw std::invalid_argument("internal: radix order does not multiply to the length");
        ept = 0;
        for (int e : { 16, 32 })
        {
            if (ept_only && e != ept_only)
                continue;
            const int t = threads_needed(n, radices, e);
            if (t > 0 && t <= max_threads_for(int(sizeof(T)), e))
            {
                ept = e;
                ts  = t;
                break;
            }
        }
        if (ept == 0)
            throw std::invalid_argument("internal: length exceeds one CTA");
    }
    gstride = padded_len_host<T>(n);
    if (ct && sizeof(T) == 4)
        gstride = ct_group_stride_f32(n, ts);
    std::memset(&desc, 0, sizeof(desc));
    desc.n     = n;
    desc.npass = int(radices.size());
    const auto table = pass_twiddles<T>(radices, desc.pass);
    tw.upload(table.data(), table.size() * sizeof(std::complex<T>));
}

template <typename T>
std::vector<std::complex<T>> pass_twiddles(const std::vector<int>& radices, pass_desc* passes)
{
    std::vector<std::complex<T>> table;
    long long ns = 1;
    for (size_t i = 0; i < radices.size(); i++)
    {
        const int R = radices[i];
        if (passes)
        {
            passes[i].radix  = R;
            passes[i].ns     = int(ns);
            passes[i].div_ns = make_fast_div(uint32_t(ns));
            passes[i].tw_off = int(table.size());
        }
        const long long L = ns * R;
        if (ns > 1)
            for (int r = 1; r < R; r++)
                for (long long k = 0; k < ns; k++)
                {
                    const auto w = twiddle(k * r, L);
                    table.emplace_back(T(w.real()), T(w.imag()));
                }
        if (passes)
            passes[i].wr_off = int(table.size());
        if (!is_codelet(R))
            for (int m = 0; m < R; m++)
            {
                const auto w = twiddle(m, R);
                table.emplace_back(T(w.real()), T(w.imag()));
            }
        ns = L;
    }
    if (table.empty())
        table.emplace_back(T(1), T(0));
    return table;
}

template <typename T>
block_cfg block_program<T>::cfg(long long batch, int spc_cap) const
{
    block_cfg c;
    c.ept              = ept;
    c.ts               = ts;
    const int per_sig  = gstride * int(2 * sizeof(T));
    const int max_thr  = ct ? (sizeof(T) == 4 ? 1024 : 512) : max_threads_for(int(sizeof(T)), ept);
    int spc            = std::max(1, 256 / ts);
    spc                = std::min(spc, std::max(1, max_thr / ts));
    spc                = std::min(spc, std::max(1, smem_budget() / per_sig));
    // keep at least ~2 CTAs per SM when the batch allows it
    const long long want_ctas = 2LL * 152;
    if (batch < want_ctas * spc)
        spc = int(std::max<long long>(1, std::min<long long>(spc, (batch + want_ctas - 1) / want_ctas)));
    if (spc_cap > 0)
        spc = std::min(spc, spc_cap);
    c.spc     = spc;
    c.threads = ((spc * ts + 31) / 32) * 32;
    c.smem    = spc * per_sig;
    c.grid    = (batch + spc - 1) / spc;
    c.ct      = ct;
    return c;
}

template <typename T>
block_cfg block_program<T>::cfg_tile(int tile) const
{
    block_cfg c;
    c.ept     = ept;
    c.ts      = ts;
    c.spc     = tile;
    c.threads = ((tile * ts + 31) / 32) * 32;
    c.smem    = tile * gstride * int(2 * sizeof(T));
    c.grid    = 1;
    c.ct      = ct;
    return c;
}

template <typename T>
std::string block_program<T>::describe() const
{
    std::ostringstream s;
    s << "block_fft n=" << n << " radices=";
    for (size_t i = 0; i < radices.size(); i++)
        s << (i ? "x" : "") << radices[i];
    s << (ct ? " compile-time" : " ept=") ;
    if (!ct)
        s << ept;
    s << " threads/signal=" << ts;
    return s.str();
}

// ------------------------------------------------------------------------------------------------------
// complex_engine
// ------------------------------------------------------------------------------------------------------

static bool is_prime(long long n)
{
    if (n < 2)
        return false;
    for (long long p = 2; p * p <= n; p++)
        if (n % p == 0)
            return false;
    return true;
}

// Relative cost of a one-CTA FFT of length n: one unit per element per codelet pass, R/4 per element for a
// generic radix-R pass (a length-R dot product per output).
static double fft_cost(long long n)
{
    const auto rad = factor_radices(n);
    if (rad.empty())
        return 1e30;
    double c = 0;
    for (int r : rad)
        c += is_codelet(r) ? 1.0 : r / 4.0;
    return double(n) * c;
}

// Twiddles of the radix-16 passes of an L-point tensor-core block FFT (L = 16^p): the pass with stride
// ns > 1 holds W_{16 ns}^{r k} at (r - 1) ns + k (r = 1..15, k < ns), passes in order.
static std::vector<std::complex<float>> tc_pass_twiddles(int L)
{
    std::vector<std::complex<float>> tw;
    for (int ns = 16; ns < L; ns *= 16)
        for (int r = 1; r < 16; r++)
            for (int k = 0; k < ns; k++)
            {
                const auto w = twiddle((long long)r * k, 16LL * ns);
                tw.emplace_back(float(w.real()), float(w.imag()));
            }
    return tw;
}

template <typename T>
complex_engine<T>::complex_engine(long long n, int tensor_mode) : n_(n)
{
    if (sizeof(T) != 4 || (tensor_mode != TC_BF16 && tensor_mode != TC_FP16))
        throw std::invalid_argument("tensor-core plans are single precision with a BF16 or FP16 split");
    // one CTA for 16^2 and 16^3; a four-step of 256- and 4096-point passes for 2^16, 2^20 and 2^24
    switch (n)
    {
    case 256:
    case 4096: break;
    case 1 << 16: n1_ = 256, n2_ = 256; break;
    case 1 << 20: n1_ = 256, n2_ = 4096; break;
    case 1 << 24: n1_ = 4096, n2_ = 4096; break;
    default:
        throw std::invalid_argument(
            "tensor-core plans support lengths 256, 4096, 65536, 2^20 and 2^24 (radix-16 passes only)");
    }
    std::vector<float> cs(512);
    for (int k = 0; k < 16; k++)
        for (int r = 0; r < 16; r++)
        {
            const auto w       = twiddle(k * r, 16); // e^{-2 pi i k r / 16} = cos - i sin
            cs[k * 16 + r]       = float(w.real());
            cs[256 + k * 16 + r] = float(-w.imag());
        }
    tc_cs_.upload(cs.data(), cs.size() * sizeof(float));
    const auto upload_tw = [](dbuf& b, int L)
    {
        const auto tw = tc_pass_twiddles(L);
        b.upload(tw.data(), std::max<size_t>(1, tw.size()) * sizeof(std::complex<float>));
    };
    if (!n1_)
        upload_tw(tc_tw1_, int(n));
    else
    {
        upload_tw(tc_tw1_, int(n1_));
        upload_tw(tc_tw2_, int(n2_));
        // two-level table for W_N^m, m < N, as for the CUDA-core four-step
        int lb = 0;
        while ((1LL << (2 * lb)) < n)
            lb++;
        lbits_             = lb;
        const long long nb = 1LL << lb, na = (n + nb - 1) / nb;
        std::vector<std::complex<T>> A(na), B(nb);
        for (long long i = 0; i < na; i++)
        {
            const auto w = twiddle(i * nb, n);
            A[i]         = std::complex<T>(T(w.real()), T(w.imag()));
        }
        for (long long j = 0; j < nb; j++)
        {
            const auto w = twiddle(j, n);
            B[j]         = std::complex<T>(T(w.real()), T(w.imag()));
        }
        twA_.upload(A.data(), A.size() * sizeof(std::complex<T>));
        twB_.upload(B.data(), B.size() * sizeof(std::complex<T>));
    }
    tc_mode_ = tensor_mode;
    k_       = kind::tensor;
}

template <typename T>
complex_engine<T>::complex_engine(long long n) : n_(n)
{
    if (n <= 1)
    {
        k_ = kind::trivial;
        return;
    }
    // one-CTA candidates: the direct mixed-radix plan, Rader (prime n) and Bluestein
    long long m = 1;
    while (m < 2 * n - 1)
        m <<= 1;
    const bool direct_ok    = block_program<T>::feasible(n);
    const bool rader_ok     = is_prime(n) && n > 13 && block_program<T>::feasible(n - 1);
    const bool bluestein_ok = block_program<T>::feasible(m);
    const double c_direct   = direct_ok ? fft_cost(n) : 1e30;
    const double c_rader    = rader_ok ? 2.0 * fft_cost(n - 1) + 2.0 * n : 1e30;
    const double c_blue     = bluestein_ok ? 2.0 * fft_cost(m) + 3.0 * n : 1e30;
    if (direct_ok && c_direct <= c_rader && c_direct <= c_blue)
    {
        k_ = kind::smem;
        prog_.build(int(n), CT_C2C);
        plan_pipe();
        return;
    }
    if (rader_ok && c_rader <= c_blue)
    {
        init_rader(n);
        return;
    }
    if (bluestein_ok)
    {
        init_bluestein(n);
        return;
    }
    if (!factor_radices(n).empty() && plan_fourstep(n))
        return;
    init_bluestein(n);
}

template <typename T>
void complex_engine<T>::init_rader(long long n)
{
    const long long L = n - 1;
    // smallest primitive root g of the prime n (the compile-time kernels derive the same one)
    const long long g = primitive_root(n);
    const auto powmod = powmod_ll;
    std::vector<int> pin(n, 0), qof(n, 0);
    std::vector<std::complex<double>> b(L);
    long long gp = 1; // g^p
    for (long long p = 0; p < L; p++)
    {
        pin[gp] = int(p);
        gp      = gp * g % n;
    }
    for (long long k = 1; k < n; k++)
        qof[k] = int((L - pin[k]) % L);
    // b[m] = W_n^{g^-m}; g^-m = g^{(L - m) mod L}
    for (long long mm = 0; mm < L; mm++)
        b[mm] = twiddle(powmod(g, (L - mm) % L, n), n);
    host_dft(b);
    std::vector<std::complex<T>> bh(L);
    for (long long q = 0; q < L; q++)
        bh[q] = std::complex<T>(T(b[q].real() / double(L)), T(b[q].imag() / double(L)));
    std::vector<int> gpow(L);
    for (long long p = 0, v = 1; p < L; p++, v = v * g % n)
        gpow[p] = int(v);
    pin_.upload(pin.data(), pin.size() * sizeof(int));
    qof_.upload(qof.data(), qof.size() * sizeof(int));
    if (sizeof(T) == 4)
    {
        err_.alloc(sizeof(int));
        check(cudaMemset(err_.get(), 0, sizeof(int)), "clear error flag");
    }
    bhat_.upload(bh.data(), bh.size() * sizeof(std::complex<T>));
    prog_.build(int(L), CT_RADER);
    k_ = kind::rader_smem;
    // The prime-factor kernel (rader_pfa.cu) where one is compiled for n: its gather, scatter and
    // kernel-spectrum tables over the row-major array of the coprime axes r_i (L_i = L / r_i): position pos
    // with coordinates c_i holds a[p] for the p with p = c_i (mod r_i) (CRT) on input, A[k] for
    // k = sum c_i L_i (mod L) (Ruritanian) between the two DFTs, and C[p] for the CRT p on output.
    pfa_spc_ = 0;
    std::vector<int> ax;
    int pspc = 0;
    if (sizeof(T) == 4 && rader_pfa_shape(n, ax, pspc))
    {
        const int D = int(ax.size());
        std::vector<long long> stride(D, 1), crt(D);
        for (int i = D - 2; i >= 0; i--)
            stride[i] = stride[i + 1] * ax[i + 1];
        for (int i = 0; i < D; i++)
        {
            // crt[i] = L_i * (L_i^-1 mod r_i): 1 mod r_i, 0 mod the other axes
            const long long Li = L / ax[i];
            long long inv = 1;
            while ((Li % ax[i]) * inv % ax[i] != 1)
                inv++;
            crt[i] = Li * inv % L;
        }
        std::vector<int> tin(L), tout(L);
        std::vector<std::complex<T>> bph(L);
        for (long long pos = 0; pos < L; pos++)
        {
            long long p = 0, k = 0;
            for (int i = 0; i < D; i++)
            {
                const long long c = (pos / stride[i]) % ax[i];
                p                 = (p + c * crt[i]) % L;
                k                 = (k + c * (L / ax[i])) % L;
            }
            tin[pos]  = gpow[p];
            tout[pos] = gpow[(L - p) % L];
            bph[pos]  = bh[k];
        }
        tin_.upload(tin.data(), tin.size() * sizeof(int));
        tout_.upload(tout.data(), tout.size() * sizeof(int));
        bphys_.upload(bph.data(), bph.size() * sizeof(std::complex<T>));
        pfa_spc_  = pspc;
        pfa_axes_ = ax;
    }
}

template <typename T>
void complex_engine<T>::plan_pipe()
{
    pipe_spc_ = 0;
    if (!prog_.ct || sizeof(T) != 4)
        return;
    const int n   = prog_.n;
    const int esz = int(2 * sizeof(T));
    // Signals per tile: the most resident threads per SM (at most 1024: the kernels use up to 64
    // registers), then the smallest tile.  A tile must be a whole number of 16-byte units.
    int best = 0, best_thr = 0;
    for (int spc = 1; spc <= 16; spc++)
    {
        if ((spc * n) % 2)
            continue;
        const int threads = ((spc * prog_.ts + 31) / 32) * 32;
        if (threads > 1024)
            break;
        const int smem = 3 * pipe_stage_len(spc, n, prog_.gstride) * esz + 64;
        if (smem > smem_budget())
            break;
        const int by_smem = (max_smem_bytes() + 1024) / (smem + 1024);
        const int by_thr  = 1024 / threads;
        const int ctas    = std::min(by_smem, by_thr);
        if (ctas < 2)
            continue;
        const int resident = ctas * threads;
        if (resident > best_thr)
        {
            best_thr = resident;
            best     = spc;
        }
    }
    if (!best)
    {
        // one signal per CTA with the signal in registers (lengths whose three tiles do not fit)
        if (n >= 8192 && ((prog_.gstride + 1) / 2 * 2 + n / 2) * esz + 16 <= smem_budget())
        {
            reg_ = true;
            err_.alloc(sizeof(int));
            check(cudaMemset(err_.get(), 0, sizeof(int)), "clear error flag");
        }
        return;
    }
    pipe_spc_ = best;
    err_.alloc(sizeof(int));
    check(cudaMemset(err_.get(), 0, sizeof(int)), "clear error flag");
}

template <typename T>
void complex_engine<T>::check_device_error() const
{
    if (!err_.get())
        return;
    int v = 0;
    check(cudaMemcpy(&v, err_.get(), sizeof(int), cudaMemcpyDeviceToHost), "read error flag");
    if (v)
    {
        cudaMemset(err_.get(), 0, sizeof(int));
        throw cuda_error("a DFT kernel gave up waiting for its input copy (device error flag set)");
    }
}

template <typename T>
void bluestein_tables(long long n, long long m, dbuf& chirp_out, dbuf& bhat_out)
{
    // chirp[k] = e^{-i pi k^2 / n} with the phase k^2 mod 2n kept in integers, as the reference does
    // (src/dft/dft-impl.hpp:217-226)
    std::vector<std::complex<T>> chirp(n);
    std::vector<std::complex<double>> chirp64(n);
    long long ph = 0;
    for (long long k = 0; k < n; k++)
    {
        if (k > 0)
        {
            ph += 2 * k - 1;
            if (ph >= 2 * n)
                ph -= 2 * n;
        }
        chirp64[k] = twiddle(ph, 2 * n);
        chirp[k]   = std::complex<T>(T(chirp64[k].real()), T(chirp64[k].imag()));
    }
    chirp_out.upload(chirp.data(), chirp.size() * sizeof(std::complex<T>));
    // bhat = conj(FFT_M(b)) / M with b[k] = b[M-k] = chirp[k]: evaluated in double on the host (mixed-radix
    // decimation in time over one table of roots) so the table is exact to double rounding before it is
    // stored as T.
    std::vector<std::complex<double>> b(m, { 0.0, 0.0 });
    for (long long k = 0; k < n; k++)
    {
        b[k] = chirp64[k];
        if (k)
            b[m - k] = chirp64[k];
    }
    host_dft_smooth(b);
    std::vector<std::complex<T>> bh(m);
    const double inv_m = 1.0 / double(m);
    for (long long k = 0; k < m; k++)
        bh[k] = std::complex<T>(T(b[k].real() * inv_m), T(-b[k].imag() * inv_m));
    bhat_out.upload(bh.data(), bh.size() * sizeof(std::complex<T>));
}

template void bluestein_tables<float>(long long, long long, dbuf&, dbuf&);
template void bluestein_tables<double>(long long, long long, dbuf&, dbuf&);

template <typename T>
void complex_engine<T>::init_bluestein(long long n)
{
    long long m = 1;
    while (m < 2 * n - 1)
        m <<= 1;
    m_ = m;
    bluestein_tables<T>(n, m, chirp_, bhat_);
    if (block_program<T>::feasible(m))
    {
        k_ = kind::bluestein_smem;
        prog_.build(int(m), CT_BLUESTEIN);
    }
    else
    {
        k_ = kind::bluestein_multi;
        inner_.reset(new complex_engine<T>(m));
    }
}

template <typename T>
int tile_for(const block_program<T>& p, int buffers)
{
    const int per_sig = buffers * (p.gstride ? p.gstride : padded_len_host<T>(p.n)) * int(2 * sizeof(T));
    const int max_thr = p.ct ? (sizeof(T) == 4 ? 1024 : 512) : max_threads_for(int(sizeof(T)), p.ept);
    int s             = 16;
    while (s > 1 && (s * per_sig > smem_budget() || s * p.ts > max_thr))
        s /= 2;
    if (s * per_sig > smem_budget() || s * p.ts > max_thr)
        return 0;
    return s;
}

template <typename T>
bool complex_engine<T>::plan_fourstep(long long n)
{
    long long best_n1 = 0;
    int best_score    = -1;
    double best_bal   = 1e30;
    for (long long n1 = 2; n1 * 2 <= n && n1 <= (1 << 16); n1++)
    {
        if (n % n1)
            continue;
        const long long n2 = n / n1;
        if (n2 > (1 << 16) || n1 * n2 != n)
            continue;
        if (!block_program<T>::feasible(n1) || !block_program<T>::feasible(n2))
            continue;
        block_program<T> a, b;
        a.n = int(n1);
        b.n = int(n2);
        // thread shape without uploading tables
        a.radices = factor_radices(n1);
        b.radices = factor_radices(n2);
        for (auto* p : { &a, &b })
            for (int e : { 16, 32 })
            {
                const int t = threads_needed(p->n, p->radices, e);
                if (t > 0 && t <= max_threads_for(int(sizeof(T)), e))
                {
                    p->ept = e;
                    p->ts  = t;
                    break;
                }
            }
        const int sc = tile_for(a), sr = tile_for(b);
        if (sc == 0 || sr == 0)
            continue;
        const int score   = std::min(std::min(sc, sr), 16);
        const double bal  = std::fabs(std::log(double(n1)) - std::log(double(n2)));
        if (score > best_score || (score == best_score && bal < best_bal))
        {
            best_score = score;
            best_bal   = bal;
            best_n1    = n1;
        }
    }
    if (best_n1 == 0)
        return false;
    k_  = kind::fourstep;
    n1_ = best_n1;
    n2_ = n / best_n1;
    pcols_.build(int(n1_), CT_FOURSTEP);
    prows_.build(int(n2_), CT_FOURSTEP);
    tile_c_ = tile_for(pcols_);
    tile_r_ = tile_for(prows_);
    // compile-time passes run ping-pong (two buffers per signal) unless that would shrink a tile below 8
    // signals (short row segments coalesce poorly)
    pp_c_ = pp_r_ = pair_ = false;
    // tiles of the generic compile-time passes (run ping-pong unless that would shrink a tile below 8)
    if (pcols_.ct)
    {
        const int t2 = tile_for(pcols_, 2);
        if (t2 >= 8 || t2 == tile_c_)
        {
            tile_c_ = t2;
            pp_c_   = true;
        }
    }
    if (prows_.ct)
    {
        const int t2 = tile_for(prows_, 2);
        if (t2 >= 8 || t2 == tile_r_)
        {
            tile_r_ = t2;
            pp_r_   = true;
        }
    }
    // both passes fully compile time (their tiles fixed by the kernels); the generic passes run where the
    // pair kernels cannot (launch_ct_fsp_f32 then answers cudaErrorNotSupported)
    if (sizeof(T) == 4 && pcols_.ct && prows_.ct && has_ct_fsp_f32(int(n1_), int(n2_)))
    {
        pair_ = true;
        err_.alloc(sizeof(int)); // the persistent tensor-copy pair kernels report a copy that never lands
        check(cudaMemset(err_.get(), 0, sizeof(int)), "clear error flag");
    }
    // two-level table for W_N^m, m < N
    int lb = 0;
    while ((1LL << (2 * lb)) < n)
        lb++;
    lbits_             = lb;
    const long long nb = 1LL << lb;
    const long long na = (n + nb - 1) / nb;
    std::vector<std::complex<T>> A(na), B(nb);
    for (long long i = 0; i < na; i++)
    {
        const auto w = twiddle(i * nb, n);
        A[i]         = std::complex<T>(T(w.real()), T(w.imag()));
    }
    for (long long j = 0; j < nb; j++)
    {
        const auto w = twiddle(j, n);
        B[j]         = std::complex<T>(T(w.real()), T(w.imag()));
    }
    twA_.upload(A.data(), A.size() * sizeof(std::complex<T>));
    twB_.upload(B.data(), B.size() * sizeof(std::complex<T>));
    return true;
}

template <typename T>
bool complex_engine<T>::pair_view_of(pair_view& v) const
{
    if (k_ != kind::fourstep || !pair_ || !err_.get())
        return false;
    v.n1      = n1_;
    v.n2      = n2_;
    v.tw_cols = pcols_.tw.get();
    v.tw_rows = prows_.tw.get();
    v.twA     = twA_.get();
    v.twB     = twB_.get();
    v.lbits   = lbits_;
    v.dcols   = pcols_.desc;
    v.drows   = prows_.desc;
    v.err     = static_cast<int*>(err_.get());
    return true;
}

template <typename T>
long long complex_engine<T>::scratch_elems(long long batch) const
{
    switch (k_)
    {
    case kind::fourstep: return batch * n_;
    case kind::tensor: return n1_ ? batch * n_ : 0;
    case kind::bluestein_multi: return batch * m_ + kAlignSlack<T> + inner_->scratch_elems(batch);
    default: return 0;
    }
}

template <typename T>
int complex_engine<T>::launches(long long batch) const
{
    switch (k_)
    {
    case kind::trivial: return 1;
    case kind::smem:
        // the pipelined kernel takes the whole tiles (if any), the per-tile kernel the rest
        if (pipe_spc_)
            return (batch / pipe_spc_ > 0 ? 1 : 0) + (batch % pipe_spc_ ? 1 : 0);
        return 1;
    case kind::bluestein_smem: return 1;
    case kind::fourstep: return 2 * int((batch + 65534) / 65535);
    case kind::bluestein_multi: return 3 + 2 * inner_->launches(batch);
    case kind::rader_smem: return 1;
    case kind::tensor: return n1_ ? 2 * int((batch + 65534) / 65535) : 1;
    }
    return 0;
}

template <typename T>
void complex_engine<T>::execute(void* out, const void* in, long long batch, long long istride, long long ostride,
                                bool inverse, void* scratch, cudaStream_t st) const
{
    if (batch <= 0)
        return;
    const size_t esz = 2 * sizeof(T);
    switch (k_)
    {
    case kind::tensor:
    {
        if (!n1_)
        {
            c2c_args a{};
            a.in      = in;
            a.out     = out;
            a.batch   = batch;
            a.istride = istride;
            a.ostride = ostride;
            a.inverse = inverse;
            a.tw      = tc_tw1_.get();
            check(launch_c2c_tc_f32(a, int(n_), tc_mode_, static_cast<const float*>(tc_cs_.get()), st),
                  "launch tensor-core DFT");
            return;
        }
        if (istride != n_ || ostride != n_ || !scratch)
            throw std::invalid_argument("tensor-core four-step plans need contiguous signals and scratch");
        // batches of at most 65535 signals (the grid's second dimension)
        for (long long b0 = 0; b0 < batch; b0 += 65535)
        {
            const long long nb = std::min<long long>(65535, batch - b0);
            tc_fs_args a{};
            a.batch   = nb;
            a.n1      = int(n1_);
            a.n2      = int(n2_);
            a.inverse = inverse;
            a.tw1     = tc_tw1_.get();
            a.tw2     = tc_tw2_.get();
            a.twA     = twA_.get();
            a.twB     = twB_.get();
            a.lbits   = lbits_;
            a.cs      = static_cast<const float*>(tc_cs_.get());
            a.in      = static_cast<const char*>(in) + b0 * n_ * esz;
            a.out     = scratch;
            check(launch_tc_fourstep_pass_f32(a, true, tc_mode_, st), "launch tensor-core column pass");
            a.in  = scratch;
            a.out = static_cast<char*>(out) + b0 * n_ * esz;
            check(launch_tc_fourstep_pass_f32(a, false, tc_mode_, st), "launch tensor-core row pass");
        }
        return;
    }
    case kind::trivial:
    {
        if (n_ == 1 && out != in)
        {
            if (istride == 1 && ostride == 1)
                check(cudaMemcpyAsync(out, in, batch * esz, cudaMemcpyDeviceToDevice, st), "copy");
            else
                check(cudaMemcpy2DAsync(out, ostride * esz, in, istride * esz, esz, batch,
                                        cudaMemcpyDeviceToDevice, st),
                      "copy");
        }
        return;
    }
    case kind::smem:
    {
        c2c_args a;
        a.in      = in;
        a.out     = out;
        a.batch   = batch;
        a.istride = istride;
        a.ostride = ostride;
        a.inverse = inverse;
        a.tw      = prog_.tw.get();
        a.div_n   = make_fast_div(uint32_t(n_));
        a.d       = prog_.desc;
        long long done = 0;
        if (reg_ && !host_io_ && istride == n_ && ostride == n_ && (reinterpret_cast<uintptr_t>(in) % 16) == 0)
        {
            block_cfg rc = prog_.cfg_tile(1);
            rc.smem      = ((prog_.gstride + 1) / 2 * 2 + int(n_ / 2)) * int(esz) + 16;
            check(launch_ct_c2c_reg_f32(a, rc, batch, static_cast<int*>(err_.get()), st), "launch c2c (one per CTA)");
            done = batch;
        }
        if (pipe_spc_ && !host_io_ && istride == n_ && ostride == n_ && (reinterpret_cast<uintptr_t>(in) % 16) == 0)
        {
            const long long ntiles = batch / pipe_spc_;
            if (ntiles > 0)
            {
                block_cfg pc = prog_.cfg_tile(pipe_spc_);
                pc.smem = 3 * pipe_stage_len(pipe_spc_, int(n_), prog_.gstride) * int(esz) + 64;
                check(launch_ct_c2c_pipe_f32(a, pc, ntiles, static_cast<int*>(err_.get()), st), "launch c2c (pipelined)");
                done = ntiles * pipe_spc_;
            }
        }
        if (done < batch)
        {
            a.in    = static_cast<const char*>(in) + done * n_ * esz;
            a.out   = static_cast<char*>(out) + done * n_ * esz;
            a.batch = batch - done;
            check(launch_c2c<T>(a, prog_.cfg(batch - done), st), "launch c2c");
        }
        return;
    }
    case kind::bluestein_smem:
    {
        bluestein_args a;
        a.in      = in;
        a.out     = out;
        a.batch   = batch;
        a.istride = istride;
        a.ostride = ostride;
        a.n       = int(n_);
        a.inverse = inverse;
        a.chirp   = chirp_.get();
        a.bhat    = bhat_.get();
        a.tw      = prog_.tw.get();
        a.div_n   = make_fast_div(uint32_t(n_));
        a.div_m   = make_fast_div(uint32_t(m_));
        a.d       = prog_.desc;
        check(launch_bluestein<T>(a, prog_.cfg(batch), st), "launch bluestein");
        return;
    }
    case kind::rader_smem:
    {
        if (pfa_spc_ && !host_io_ && err_.get() && istride == n_ && ostride == n_ && (reinterpret_cast<uintptr_t>(in) % 16) == 0 &&
            (reinterpret_cast<uintptr_t>(out) % 16) == 0)
        {
            // the prime-factor kernel takes every signal (its last tile may be shorter)
            rader_pfa_args p;
            p.in      = in;
            p.out     = out;
            p.batch   = batch;
            p.inverse = inverse;
            p.tin     = static_cast<const int*>(tin_.get());
            p.tout    = static_cast<const int*>(tout_.get());
            p.bphys   = bphys_.get();
            p.err     = static_cast<int*>(err_.get());
            check(launch_rader_pfa_f32(p, n_, st), "launch rader (prime factor)");
            return;
        }
        rader_args a;
        a.in      = in;
        a.out     = out;
        a.batch   = batch;
        a.istride = istride;
        a.ostride = ostride;
        a.n       = int(n_);
        a.inverse = inverse;
        a.pin     = static_cast<const int*>(pin_.get());
        a.qof     = static_cast<const int*>(qof_.get());
        a.bhat    = bhat_.get();
        a.tw      = prog_.tw.get();
        a.div_n   = make_fast_div(uint32_t(n_));
        a.div_l   = make_fast_div(uint32_t(n_ - 1));
        a.d       = prog_.desc;
        // the per-tile kernel where the prime-factor kernel cannot run (misaligned or strided signals, c64)
        block_cfg c = prog_.cfg(batch);
        c.smem += 2 * c.spc * int(esz);
        check(launch_rader<T>(a, c, st), "launch rader");
        return;
    }
    case kind::fourstep:
    {
        if (istride != n_ || ostride != n_)
            throw std::invalid_argument("internal: four-step needs contiguous signals");
        // a pair kernel for this pass, or false when neither of them can run (the generic pass runs instead)
        const auto run_pair = [&](const fourstep_args& fa, bool cols)
        {
            const cudaError_t e = launch_ct_fsp_f32(fa, cols, st);
            if (e == cudaErrorNotSupported)
                return false;
            check(e, cols ? "launch four-step columns" : "launch four-step rows");
            return true;
        };
        for (long long b0 = 0; b0 < batch; b0 += 65535)
        {
            const long long nb  = std::min<long long>(65535, batch - b0);
            const char* inb     = static_cast<const char*>(in) + b0 * n_ * esz;
            char* outb          = static_cast<char*>(out) + b0 * n_ * esz;
            char* scr           = static_cast<char*>(scratch) + b0 * n_ * esz;
            fourstep_args a;
            // the tensor-copy pair kernels run only with an error flag: host-mapped buffers take the plain-load
            // pair kernels
            a.err        = pair_ && !host_io_ ? static_cast<int*>(err_.get()) : nullptr;
            a.batch      = nb;
            a.sig_stride = n_;
            a.n1         = int(n1_);
            a.n2         = int(n2_);
            a.same_layout = 0;
            a.twA        = twA_.get();
            a.twB        = twB_.get();
            a.lbits      = lbits_;
            // column pass: x -> scratch
            a.in       = inb;
            a.out      = scr;
            a.tile       = tile_c_;
            a.tile_shift = ilog2(tile_c_);
            a.conj_in    = inverse;
            a.conj_out = 0;
            a.tw       = pcols_.tw.get();
            a.d        = pcols_.desc;
            a.div_n    = make_fast_div(uint32_t(n1_));
            a.pingpong   = pp_c_;
            if (!pair_ || !run_pair(a, true))
            {
                block_cfg cc = pcols_.cfg_tile(tile_c_);
                if (pp_c_)
                    cc.smem *= 2; // ping-pong buffers
                cc.grid = (n2_ + tile_c_ - 1) / tile_c_;
                check(launch_fs_cols<T>(a, cc, st), "launch four-step columns");
            }
            // row pass: scratch -> out
            a.in       = scr;
            a.out      = outb;
            a.tile       = tile_r_;
            a.tile_shift = ilog2(tile_r_);
            a.conj_in    = 0;
            a.conj_out = inverse;
            a.tw       = prows_.tw.get();
            a.d        = prows_.desc;
            a.div_n    = make_fast_div(uint32_t(n2_));
            a.pingpong   = pp_r_;
            if (!pair_ || !run_pair(a, false))
            {
                block_cfg cr = prows_.cfg_tile(tile_r_);
                if (pp_r_)
                    cr.smem *= 2;
                cr.grid = (n1_ + tile_r_ - 1) / tile_r_;
                check(launch_fs_rows<T>(a, cr, st), "launch four-step rows");
            }
        }
        return;
    }
    case kind::bluestein_multi:
    {
        if (istride != n_ || ostride != n_)
            throw std::invalid_argument("internal: Bluestein needs contiguous signals");
        char* A     = static_cast<char*>(scratch);
        char* inner = align_scratch(A + batch * m_ * esz);
        ew_args e;
        e.batch   = batch;
        e.t1      = nullptr;
        e.flag    = inverse;
        // A = x * chirp, zero padded to M
        e.in      = in;
        e.out     = A;
        e.n       = m_;
        e.istride = n_;
        e.ostride = m_;
        e.t0      = chirp_.get();
        e.n_src   = n_;
        check(launch_elementwise<T>(EW_BS_PRE, e, st), "launch bluestein pre");
        inner_->execute(A, A, batch, m_, m_, false, inner, st);
        e.in      = A;
        e.out     = A;
        e.istride = m_;
        e.t0      = bhat_.get();
        check(launch_elementwise<T>(EW_BS_MID, e, st), "launch bluestein mid");
        inner_->execute(A, A, batch, m_, m_, false, inner, st);
        e.in      = A;
        e.out     = out;
        e.n       = n_;
        e.istride = m_;
        e.ostride = n_;
        e.t0      = chirp_.get();
        check(launch_elementwise<T>(EW_BS_POST, e, st), "launch bluestein post");
        return;
    }
    }
}

template <typename T>
std::string complex_engine<T>::describe() const
{
    std::ostringstream s;
    switch (k_)
    {
    case kind::trivial: s << "trivial n=" << n_; break;
    case kind::tensor:
        s << "tensor-core n=" << n_;
        if (n1_)
            s << " = " << n1_ << " x " << n2_ << " four-step";
        s << ", radix-16 passes as mma.sync contractions, "
          << (tc_mode_ == TC_BF16 ? "BF16 hi+mid+lo" : "FP16 hi+lo per-butterfly scaled")
          << " operands, FP32 accumulation";
        break;
    case kind::smem:
        s << "smem " << prog_.describe();
        if (pipe_spc_)
            s << " pipelined spc=" << pipe_spc_;
        if (reg_)
            s << " persistent one per CTA";
        break;
    case kind::bluestein_smem: s << "bluestein_smem n=" << n_ << " m=" << m_ << " [" << prog_.describe() << "]"; break;
    case kind::fourstep:
        s << "fourstep" << (pair_ ? " (compile-time pair)" : "") << " n=" << n_ << " = " << n1_ << " x " << n2_
          << " cols[" << pcols_.describe() << " tile=" << tile_c_ << "] rows[" << prows_.describe()
          << " tile=" << tile_r_ << "]";
        break;
    case kind::bluestein_multi: s << "bluestein_multi n=" << n_ << " m=" << m_ << " inner{" << inner_->describe() << "}"; break;
    case kind::rader_smem:
        if (pfa_spc_)
        {
            s << "rader n=" << n_ << " prime-factor axes=";
            for (size_t i = 0; i < pfa_axes_.size(); i++)
                s << (i ? "x" : "") << pfa_axes_[i];
            s << " in place, spc=" << pfa_spc_;
            break;
        }
        s << "rader n=" << n_ << " [" << prog_.describe() << "]";
        break;
    }
    return s.str();
}

// ------------------------------------------------------------------------------------------------------
// real_engine
// ------------------------------------------------------------------------------------------------------

template <typename T>
void real_engine<T>::check_device_error() const
{
    ceng_.check_device_error();
    if (!err_.get())
        return;
    int v = 0;
    check(cudaMemcpy(&v, err_.get(), sizeof(int), cudaMemcpyDeviceToHost), "read error flag");
    if (v)
    {
        cudaMemset(err_.get(), 0, sizeof(int));
        throw cuda_error("a real DFT kernel gave up waiting for its input copy (device error flag set)");
    }
}

template <typename T>
real_engine<T>::real_engine(long long n) : n_(n), c_(n / 2), ceng_(n / 2)
{
    if (n <= 0 || n % 2)
        throw std::invalid_argument("dft_plan_real requires size to be even");
    // W_n^k for k = 0..c
    std::vector<std::complex<T>> r(c_ + 1);
    for (long long k = 0; k <= c_; k++)
    {
        const auto w = twiddle(k, n);
        r[k]         = std::complex<T>(T(w.real()), T(w.imag()));
    }
    rtw_.upload(r.data(), r.size() * sizeof(std::complex<T>));
    fused_ = ceng_.strategy() == complex_engine<T>::kind::smem;
    if (fused_)
        prog_.build(int(c_), CT_REAL);
    typename complex_engine<T>::pair_view pv;
    rfsp_ = sizeof(T) == 4 && !fused_ && ceng_.pair_view_of(pv) && has_ct_fsp_r2c_f32(int(pv.n1), int(pv.n2));
    if (rfsp_)
    {
        std::vector<std::complex<T>> r2(pv.n1 + pv.n2);
        for (long long k1 = 0; k1 < pv.n1; k1++)
        {
            const auto w = twiddle(k1, n);
            r2[k1]       = std::complex<T>(T(w.real()), T(w.imag()));
        }
        for (long long k2 = 0; k2 < pv.n2; k2++)
        {
            const auto w     = twiddle(pv.n1 * k2, n);
            r2[pv.n1 + k2] = std::complex<T>(T(w.real()), T(w.imag()));
        }
        rtw2_.upload(r2.data(), r2.size() * sizeof(std::complex<T>));
    }
    // Pipelined forward and inverse kernels (compile-time c, single precision): an even number of signals
    // per tile, the most resident threads per SM with at least two CTAs, then the smallest tile.
    if (fused_ && prog_.ct && sizeof(T) == 4)
    {
        int best = 0, best_thr = 0;
        for (int spc = 2; spc <= 32; spc += 2)
        {
            const int threads = ((spc * prog_.ts + 31) / 32) * 32;
            if (threads > 1024)
                break;
            const int slen = (std::max(spc * int(c_ + 1), spc * prog_.gstride) + 15) / 16 * 16;
            const int smem = 3 * slen * int(2 * sizeof(T)) + 64;
            if (smem > smem_budget())
                break;
            const int ctas = std::min((max_smem_bytes() + 1024) / (smem + 1024), 1024 / threads);
            if (ctas >= 2 && ctas * threads > best_thr)
            {
                best_thr = ctas * threads;
                best     = spc;
            }
        }
        if (best)
        {
            pipe_spc_ = best;
            err_.alloc(sizeof(int));
            check(cudaMemset(err_.get(), 0, sizeof(int)), "clear error flag");
        }
    }
}

template <typename T>
long long real_engine<T>::scratch_elems(long long batch) const
{
    if (fused_)
        return 0;
    return batch * (c_ + 1) + kAlignSlack<T> + ceng_.scratch_elems(batch);
}

template <typename T>
int real_engine<T>::launches(long long batch) const
{
    if (rfsp_)
        return 2 * int((batch + 65534) / 65535); // forward (the inverse merges separately)
    return fused_ ? ((pipe_spc_ && batch % pipe_spc_) ? 2 : 1) : 1 + ceng_.launches(batch);
}

template <typename T>
void real_engine<T>::forward(void* out, const void* in, long long batch, bool ccs, void* scratch,
                             cudaStream_t st) const
{
    if (batch <= 0)
        return;
    const long long olen = ccs ? c_ + 1 : c_;
    if (c_ == 1)
    {
        // n = 2: X0 = x0 + x1, X1 = x0 - x1 (the split of a one-point DFT)
        ew_args e;
        e.in      = in;
        e.out     = out;
        e.batch   = batch;
        e.n       = olen;
        e.istride = 1;
        e.ostride = olen;
        e.t0      = rtw_.get();
        e.t1      = nullptr;
        e.n_src   = 1;
        e.flag    = ccs;
        check(launch_real_pairs<T>(e, false, st), "launch r2c split");
        return;
    }
    if (fused_)
    {
        const block_program<T>& p = prog_;
        real_args a;
        a.in      = in;
        a.out     = out;
        a.batch   = batch;
        a.istride = n_;
        a.ostride = olen;
        a.ccs     = ccs;
        a.rtw     = rtw_.get();
        a.tw      = p.tw.get();
        a.div_n   = make_fast_div(uint32_t(c_));
        a.div_out = make_fast_div(uint32_t(olen));
        a.d       = p.desc;
        long long done = 0;
        if (pipe_spc_ && (reinterpret_cast<uintptr_t>(in) % 16) == 0 && (reinterpret_cast<uintptr_t>(out) % 16) == 0)
        {
            const long long ntiles = batch / pipe_spc_;
            if (ntiles > 0)
            {
                block_cfg pc = p.cfg_tile(pipe_spc_);
                pc.smem = 3 * ((std::max(pipe_spc_ * int(c_ + 1), pipe_spc_ * p.gstride) + 15) / 16 * 16) *
                              int(2 * sizeof(T)) + 64;
                check(launch_ct_r2c_pipe_f32(a, pc, ntiles, static_cast<int*>(err_.get()), st), "launch r2c (pipelined)");
                done = ntiles * pipe_spc_;
            }
        }
        if (done < batch)
        {
            a.in    = static_cast<const T*>(in) + done * n_;
            a.out   = static_cast<std::complex<T>*>(out) + done * olen;
            a.batch = batch - done;
            check(launch_r2c<T>(a, p.cfg(batch - done), st), "launch r2c");
        }
        return;
    }
    typename complex_engine<T>::pair_view pv;
    if (rfsp_ && (reinterpret_cast<uintptr_t>(in) % 16) == 0 && ceng_.pair_view_of(pv))
    {
        // column pass into the real-fused layout (scratch), row pass with the split into out
        char* y = align_scratch(static_cast<char*>(scratch));
        for (long long b0 = 0; b0 < batch; b0 += 65535)
        {
            const long long nb = std::min<long long>(65535, batch - b0);
            fourstep_args a{};
            a.err         = pv.err;
            a.batch       = nb;
            a.sig_stride  = c_;
            a.n1          = int(pv.n1);
            a.n2          = int(pv.n2);
            a.twA         = pv.twA;
            a.twB         = pv.twB;
            a.lbits       = pv.lbits;
            a.rtw         = rtw2_.get();
            a.ccs         = ccs;
            a.in          = static_cast<const T*>(in) + b0 * n_;
            a.out         = y;
            a.tw          = pv.tw_cols;
            a.d           = pv.dcols;
            a.div_n       = make_fast_div(uint32_t(pv.n1));
            check(launch_ct_fsp_r2c_f32(a, true, st), "launch r2c four-step columns");
            a.in    = y;
            a.out   = static_cast<std::complex<T>*>(out) + b0 * olen;
            a.tw    = pv.tw_rows;
            a.d     = pv.drows;
            a.div_n = make_fast_div(uint32_t(pv.n2));
            check(launch_ct_fsp_r2c_f32(a, false, st), "launch r2c four-step rows with the split");
        }
        return;
    }
    char* Z     = static_cast<char*>(scratch);
    char* inner = align_scratch(Z + batch * (c_ + 1) * 2 * sizeof(T));
    if (reinterpret_cast<uintptr_t>(in) % (2 * sizeof(T)))
    {
        // the complex kernels read the reals in pairs: stage an input that is not aligned to a pair into
        // Z (which the transform then overwrites in place)
        check(cudaMemcpyAsync(Z, in, size_t(batch * n_) * sizeof(T), cudaMemcpyDeviceToDevice, st), "align input");
        in = Z;
    }
    ceng_.execute(Z, in, batch, c_, c_, false, inner, st);
    ew_args e;
    e.in      = Z;
    e.out     = out;
    e.batch   = batch;
    e.n       = olen;
    e.istride = c_;
    e.ostride = olen;
    e.t0      = rtw_.get();
    e.t1      = nullptr;
    e.n_src   = c_;
    e.flag    = ccs;
    check(launch_real_pairs<T>(e, false, st), "launch r2c split");
}

template <typename T>
void real_engine<T>::inverse(void* out, const void* in, long long batch, bool ccs, void* scratch,
                             cudaStream_t st) const
{
    if (batch <= 0)
        return;
    const long long ilen = ccs ? c_ + 1 : c_;
    if (fused_)
    {
        const block_program<T>& p = prog_;
        real_args a;
        a.in      = in;
        a.out     = out;
        a.batch   = batch;
        a.istride = ilen;
        a.ostride = n_;
        a.ccs     = ccs;
        a.rtw     = rtw_.get();
        a.tw      = p.tw.get();
        a.div_n   = make_fast_div(uint32_t(c_));
        a.div_out = make_fast_div(uint32_t(c_));
        a.d       = p.desc;
        long long done = 0;
        if (pipe_spc_ && (reinterpret_cast<uintptr_t>(in) % 16) == 0 && (reinterpret_cast<uintptr_t>(out) % 16) == 0)
        {
            const long long ntiles = batch / pipe_spc_;
            if (ntiles > 0)
            {
                block_cfg pc = p.cfg_tile(pipe_spc_);
                pc.smem = 3 * ((std::max(pipe_spc_ * int(c_ + 1), pipe_spc_ * p.gstride) + 15) / 16 * 16) *
                              int(2 * sizeof(T)) + 64;
                check(launch_ct_c2r_pipe_f32(a, pc, ntiles, static_cast<int*>(err_.get()), st), "launch c2r (pipelined)");
                done = ntiles * pipe_spc_;
            }
        }
        if (done < batch)
        {
            a.in    = static_cast<const std::complex<T>*>(in) + done * ilen;
            a.out   = static_cast<T*>(out) + done * n_;
            a.batch = batch - done;
            check(launch_c2r<T>(a, p.cfg(batch - done), st), "launch c2r");
        }
        return;
    }
    char* Z     = static_cast<char*>(scratch);
    char* inner = align_scratch(Z + batch * (c_ + 1) * 2 * sizeof(T));
    ew_args e;
    e.in      = in;
    e.out     = Z;
    e.batch   = batch;
    e.n       = c_;
    e.istride = ilen;
    e.ostride = c_;
    e.t0      = rtw_.get();
    e.t1      = nullptr;
    e.n_src   = c_;
    e.flag    = ccs;
    check(launch_real_pairs<T>(e, true, st), "launch c2r merge");
    if (reinterpret_cast<uintptr_t>(out) % (2 * sizeof(T)))
    {
        // the complex kernels write the reals in pairs: transform in place in Z, then copy out
        ceng_.execute(Z, Z, batch, c_, c_, true, inner, st);
        check(cudaMemcpyAsync(out, Z, size_t(batch * n_) * sizeof(T), cudaMemcpyDeviceToDevice, st), "copy output");
        return;
    }
    ceng_.execute(out, Z, batch, c_, c_, true, inner, st);
}

template <typename T>
std::string real_engine<T>::describe() const
{
    std::ostringstream s;
    s << "real n=" << n_
      << (fused_ ? " fused split/merge" : rfsp_ ? " split fused into the four-step row pass" : " separate split/merge");
    if (pipe_spc_)
        s << " pipelined spc=" << pipe_spc_;
    s << " complex{" << ceng_.describe() << "}";
    return s.str();
}

// ------------------------------------------------------------------------------------------------------
// dct_engine
// ------------------------------------------------------------------------------------------------------

template <typename T>
dct_engine<T>::dct_engine(long long n) : n_(n), ceng_(n)
{
    if (n <= 0)
        throw std::invalid_argument("dct_plan requires a positive size");
    std::vector<std::complex<T>> d(n);
    for (long long k = 0; k < n; k++)
    {
        // (cos, sin) of pi k / (2n) = -twiddle(k, 4n)
        const auto w = twiddle(k, 4 * n);
        d[k]         = std::complex<T>(T(w.real()), T(-w.imag()));
    }
    dtw_.upload(d.data(), d.size() * sizeof(std::complex<T>));
    fused_ = ceng_.strategy() == complex_engine<T>::kind::smem;
    if (fused_)
        prog_.build(int(n), CT_DCT);
    // Pipelined kernels (compile-time n, single precision): the most resident threads per SM with at least
    // two CTAs, then the smallest tile.
    if (fused_ && prog_.ct && sizeof(T) == 4 && n % 4 == 0)
    {
        int best = 0, best_thr = 0;
        for (int spc = 1; spc <= 32; spc++)
        {
            const int threads = ((spc * prog_.ts + 31) / 32) * 32;
            if (threads > 1024)
                break;
            const int slen = (std::max(spc * int(n) / 2, spc * prog_.gstride) + 15) / 16 * 16;
            const int smem = 3 * slen * int(2 * sizeof(T)) + 64;
            if (smem > smem_budget())
                break;
            const int ctas = std::min((max_smem_bytes() + 1024) / (smem + 1024), 1024 / threads);
            if (ctas >= 2 && ctas * threads > best_thr)
            {
                best_thr = ctas * threads;
                best     = spc;
            }
        }
        if (best)
        {
            pipe_spc_ = best;
            err_.alloc(sizeof(int));
            check(cudaMemset(err_.get(), 0, sizeof(int)), "clear error flag");
        }
    }
}

template <typename T>
void dct_engine<T>::check_device_error() const
{
    ceng_.check_device_error();
    if (!err_.get())
        return;
    int v = 0;
    check(cudaMemcpy(&v, err_.get(), sizeof(int), cudaMemcpyDeviceToHost), "read error flag");
    if (v)
    {
        cudaMemset(err_.get(), 0, sizeof(int));
        throw cuda_error("a DCT kernel gave up waiting for its input copy (device error flag set)");
    }
}

template <typename T>
long long dct_engine<T>::scratch_elems(long long batch) const
{
    if (fused_)
        return 0;
    return batch * n_ + kAlignSlack<T> + ceng_.scratch_elems(batch);
}

template <typename T>
int dct_engine<T>::launches(long long batch) const
{
    if (fused_ && pipe_spc_)
        return (batch / pipe_spc_ > 0 ? 1 : 0) + (batch % pipe_spc_ ? 1 : 0);
    return fused_ ? 1 : 2 + ceng_.launches(batch);
}

template <typename T>
void dct_engine<T>::execute(void* out, const void* in, long long batch, bool inverse, void* scratch,
                            cudaStream_t st) const
{
    if (batch <= 0)
        return;
    if (fused_)
    {
        const block_program<T>& p = prog_;
        dct_args a;
        a.in     = in;
        a.out    = out;
        a.batch  = batch;
        a.stride = n_;
        a.dtw    = dtw_.get();
        a.tw     = p.tw.get();
        a.div_n  = make_fast_div(uint32_t(n_));
        a.d      = p.desc;
        long long done = 0;
        if (pipe_spc_ && (reinterpret_cast<uintptr_t>(in) % 16) == 0 && (reinterpret_cast<uintptr_t>(out) % 16) == 0)
        {
            const long long ntiles = batch / pipe_spc_;
            if (ntiles > 0)
            {
                block_cfg pc = p.cfg_tile(pipe_spc_);
                pc.smem = 3 * ((std::max(pipe_spc_ * int(n_) / 2, pipe_spc_ * p.gstride) + 15) / 16 * 16) *
                              int(2 * sizeof(T)) + 64;
                check(launch_ct_dct_pipe_f32(a, pc, ntiles, static_cast<int*>(err_.get()), inverse, st),
                      "launch dct (pipelined)");
                done = ntiles * pipe_spc_;
            }
        }
        if (done < batch)
        {
            a.in    = static_cast<const T*>(in) + done * n_;
            a.out   = static_cast<T*>(out) + done * n_;
            a.batch = batch - done;
            check(inverse ? launch_dct3<T>(a, p.cfg(batch - done), st) : launch_dct2<T>(a, p.cfg(batch - done), st),
                  "launch dct");
        }
        return;
    }
    char* V     = static_cast<char*>(scratch);
    char* inner = align_scratch(V + batch * n_ * 2 * sizeof(T));
    ew_args e;
    e.batch = batch;
    e.n     = n_;
    e.t0    = dtw_.get();
    e.t1    = nullptr;
    e.n_src = n_;
    e.flag  = 0;
    e.in      = in;
    e.out     = V;
    e.istride = n_;
    e.ostride = n_;
    check(launch_elementwise<T>(inverse ? EW_DCT3_PRE : EW_DCT2_PRE, e, st), "launch dct pre");
    ceng_.execute(V, V, batch, n_, n_, false, inner, st);
    e.in  = V;
    e.out = out;
    check(launch_elementwise<T>(inverse ? EW_DCT3_POST : EW_DCT2_POST, e, st), "launch dct post");
}

template <typename T>
std::string dct_engine<T>::describe() const
{
    std::ostringstream s;
    s << "dct n=" << n_ << (fused_ ? " fused" : " separate pre/post");
    if (pipe_spc_)
        s << " pipelined spc=" << pipe_spc_;
    s << " complex{" << ceng_.describe() << "}";
    return s.str();
}

template int tile_for<float>(const block_program<float>&, int);
template int tile_for<double>(const block_program<double>&, int);
template struct block_program<float>;
template struct block_program<double>;
template class complex_engine<float>;
template class complex_engine<double>;
template class real_engine<float>;
template class real_engine<double>;
template class dct_engine<float>;
template class dct_engine<double>;

} // namespace kfr_gpu
