// Host-side planner and executors of the GB300 DFT engine.
//
// A plan for length N picks one of five strategies (the GPU counterpart of the reference's stage lists,
// include/kfr/dft/fft.hpp:372-381, built by init_fft / init_dft, src/dft/fft-impl.hpp:1903-1918 and
// src/dft/dft-impl.hpp:512-583):
//   trivial          N <= 1
//   smem             one CTA per signal (or several signals per CTA): load, all passes in shared memory,
//                    store.  N up to 16384 (c32) / 8192 (c64).
//   bluestein_smem   a prime factor above kGenericMax and M = next_pow2(2N-1) fits one CTA: the whole
//                    chirp-z transform in one kernel.
//   fourstep         N = n1 * n2, both one-CTA lengths: a column pass (FFT_n1, twiddle, transpose-store)
//                    and a row pass (FFT_n2, transpose-store), each one HBM round trip.
//   rader_smem       a prime N whose cyclic convolution length N - 1 fits one CTA: Rader's permutation
//                    into an (N-1)-point convolution, computed in one kernel (half the work of Bluestein).
//   bluestein_multi  anything else: chirp pre-multiply, M-point engine, spectral product, M-point engine,
//                    chirp post-multiply.
#pragma once

#include <complex>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "launch.hpp"

namespace kfr_gpu
{

constexpr int kGenericMax = 127; // largest prime handled by a generic radix pass (above: Bluestein)

struct cuda_error : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

void check(cudaError_t e, const char* what);

// Owning device allocation.
class dbuf
{
public:
    dbuf() = default;
    dbuf(const dbuf&)            = delete;
    dbuf& operator=(const dbuf&) = delete;
    ~dbuf() { release(); }
    void alloc(size_t bytes);
    void ensure(size_t bytes); // grows (never shrinks) the allocation
    void release();
    void upload(const void* host, size_t bytes);
    void* get() const { return p_; }
    size_t size() const { return bytes_; }

private:
    void* p_      = nullptr;
    size_t bytes_ = 0;
};

// e^{-2 pi i k / n} in double, with the exact quadrant folding of the reference's calculate_twiddle
// (src/dft/ft.hpp:1803-1827).
std::complex<double> twiddle(long long k, long long n);

// In-place forward DFT of a power-of-two length in double precision (host; used for precomputed spectra).
void host_fft_pow2(std::vector<std::complex<double>>& a);
// Forward DFT of any length in double precision (host; recursive mixed radix, O(N * sum of prime factors)).
void host_dft(std::vector<std::complex<double>>& a);
// The same for lengths with small prime factors, over one table of roots (fast for long smooth lengths).
void host_dft_smooth(std::vector<std::complex<double>>& a);

// Radix sequence for a one-CTA length; empty if a prime factor exceeds kGenericMax.
std::vector<int> factor_radices(long long n);

// Kernel kinds with compile-time specialised lengths (ct_table.hpp).
enum ct_kind
{
    CT_NONE = -1,
    CT_C2C,
    CT_BLUESTEIN,
    CT_RADER,
    CT_FOURSTEP,
    CT_REAL,
    CT_DCT,
    CT_CONV
};

// True (with the thread count and radix order) if `kind` has a compile-time kernel of length n for T.
template <typename T>
bool ct_lookup(int kind, int n, int& ts, std::vector<int>& radices);

// Descriptor, twiddles and thread shape of a one-CTA FFT of length n.
template <typename T>
struct block_program
{
    int n   = 0;
    int ept = 16;
    int ts  = 1;
    int ct  = 0; // nonzero: the compile-time kernel of this length is used
    int gstride = 0; // elements between the shared-memory slots of consecutive signals
    fft_desc desc{};
    std::vector<int> radices;
    dbuf tw;

    // False if n cannot run in one CTA (size, registers or a large prime factor).
    static bool feasible(long long n);
    // `kind` selects the compile-time kernel list to look in (CT_NONE: always the runtime kernel).  `order`
    // forces a runtime radix sequence (product n) and `ept_only` (16 or 32) the register array size.
    void build(int n, int kind = CT_NONE, const std::vector<int>* order = nullptr, int ept_only = 0);
    // Launch shape for `batch` signals (`spc_cap` bounds the signals per CTA, 0 = no bound).
    block_cfg cfg(long long batch, int spc_cap = 0) const;
    // Launch shape of a four-step tile: exactly `tile` signals per CTA.
    block_cfg cfg_tile(int tile) const;
    std::string describe() const;
};

// Threads per signal a runtime radix sequence needs at `ept` complex values per thread (0 = infeasible).
int threads_needed(long long n, const std::vector<int>& radices, int ept);
// twiddle table of a radix order (ns * (R - 1) values W_{ns R}^{k r} per pass with ns > 1, then R roots for a
// radix without a codelet); fills the passes' offsets when passes is not null
template <typename T>
std::vector<std::complex<T>> pass_twiddles(const std::vector<int>& radices, pass_desc* passes);
// Bluestein tables for length n and convolution length m: chirp[k] = e^{-i pi k^2 / n} (n values) and
// bhat = conj(DFT_m(b)) / m of the symmetric chirp sequence b (m values).
template <typename T>
void bluestein_tables(long long n, long long m, dbuf& chirp, dbuf& bhat);

// Dynamic shared memory a block FFT kernel may use (device limit less the static pass list and a reserve).
int smem_budget();
// Largest power-of-two number of signals (<= 16) of `p` that fit one CTA with `buffers` shared-memory
// buffers per signal: the column / row tile of the strided passes.  0 if not even one fits.
template <typename T>
int tile_for(const block_program<T>& p, int buffers = 1);

template <typename T>
class complex_engine
{
public:
    enum class kind
    {
        trivial,
        smem,
        bluestein_smem,
        fourstep,
        bluestein_multi,
        rader_smem,
        tensor
    };

    explicit complex_engine(long long n);
    // Tensor-core form (single precision, n = 256, 4096, 2^16, 2^20 or 2^24): every radix-16 pass as a
    // contraction on the tensor cores with operands split into 16-bit parts (mode: TC_BF16 or TC_FP16,
    // tensor.hpp); lengths above 4096 run as a four-step of 256- and 4096-point passes.
    complex_engine(long long n, int tensor_mode);

    // Device scratch (in complex elements) that execute() needs for `batch` signals.
    long long scratch_elems(long long batch) const;
    // out/in: `batch` signals, istride/ostride complex elements apart (fourstep and bluestein_multi
    // require istride == ostride == n).  out may alias in.  scratch: scratch_elems(batch) elements.
    void execute(void* out, const void* in, long long batch, long long istride, long long ostride, bool inverse,
                 void* scratch, cudaStream_t st) const;
    std::string describe() const;
    kind strategy() const { return k_; }
    // The one-CTA program (smem: length n; bluestein_smem: length m).
    const block_program<T>& program() const { return prog_; }
    long long size() const { return n_; }
    // Kernel launches one execute() issues (for the launch count reported by the benchmark).
    int launches(long long batch) const;
    // Throws if a kernel of this engine recorded a device-side error (a bounded wait that ran out).
    void check_device_error() const;
    // The compile-time pair four-step's split and tables (false unless this engine runs one), for the real
    // engine's kernels that run the two passes with the real split fused in.
    struct pair_view
    {
        long long n1, n2;
        const void* tw_cols;
        const void* tw_rows;
        const void* twA;
        const void* twB;
        int lbits;
        fft_desc dcols, drows;
        int* err;
    };
    bool pair_view_of(pair_view& v) const;
    // While set, in and out of execute() are host memory mapped into the device's address space (zero-copy
    // calls): the kernels that read or write through bulk and tensor copies give way to the plain-load ones.
    // The caller holds the plan's lock around the call.
    void set_host_io(bool on) const { host_io_ = on; }

private:
    long long n_;
    kind k_ = kind::trivial;
    mutable bool host_io_ = false;
    block_program<T> prog_; // smem: length n; bluestein_smem: length m
    // Bluestein
    long long m_ = 0;
    dbuf chirp_, bhat_;
    std::unique_ptr<complex_engine<T>> inner_;
    // four-step
    long long n1_ = 0, n2_ = 0;
    block_program<T> pcols_, prows_;
    int tile_c_ = 1, tile_r_ = 1;
    bool pp_c_ = false, pp_r_ = false; // ping-pong column / row passes
    bool pair_ = false;                 // both passes as fully compile-time pair kernels
    dbuf twA_, twB_;
    int lbits_ = 0;
    // pipelined smem path (compile-time lengths): signals per tile, 0 = not used
    int pipe_spc_ = 0;
    bool reg_     = false; // persistent one-signal-per-CTA kernel (pipeline does not fit)
    dbuf err_;

    void init_bluestein(long long n);
    void init_rader(long long n);
    bool plan_fourstep(long long n);
    void plan_pipe();
    // tensor-core form (n1_, n2_, twA_, twB_, lbits_ as for the four-step when n > 4096)
    int tc_mode_ = 0;
    dbuf tc_cs_, tc_tw1_, tc_tw2_;
    // Rader
    dbuf pin_, qof_;
    // Rader with prime-factor convolution DFTs (rader_pfa.cu): signals per tile (0 = not used), its axes and
    // its gather / scatter / kernel-spectrum tables
    int pfa_spc_ = 0;
    std::vector<int> pfa_axes_;
    dbuf tin_, tout_, bphys_;
};

// dft_plan_real<T>: N even, N/2-point complex engine plus the CCs/Perm split / merge.
template <typename T>
class real_engine
{
public:
    explicit real_engine(long long n);
    long long scratch_elems(long long batch) const;
    void forward(void* out, const void* in, long long batch, bool ccs, void* scratch, cudaStream_t st) const;
    void inverse(void* out, const void* in, long long batch, bool ccs, void* scratch, cudaStream_t st) const;
    std::string describe() const;
    long long size() const { return n_; }
    int launches(long long batch) const;
    // Throws if a kernel of this engine recorded a device-side error (a bounded wait that ran out).
    void check_device_error() const;

private:
    long long n_, c_;
    complex_engine<T> ceng_;
    block_program<T> prog_; // fused kernels: c-point program
    dbuf rtw_;
    bool fused_ = false;
    int pipe_spc_ = 0; // signals per tile of the pipelined forward / inverse kernels, 0 = not used
    dbuf err_;
    // forward on the complex engine's pair kernels with the split fused into the row pass (16-byte-aligned
    // input; launch_ct_fsp_r2c_f32), and its two-level table of W_n^k: W_n^k1 (k1 < n1), W_n^(n1 k2)
    bool rfsp_ = false;
    dbuf rtw2_;
};

// dct_plan<T>: DCT-II forward, DCT-III (X0 halved) inverse, unscaled.
template <typename T>
class dct_engine
{
public:
    explicit dct_engine(long long n);
    long long scratch_elems(long long batch) const;
    void execute(void* out, const void* in, long long batch, bool inverse, void* scratch, cudaStream_t st) const;
    std::string describe() const;
    long long size() const { return n_; }
    int launches(long long batch) const;
    void check_device_error() const;

private:
    long long n_;
    complex_engine<T> ceng_;
    block_program<T> prog_; // fused kernels: n-point program
    dbuf dtw_;
    bool fused_ = false;
    int pipe_spc_ = 0; // signals per tile of the pipelined kernels, 0 = not used
    dbuf err_;
};

} // namespace kfr_gpu
