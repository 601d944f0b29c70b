// Kernel launch interface between the host planner (plan.cpp) and the CUDA kernels (kernels.cuh).
// Everything here is plain C++: pointers are device addresses, strides are in elements.
#pragma once

#include <cstddef>
#include <vector>
#include <cuda_runtime.h>

#include "fft_desc.hpp"

namespace kfr_gpu
{

// Polling rounds after which a kernel's wait for a bulk copy (mbarrier try_wait rounds, each suspending for
// a bounded, hardware-defined time) or for an earlier stage of its signal (256 ns sleeps) gives up: about a
// second or more.  On expiry the kernel sets its plan's device error flag, lets its own copies in flight
// land (waiting at most this default again) and returns.
constexpr unsigned kDefaultWaitSpins = 1u << 22;
// The limit that launches issued from now on carry (kfr_set_wait_limit; 0 gives up at the first poll).
unsigned wait_limit();
unsigned set_wait_limit(unsigned spins);

// Shape of one shared-memory FFT launch: `spc` signals per CTA, `ts` threads per signal, each thread owning
// at most `ept` elements per pass.
struct block_cfg
{
    int ept;
    int ts;
    int spc;
    int threads;
    int smem;
    long long grid;
    int ct = 0; // nonzero: length of the compile-time specialised kernel to use (ct_table.hpp)
};

// Batched complex DFT of contiguous signals that fit one CTA's shared memory.
struct c2c_args
{
    const void* in;
    void* out;
    long long batch;
    long long istride, ostride; // complex elements between consecutive signals
    int inverse;
    const void* tw;
    fast_div div_n;
    fft_desc d;
    unsigned wait_spins = kDefaultWaitSpins; // persistent pipelined kernels: see kDefaultWaitSpins
};

// Bluestein chirp-z for lengths n whose power-of-two convolution size M = d.n fits one CTA.
struct bluestein_args
{
    const void* in;
    void* out;
    long long batch;
    long long istride, ostride;
    int n;
    int inverse;
    const void* chirp; // n values e^{-i pi k^2 / n}
    const void* bhat;  // M values: FFT_M of the conjugate chirp, scaled by 1/M
    const void* tw;
    fast_div div_n, div_m;
    fft_desc d;
};

// Rader's algorithm for a prime length n whose cyclic convolution length L = n - 1 = d.n fits one CTA:
// x[g^p] (p < L) is permuted into the convolution input on load, convolved with b[m] = W_n^{g^-m} through
// two L-point DFTs, and X[g^-q] = x[0] + c[q] is gathered back on store (X[0] = x[0] + sum x).
struct rader_args
{
    const void* in;
    void* out;
    long long batch;
    long long istride, ostride;
    int n;
    int inverse;
    const int* pin;   // pin[v] = p with g^p = v (mod n), v = 1..n-1
    const int* qof;   // qof[k] = q with g^-q = k (mod n), k = 1..n-1
    const void* bhat; // L values: DFT_L(b) / L
    const void* tw;
    fast_div div_n, div_l;
    fft_desc d;
};

// Rader's algorithm with prime-factor convolution DFTs (rader_pfa.cu): in and out 16-byte aligned, signals
// contiguous (stride n); tin / tout / bphys: the gather, scatter and kernel-spectrum tables over the
// prime-factor array of L = n - 1 points (see rader_pfa.cu).
struct rader_pfa_args
{
    const void* in;
    void* out;
    long long batch;
    int inverse;
    const int* tin;
    const int* tout;
    const void* bphys;
    int* err; // set when a wait for a tile copy runs out
    unsigned wait_spins = kDefaultWaitSpins;
};
// Whether a compile-time prime-factor Rader kernel exists for n (single precision): its axes (axis 0 first,
// the fused axis last) and signals per tile.
bool rader_pfa_shape(long long n, std::vector<int>& axes, int& spc);
cudaError_t launch_rader_pfa_f32(const rader_pfa_args& a, long long n, cudaStream_t st);

// Real DFT of even length 2c through a c-point complex DFT (d.n = c).
// Forward: in = reals (istride reals apart), out = c+1 (CCs) or c (Perm) complex (ostride complex apart).
// Inverse: in = c+1 / c complex (istride complex apart), out = 2c reals (ostride reals apart).
struct real_args
{
    const void* in;
    void* out;
    long long batch;
    long long istride, ostride;
    int ccs;
    const void* rtw; // W_{2c}^k for k = 0..c
    const void* tw;
    fast_div div_n, div_out;
    fft_desc d;
    unsigned wait_spins = kDefaultWaitSpins; // persistent pipelined kernels: see kDefaultWaitSpins
};

// DCT-II / DCT-III of length n = d.n through an n-point complex DFT.
struct dct_args
{
    const void* in;
    void* out;
    long long batch;
    long long stride; // reals between consecutive signals (in and out)
    const void* dtw;  // (cos(pi k / 2n), sin(pi k / 2n)) for k < n
    const void* tw;
    fast_div div_n;
    fft_desc d;
    unsigned wait_spins = kDefaultWaitSpins; // pipelined kernels: see kDefaultWaitSpins
};

// One pass of the four-step decomposition of N = n1 * n2 (x viewed as n1 rows by n2 columns).
//   cols pass: FFT_n1 down each column, times W_N^{col * k1}, written column-contiguous to out[col*n1 + k1]
//   rows pass: FFT_n2 along each k1 of the cols output, written to out[k1 + n1*k2]
struct fourstep_args
{
    const void* in;
    void* out;
    long long batch;
    long long sig_stride; // complex elements between consecutive signals
    int n1, n2;
    int tile;             // columns (cols pass) or k1 rows (rows pass) per CTA
    int conj_in, conj_out;
    const void* tw;
    fft_desc d;
    // two-level table for W_N^m: W_N^m = twA[m >> lbits] * twB[m & ((1 << lbits) - 1)]
    const void* twA;
    const void* twB;
    int lbits;
    int tile_shift;  // log2(tile)
    int same_layout; // cols pass: store back to x's own layout (multi-dimensional axes) and skip the twiddle
    int pingpong;    // compile-time kernels: ping-pong passes over two buffers per signal (2x shared memory)
    fast_div div_n;  // divides by the FFT length of this pass
    int* err;        // persistent pair kernels: set when a wait for a tile copy runs out (may be null)
    unsigned wait_spins = kDefaultWaitSpins;
    // real forward DFT fused into the pair kernels (launch_ct_fsp_r2c_f32): x is the real signal viewed as
    // n = n1 n2 complex values; the cols pass writes out[col*p1 + pos(k1)] with p1 = n1 rounded up to even and
    // pos() placing k1 and n1 - k1 side by side; the rows pass writes the real spectrum (n + 1 bins for CCs,
    // n for Perm) from both rows of each pair, with rtw = W_2n^k1 (k1 < n1) followed by W_2n^(n1 k2) (k2 < n2)
    const void* rtw = nullptr;
    int ccs         = 1;
};

template <typename T>
cudaError_t launch_c2c(const c2c_args& a, const block_cfg& c, cudaStream_t st);
template <typename T>
cudaError_t launch_bluestein(const bluestein_args& a, const block_cfg& c, cudaStream_t st);
template <typename T>
cudaError_t launch_rader(const rader_args& a, const block_cfg& c, cudaStream_t st);
template <typename T>
cudaError_t launch_r2c(const real_args& a, const block_cfg& c, cudaStream_t st);
template <typename T>
cudaError_t launch_c2r(const real_args& a, const block_cfg& c, cudaStream_t st);
template <typename T>
cudaError_t launch_dct2(const dct_args& a, const block_cfg& c, cudaStream_t st);
template <typename T>
cudaError_t launch_dct3(const dct_args& a, const block_cfg& c, cudaStream_t st);
template <typename T>
cudaError_t launch_fs_cols(const fourstep_args& a, const block_cfg& c, cudaStream_t st);
template <typename T>
cudaError_t launch_fs_rows(const fourstep_args& a, const block_cfg& c, cudaStream_t st);

// Grid-stride elementwise kernels for the multi-kernel paths: Bluestein at lengths whose convolution does
// not fit one CTA, and real-DFT / DCT pre- and post-processing around a multi-kernel complex DFT.  The
// single-CTA paths fuse the same arithmetic into the FFT kernels.
struct ew_args
{
    const void* in;
    void* out;
    long long batch;
    long long n;     // elements per signal of the produced array
    long long istride, ostride;
    const void* t0;  // first table
    const void* t1;  // second table
    long long n_src; // length of the source signal (Bluestein) or the complex length c (real DFT)
    int flag;        // inverse (Bluestein) / CCs (real DFT)
};

enum ew_op
{
    EW_BS_PRE    = 0, // out[e] = e < n_src ? conj_if(in[e], flag) * chirp[e] : 0   (n = M)
    EW_BS_MID    = 1, // out[e] = conj(in[e] * bhat[e])                               (n = M)
    EW_BS_POST   = 2, // out[k] = conj_if(conj(in[k]) * chirp[k], flag)               (n = N)
    EW_DCT2_PRE  = 5, // mirrored complex input (n = N)
    EW_DCT2_POST = 6, // Re*cos + Im*sin (n = N)
    EW_DCT3_PRE  = 7, // x * e^{-i pi k / 2N}, X0 halved (n = N)
    EW_DCT3_POST = 8, // un-mirror real parts (n = N)
};

template <typename T>
cudaError_t launch_elementwise(int op, const ew_args& a, cudaStream_t st);
// The real-DFT split (forward: X[k] = (Z[k] + conj Z[c-k]) / 2 - i W_2c^k (Z[k] - conj Z[c-k]) / 2 from the
// c-point spectrum Z of the reals taken in pairs; n = c + 1 bins for CCs, c for Perm) or merge (inverse: the
// c-point spectrum whose inverse gives the reals) with one thread per mirror pair (e, c - e) of each
// spectrum, so that every spectrum element is read once: a.n_src = c, a.flag = CCs, strides as for
// launch_elementwise, a.t0 = W_2c^k for k = 0..c.
template <typename T>
cudaError_t launch_real_pairs(const ew_args& a, bool inverse, cudaStream_t st);

// Batched transpose of complex matrices: out[b][c][r] = in[b][r][c] (b < batch, r < rows, c < cols).
template <typename T>
cudaError_t launch_transpose(void* out, const void* in, long long batch, long long rows, long long cols,
                             cudaStream_t st);

// fft_multiply / fft_multiply_accumulate over `batch` spectra of `size` elements stored back to back:
// dest = (acc ? acc : 0) + src1 * src2, with the Perm format's element 0 formed from the real and the
// imaginary parts separately.  src2_stride: 0 (one spectrum shared by every signal) or size.  acc may alias
// dest; src1 / src2 may alias dest.
template <typename T>
cudaError_t launch_fft_multiply(void* dest, const void* acc, const void* src1, const void* src2, long long size,
                                long long batch, long long src2_stride, bool perm, cudaStream_t st);

// Compile-time specialised kernels (single precision; lengths in ct_table.hpp).  kind: see ct_kind.
cudaError_t launch_ct_c2c_f32(const c2c_args& a, const block_cfg& c, cudaStream_t st);
// Persistent TMA-pipelined complex DFT over `ntiles` whole tiles of c.spc contiguous signals (c.smem must
// hold two unpadded tiles, the padded work tile and two mbarriers; in must be 16-byte aligned).
cudaError_t launch_ct_c2c_pipe_f32(const c2c_args& a, const block_cfg& c, long long ntiles, int* err,
                                   cudaStream_t st);
// real forward DFT, persistent and pipelined over tiles of c.spc (even) signals (compile-time c = n / 2)
cudaError_t launch_ct_r2c_pipe_f32(const real_args& a, const block_cfg& c, long long ntiles, int* err, cudaStream_t st);
// real inverse DFT, persistent and pipelined over tiles of c.spc (even) signals (compile-time c = n / 2)
cudaError_t launch_ct_c2r_pipe_f32(const real_args& a, const block_cfg& c, long long ntiles, int* err, cudaStream_t st);
// DCT-II (inverse = false) or DCT-III, persistent and pipelined over tiles of c.spc signals (compile-time n;
// in and out 16-byte aligned, a.stride == n)
cudaError_t launch_ct_dct_pipe_f32(const dct_args& a, const block_cfg& c, long long ntiles, int* err, bool inverse,
                                   cudaStream_t st);
// one signal per CTA, persistent, signal in registers between the passes (compile-time lengths >= 8192)
cudaError_t launch_ct_c2c_reg_f32(const c2c_args& a, const block_cfg& c, long long nsig, int* err, cudaStream_t st);
cudaError_t launch_ct_bluestein_f32(const bluestein_args& a, const block_cfg& c, cudaStream_t st);
cudaError_t launch_ct_rader_f32(const rader_args& a, const block_cfg& c, cudaStream_t st);
cudaError_t launch_ct_r2c_f32(const real_args& a, const block_cfg& c, cudaStream_t st);
cudaError_t launch_ct_c2r_f32(const real_args& a, const block_cfg& c, cudaStream_t st);
cudaError_t launch_ct_dct2_f32(const dct_args& a, const block_cfg& c, cudaStream_t st);
cudaError_t launch_ct_dct3_f32(const dct_args& a, const block_cfg& c, cudaStream_t st);
cudaError_t launch_ct_fs_cols_f32(const fourstep_args& a, const block_cfg& c, cudaStream_t st);
// Compile-time pair kernels (KFR_CT_FSPAIR_F32): the column pass (cols = true) or the row pass of the split
// a.n1 x a.n2 over a.batch signals (contiguous, a.batch <= 65535).  False / cudaErrorInvalidValue if the pair
// has no kernel.
bool has_ct_fsp_f32(int n1, int n2);
cudaError_t launch_ct_fsp_f32(const fourstep_args& a, bool cols, cudaStream_t st);
// The real forward DFT of length 2 n1 n2 on the tensor-copy pair kernels with its split fused into the row
// pass (two HBM round trips instead of three): whether the split n1 x n2 has them, and the two launches
// (cols: the permuted column pass into a.out = scratch of batch n2 p1 values; rows: the fused row pass into
// the spectrum).  The caller checks the alignment first: a.in and the scratch 16-byte aligned.
bool has_ct_fsp_r2c_f32(int n1, int n2);
cudaError_t launch_ct_fsp_r2c_f32(const fourstep_args& a, bool cols, cudaStream_t st);
cudaError_t launch_ct_fs_rows_f32(const fourstep_args& a, const block_cfg& c, cudaStream_t st);

// Launch bookkeeping done once per process instead of on every launch (launch_cache.cpp): the kernel's
// dynamic shared-memory limit is raised to at least `smem` the first time it is needed, and *per_sm (if
// given) receives how many blocks of `threads` threads and `smem` bytes of dynamic shared memory fit one SM.
// Keyed by device, kernel, threads and smem.
cudaError_t prepare_launch(const void* kernel, int threads, int smem, int* per_sm = nullptr);
// SMs of the current device (0 if the query fails), queried once per device.
int device_sm_count();

// Largest thread count a block FFT kernel may be launched with (elem_bytes = sizeof(real type)).
int max_threads_for(int elem_bytes, int ept);
// Largest dynamic shared memory a kernel may use on this device.
int max_smem_bytes();

} // namespace kfr_gpu
