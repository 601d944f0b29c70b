// Transform kernels.  Each kernel stages its signals in shared memory (coalesced global loads, with the
// transform's pre-processing fused into the load), runs block_fft, and writes the result back with the
// post-processing fused into the store, so a signal crosses HBM exactly once in each direction.
//
// Inverse transforms use conj(DFT(conj(x))), which is the unscaled inverse DFT of the reference
// (include/kfr/dft/fft.hpp:262: no scaling), so only forward codelets and forward twiddles exist.
#pragma once

#include <type_traits>

#include "ct_table.hpp"
#include "fft_device.cuh"
#include "launch.hpp"
#include "tma.cuh"

namespace kfr_gpu
{

// FFT policies.  A kernel is instantiated with one of them:
//   rt_fft<T, EPT>          runtime radix sequence (any one-CTA length), pass list staged in shared memory
//   ct_fft<T, N, TS, Rs...> compile-time length and radices (ct_table.hpp)
// Both expose n (length), ts (threads per signal), max_threads (launch bound) and run(buf, tw, lt).
template <typename T, int EPT>
struct rt_fft
{
    static constexpr bool compile_time = false;
    // the block FFT keeps EPT complex values per thread in registers
    static constexpr int max_threads = (sizeof(T) == 4 ? 1024 : 512) / (EPT / 16);
    const pass_desc* sp;
    int npass, n, ts;
    __device__ __forceinline__ rt_fft(pass_desc* s, const fft_desc& d, int ts_) : sp(s), npass(d.npass), n(d.n), ts(ts_)
    {
        stage_passes(s, d);
    }
    __device__ __forceinline__ void run(cpx<T>* buf, const cpx<T>* __restrict__ tw, int lt) const
    {
        block_fft<T, EPT>(buf, sp, npass, n, tw, lt, ts);
    }
    // shared-memory layout: signals gstride(n) elements apart, element i at pi(i)
    static __host__ __device__ constexpr int gstride(int len) { return padded_len<T>(len); }
    static __device__ __forceinline__ int pi(int i) { return pidx<T>(i); }
};

template <typename T, int N, int TS, int... Rs>
struct ct_fft
{
    static constexpr bool compile_time = true;
    static constexpr int max_threads = sizeof(T) == 4 ? 1024 : 512;
    static constexpr int n           = N;
    static constexpr int ts          = TS;
    // shared-memory layout (ct_table.hpp): signals gstride() elements apart, element i at pi(i)
    static constexpr int ps = ct_ps<T>(N, TS);
    static __host__ __device__ constexpr int gstride(int = N)
    {
        return sizeof(T) == 4 ? ct_group_stride_f32(N, TS) : padded_len<T>(N);
    }
    static __device__ __forceinline__ int pi(int i) { return pidx_s<ps>(i); }
    __device__ __forceinline__ ct_fft(pass_desc*, const fft_desc&, int) {}
    __device__ __forceinline__ void run(cpx<T>* buf, const cpx<T>* __restrict__ tw, int lt) const
    {
        ct_block_fft<T, N, TS, Rs...>(buf, tw, lt);
    }
    static constexpr int npass = sizeof...(Rs);
    // radix of the last pass (whose butterfly j produces outputs j + r n / rlast)
    static constexpr int rlast = [] {
        constexpr int r[] = { Rs... };
        return r[sizeof...(Rs) - 1];
    }();
    template <class LD, class ST, class H, class P>
    __device__ __forceinline__ void run_pp(const LD& ld, const ST& st, const H& hook, const P& pre_last, cpx<T>* A,
                                           cpx<T>* B, const cpx<T>* __restrict__ tw, int lt) const
    {
        ct_block_fft_pp<T, N, TS, Rs...>(ld, st, hook, pre_last, A, B, tw, lt);
    }
    // in place with the signal in registers: first pass reads ld(p), hook() after it, last pass stores
    // st(q, x) after mid()
    template <class LD, class MID, class ST, class H>
    __device__ __forceinline__ void run_io(const LD& ld, const MID& mid, const ST& st, const H& hook, cpx<T>* buf,
                                           const cpx<T>* __restrict__ tw, int lt) const
    {
        ct_block_fft_io<T, N, TS, Rs...>(ld, mid, st, hook, buf, tw, lt);
    }
    // as run_pp, with post(j, o) applied to each last-pass butterfly's outputs before they are stored
    template <class LD, class PO, class ST>
    __device__ __forceinline__ void run_pp_post(const LD& ld, const PO& post, const ST& st, cpx<T>* A, cpx<T>* B,
                                                const cpx<T>* __restrict__ tw, int lt) const
    {
        const auto nothing = []() {};
        ct_block_fft_pp<T, N, TS, Rs...>(ld, st, nothing, nothing, A, B, tw, lt, post);
    }
};

__device__ __forceinline__ uint32_t div_by(uint32_t x, const fast_div f) { return fdiv(x, f); }

// Block-wide strided copy i = threadIdx.x + k * blockDim.x, i < total: U loads ld(i) are issued before
// their U stores st(i, v), so each thread keeps U global loads in flight.
template <int U, class LD, class ST>
__device__ __forceinline__ void copy_batched(const int total, const LD& ld, const ST& st)
{
    for (int base = threadIdx.x; base < total; base += U * int(blockDim.x))
    {
        decltype(ld(0)) v[U];
#pragma unroll
        for (int e = 0; e < U; e++)
        {
            const int i = base + e * int(blockDim.x);
            if (i < total)
                v[e] = ld(i);
        }
#pragma unroll
        for (int e = 0; e < U; e++)
        {
            const int i = base + e * int(blockDim.x);
            if (i < total)
                st(i, v[e]);
        }
    }
}

// thread -> (signal slot, lane within the signal's thread group)
struct group_map
{
    int g, lt;
    __device__ __forceinline__ group_map(int ts, int spc)
    {
        g  = int(threadIdx.x) / ts;
        lt = g < spc ? int(threadIdx.x) - g * ts : ts;
        if (g >= spc)
            g = 0;
    }
};

// ---------------------------------------------------------------------------------------------------
// Complex DFT, contiguous batch (dft_plan<T>::execute over many signals)
// ---------------------------------------------------------------------------------------------------
template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1) k_c2c(const c2c_args a, const int ts, const int spc)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ pass_desc sp[kMaxPasses];
    const F fft(sp, a.d, ts);
    cpx<T>* sm        = reinterpret_cast<cpx<T>*>(smem_raw);
    const int n       = fft.n;
    const int stride  = F::gstride(n);
    const long long s0 = (long long)blockIdx.x * spc;
    const cpx<T>* __restrict__ in = reinterpret_cast<const cpx<T>*>(a.in);
    cpx<T>* __restrict__ out      = reinterpret_cast<cpx<T>*>(a.out);
    const bool inv  = a.inverse != 0;
    const int total = spc * n;
#pragma unroll 4
    for (int i = threadIdx.x; i < total; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_n));
        const int e = i - s * n;
        const long long sig = s0 + s;
        if (sig < a.batch)
            sm[s * stride + F::pi(e)] = conj_if(in[sig * a.istride + e], inv);
    }
    __syncthreads();
    const group_map gm(ts, spc);
    fft.run(sm + gm.g * stride, reinterpret_cast<const cpx<T>*>(a.tw), gm.lt);
#pragma unroll 4
    for (int i = threadIdx.x; i < total; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_n));
        const int e = i - s * n;
        const long long sig = s0 + s;
        if (sig < a.batch)
            out[sig * a.ostride + e] = conj_if(sm[s * stride + F::pi(e)], inv);
    }
}

// ---------------------------------------------------------------------------------------------------
// Complex DFT, contiguous batch, persistent and pipelined (compile-time lengths).  Each CTA walks tiles of
// `spc` whole signals (tile t = signals [t*spc, t*spc + spc), a whole number of 16-byte units).  Three tile
// buffers rotate: the input tile (loaded by one bulk asynchronous copy, TMA; then the passes' A buffer), the
// scratch tile (the passes' B buffer) and the spare tile, into which the next tile streams while the CTA
// transforms the current one.  The first pass reads the input tile, the passes ping-pong between A and B in
// the padded layout, and the last pass writes the tile's output in natural order into whichever of the two
// it does not read; one bulk copy stores it.  The next tile's input is this one's spare, its scratch the
// buffer the last pass read, its spare this one's output (reloaded once its bulk store has read it).  Only
// whole tiles are handled here; the host runs the remainder with k_c2c.  A wait that runs out sets *err and
// the CTA returns.
// ---------------------------------------------------------------------------------------------------
template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1)
    k_c2c_pipe(const c2c_args a, const long long ntiles, const int spc, int* err)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int N      = F::n;
    constexpr int STRIDE = F::gstride(N);
    const F fft(nullptr, a.d, F::ts);
    const int tile      = spc * N;
    const int slen      = pipe_stage_len(spc, N, STRIDE);
    cpx<T>* const tiles = reinterpret_cast<cpx<T>*>(smem_raw);
    uint64_t* bars      = reinterpret_cast<uint64_t*>(tiles + 3 * slen);
    const uint32_t bytes = uint32_t(tile) * uint32_t(sizeof(cpx<T>));
    const cpx<T>* in = reinterpret_cast<const cpx<T>*>(a.in);
    cpx<T>* out      = reinterpret_cast<cpx<T>*>(a.out);
    const cpx<T>* tw = reinterpret_cast<const cpx<T>*>(a.tw);
    const bool inv   = a.inverse != 0;
    const group_map gm(F::ts, spc);
    if (threadIdx.x == 0)
    {
        for (int b = 0; b < 3; b++)
            mbar_init(&bars[b], 1);
        mbar_fence_init();
    }
    __syncthreads();
    long long t = blockIdx.x;
    if (threadIdx.x == 0 && t < ntiles)
    {
        mbar_arrive_expect_tx(&bars[0], bytes);
        bulk_g2s(tiles, in + t * tile, bytes, &bars[0]);
    }
    uint32_t phase = 0;              // bit b: parity to wait for on tile buffer b
    int bi = 0, bs = 1, bn = 2;      // input, scratch and spare tile buffers
    for (; t < ntiles; t += gridDim.x)
    {
        cpx<T>* in_t   = tiles + bi * slen;
        cpx<T>* scr_t  = tiles + bs * slen;
        const bool got = mbar_wait(&bars[bi], (phase >> bi) & 1, a.wait_spins);
        if (!__syncthreads_and(got))
        {
            if (threadIdx.x == 0)
            {
                atomicExch(err, 1);
                // the copy waited for is the only load in flight (the next one is issued after this wait):
                // give it a bounded chance to land in this CTA's shared memory before the CTA exits
                mbar_wait(&bars[bi], (phase >> bi) & 1);
                bulk_wait_all();
            }
            return;
        }
        phase ^= 1u << bi;
        const long long tn = t + gridDim.x;
        // after the first pass: the spare buffer holds the previous tile's output; once its bulk store has
        // read it, stream the next tile in
        const auto prefetch = [&]()
        {
            if (threadIdx.x == 0 && tn < ntiles)
            {
                bulk_wait_read();
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(&bars[bn], bytes);
                bulk_g2s(tiles + bn * slen, in + tn * tile, bytes, &bars[bn]);
            }
        };
        // pass i writes B (i even) or A (i odd): the last pass reads A when the pass count is odd
        constexpr bool odd = F::npass % 2 == 1;
        cpx<T>* ob         = odd ? scr_t : in_t;
        const cpx<T>* src  = in_t + gm.g * N;
        cpx<T>* osig       = ob + gm.g * N;
        const auto nothing = []() {};
        fft.run_pp([&](int p) { return conj_if(src[p], inv); }, [&](int q, cpx<T> x) { osig[q] = conj_if(x, inv); },
                   prefetch, nothing, in_t + gm.g * STRIDE, scr_t + gm.g * STRIDE, tw, gm.lt);
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0)
        {
            bulk_s2g(out + t * tile, ob, bytes);
            bulk_commit();
        }
        const int ob_i = odd ? bs : bi, free_i = odd ? bi : bs;
        bi = bn;
        bs = free_i;
        bn = ob_i;
    }
    if (threadIdx.x == 0)
        bulk_wait_all();
}

// ---------------------------------------------------------------------------------------------------
// Complex DFT, one signal per CTA, persistent (compile-time lengths whose three-tile pipeline does not fit,
// e.g. N = 8192, 16384).  The signal lives in registers between the passes, which exchange through one
// padded shared buffer.  Each signal arrives by two bulk copies (TMA): its first half into a spare half-size
// buffer, issued as soon as the previous signal's first pass has read that buffer, and its second half into
// the exchange buffer, issued once the previous signal's last pass has read it (its outputs then go straight
// to global memory while the copy lands).  A wait that runs out sets *err and the CTA returns.
// ---------------------------------------------------------------------------------------------------
template <typename T, class F>
__host__ __device__ constexpr int reg_smem_bytes()
{
    // exchange buffer (rounded to an even count: 16-byte boundary), spare first half, two mbarriers
    return ((F::gstride(F::n) + 1) / 2 * 2 + F::n / 2) * int(sizeof(cpx<T>)) + 16;
}

template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1)
    k_c2c_reg(const c2c_args a, const long long nsig, int* err)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int N          = F::n;
    constexpr int H          = N / 2;
    constexpr uint32_t hbytes = uint32_t(H) * uint32_t(sizeof(cpx<T>));
    const F fft(nullptr, a.d, F::ts);
    static_assert(N % 2 == 0 && hbytes % 16 == 0, "two halves of whole 16-byte units per signal");
    cpx<T>* buf      = reinterpret_cast<cpx<T>*>(smem_raw);
    cpx<T>* spare    = buf + (F::gstride(N) + 1) / 2 * 2; // on a 16-byte boundary
    uint64_t* bars   = reinterpret_cast<uint64_t*>(spare + H); // [0]: first half (spare), [1]: second half
    const cpx<T>* in = reinterpret_cast<const cpx<T>*>(a.in);
    cpx<T>* out      = reinterpret_cast<cpx<T>*>(a.out);
    const cpx<T>* tw = reinterpret_cast<const cpx<T>*>(a.tw);
    const bool inv   = a.inverse != 0;
    const int lt     = int(threadIdx.x);
    if (threadIdx.x == 0)
    {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    long long s = blockIdx.x;
    if (threadIdx.x == 0 && s < nsig)
    {
        mbar_arrive_expect_tx(&bars[0], hbytes);
        bulk_g2s(spare, in + s * N, hbytes, &bars[0]);
        mbar_arrive_expect_tx(&bars[1], hbytes);
        bulk_g2s(buf + H, in + s * N + H, hbytes, &bars[1]);
    }
    for (uint32_t phase = 0; s < nsig; s += gridDim.x, phase ^= 1)
    {
        const bool got = mbar_wait(&bars[0], phase, a.wait_spins) && mbar_wait(&bars[1], phase, a.wait_spins);
        if (!__syncthreads_and(got))
        {
            if (threadIdx.x == 0)
            {
                atomicExch(err, 1);
                // the two halves waited for are the only copies in flight (the next ones are issued after
                // these waits): give them a bounded chance to land before the CTA exits
                mbar_wait(&bars[0], phase);
                mbar_wait(&bars[1], phase);
                bulk_wait_all();
            }
            return;
        }
        const long long sn = s + gridDim.x;
        cpx<T>* o          = out + s * N;
        fft.run_io([&](int p) { return conj_if(p < H ? spare[p] : buf[p], inv); },
                   [&]()
                   {
                       // every thread has read the exchange buffer: the next signal's second half may land in it
                       __syncthreads();
                       if (threadIdx.x == 0 && sn < nsig)
                       {
                           fence_proxy_async_smem();
                           mbar_arrive_expect_tx(&bars[1], hbytes);
                           bulk_g2s(buf + H, in + sn * N + H, hbytes, &bars[1]);
                       }
                   },
                   [&](int q, cpx<T> x) { o[q] = conj_if(x, inv); },
                   [&]()
                   {
                       // the first pass has read the spare buffer: the next signal's first half may land in it
                       if (threadIdx.x == 0 && sn < nsig)
                       {
                           fence_proxy_async_smem();
                           mbar_arrive_expect_tx(&bars[0], hbytes);
                           bulk_g2s(spare, in + sn * N, hbytes, &bars[0]);
                       }
                   },
                   buf, tw, lt);
    }
}

// ---------------------------------------------------------------------------------------------------
// Bluestein (dft_arblen_stage_impl, src/dft/dft-impl.hpp:248-272), fused into one kernel:
//   a = x * chirp (zero padded to M) -> FFT_M -> * bhat -> inverse FFT_M -> * chirp
// ---------------------------------------------------------------------------------------------------
template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1) k_bluestein(const bluestein_args a, const int ts,
                                                                        const int spc)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ pass_desc sp[kMaxPasses];
    const F fft(sp, a.d, ts);
    cpx<T>* sm        = reinterpret_cast<cpx<T>*>(smem_raw);
    const int m       = fft.n;
    const int n       = a.n;
    const int stride  = F::gstride(m);
    const long long s0 = (long long)blockIdx.x * spc;
    const cpx<T>* __restrict__ in    = reinterpret_cast<const cpx<T>*>(a.in);
    cpx<T>* __restrict__ out         = reinterpret_cast<cpx<T>*>(a.out);
    const cpx<T>* __restrict__ chirp = reinterpret_cast<const cpx<T>*>(a.chirp);
    const cpx<T>* __restrict__ bhat  = reinterpret_cast<const cpx<T>*>(a.bhat);
    const bool inv = a.inverse != 0;
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * m; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_m));
        const int e = i - s * m;
        const long long sig = s0 + s;
        cpx<T> v = mk<T>(0, 0);
        if (e < n && sig < a.batch)
            v = conj_if(in[sig * a.istride + e], inv) * ldg(chirp + e);
        sm[s * stride + F::pi(e)] = v;
    }
    __syncthreads();
    const group_map gm(ts, spc);
    const cpx<T>* tw = reinterpret_cast<const cpx<T>*>(a.tw);
    fft.run(sm + gm.g * stride, tw, gm.lt);
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * m; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_m));
        const int e = i - s * m;
        cpx<T>& r   = sm[s * stride + F::pi(e)];
        r           = conj(r * ldg(bhat + e));
    }
    __syncthreads();
    fft.run(sm + gm.g * stride, tw, gm.lt);
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * n; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_n));
        const int k = i - s * n;
        const long long sig = s0 + s;
        if (sig < a.batch)
            out[sig * a.ostride + k] = conj_if(conj(sm[s * stride + F::pi(k)]) * ldg(chirp + k), inv);
    }
}

// ---------------------------------------------------------------------------------------------------
// Rader (prime n, L = n - 1 fits one CTA): permute on load, L-point DFT, times bhat, inverse L-point DFT,
// gather on store.  x[0] and the DC term of the permuted input's DFT are kept per signal after the
// signals' slots in shared memory.
// ---------------------------------------------------------------------------------------------------
template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1) k_rader(const rader_args a, const int ts, const int spc)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ pass_desc sp[kMaxPasses];
    const F fft(sp, a.d, ts);
    cpx<T>* sm         = reinterpret_cast<cpx<T>*>(smem_raw);
    const int L        = fft.n;
    const int n        = L + 1;
    const int stride   = F::gstride(L);
    cpx<T>* x0s        = sm + spc * stride; // spc values
    cpx<T>* dcs        = x0s + spc;        // spc values
    const long long s0 = (long long)blockIdx.x * spc;
    const cpx<T>* __restrict__ in   = reinterpret_cast<const cpx<T>*>(a.in);
    cpx<T>* __restrict__ out        = reinterpret_cast<cpx<T>*>(a.out);
    const cpx<T>* __restrict__ bhat = reinterpret_cast<const cpx<T>*>(a.bhat);
    const bool inv = a.inverse != 0;
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * n; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_n));
        const int e = i - s * n;
        const long long sig = s0 + s;
        const cpx<T> v = sig < a.batch ? conj_if(in[sig * a.istride + e], inv) : mk<T>(0, 0);
        if (e == 0)
            x0s[s] = v;
        else
            sm[s * stride + F::pi(__ldg(a.pin + e))] = v;
    }
    __syncthreads();
    const group_map gm(ts, spc);
    const cpx<T>* tw = reinterpret_cast<const cpx<T>*>(a.tw);
    fft.run(sm + gm.g * stride, tw, gm.lt);
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * L; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_l));
        const int q = i - s * L;
        cpx<T>& r   = sm[s * stride + F::pi(q)];
        const cpx<T> A = r;
        if (q == 0)
            dcs[s] = A;
        r = conj(A * ldg(bhat + q));
    }
    __syncthreads();
    fft.run(sm + gm.g * stride, tw, gm.lt);
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * n; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_n));
        const int k = i - s * n;
        const long long sig = s0 + s;
        if (sig >= a.batch)
            continue;
        const cpx<T> x0 = x0s[s];
        const cpx<T> X  = k == 0 ? x0 + dcs[s] : x0 + conj(sm[s * stride + F::pi(__ldg(a.qof + k))]);
        out[sig * a.ostride + k] = conj_if(X, inv);
    }
}


// ---------------------------------------------------------------------------------------------------
// Real forward DFT (dft_plan_real, CCs / Perm): c-point complex DFT of the reals viewed as c complex
// values, then the split of to_fmt (src/dft/fft-impl.hpp:1799-1841) fused into the store.
// ---------------------------------------------------------------------------------------------------
template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1) k_r2c(const real_args a, const int ts, const int spc)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ pass_desc sp[kMaxPasses];
    const F fft(sp, a.d, ts);
    cpx<T>* sm        = reinterpret_cast<cpx<T>*>(smem_raw);
    const int c       = fft.n;
    const int stride  = F::gstride(c);
    const long long s0 = (long long)blockIdx.x * spc;
    const T* __restrict__ inr      = reinterpret_cast<const T*>(a.in);
    cpx<T>* __restrict__ out       = reinterpret_cast<cpx<T>*>(a.out);
    const cpx<T>* __restrict__ rtw = reinterpret_cast<const cpx<T>*>(a.rtw);
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * c; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_n));
        const int e = i - s * c;
        const long long sig = s0 + s;
        if (sig < a.batch)
        {
            const T* xr = inr + sig * a.istride + 2 * e;
            // reals at an odd element offset (a pointer aligned to one real only) load one by one
            sm[s * stride + F::pi(e)] = (reinterpret_cast<uintptr_t>(xr) % sizeof(cpx<T>)) == 0
                                            ? *reinterpret_cast<const cpx<T>*>(xr)
                                            : mk<T>(xr[0], xr[1]);
        }
    }
    __syncthreads();
    const group_map gm(ts, spc);
    fft.run(sm + gm.g * stride, reinterpret_cast<const cpx<T>*>(a.tw), gm.lt);
    const int olen = a.ccs ? c + 1 : c;
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * olen; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_out));
        const int k = i - s * olen;
        const long long sig = s0 + s;
        if (sig >= a.batch)
            continue;
        const cpx<T>* z = sm + s * stride;
        cpx<T> v;
        if (k == 0)
        {
            const cpx<T> z0 = z[0];
            v = a.ccs ? mk<T>(z0.x + z0.y, 0) : mk<T>(z0.x + z0.y, z0.x - z0.y);
        }
        else if (k == c)
        {
            const cpx<T> z0 = z[0];
            v               = mk<T>(z0.x - z0.y, 0);
        }
        else
        {
            const cpx<T> zk  = z[F::pi(k)];
            const cpx<T> znk = conj(z[F::pi(c - k)]);
            const cpx<T> e   = scale(zk + znk, T(0.5));
            const cpx<T> o   = scale(mul_mi(zk - znk), T(0.5));
            v                = e + ldg(rtw + k) * o;
        }
        out[sig * a.ostride + k] = v;
    }
}

// ---------------------------------------------------------------------------------------------------
// Real forward DFT, contiguous batch, persistent and pipelined (compile-time c): tiles of `spc` signals (spc
// even, so that each tile's input, 2c reals per signal, and output, olen complex bins per signal, are whole
// 16-byte units).  Three tile buffers rotate: the input tile (bulk copy, then the passes' A buffer), the
// scratch tile (B) and the spare tile for the next tile's copy, issued after the first pass.  The passes
// leave Z, the c-point DFT of the reals viewed as complex values, in natural order in one of the two
// buffers; the split (to_fmt, src/dft/fft-impl.hpp:1799-1841) reads it and writes the tile's spectrum into
// the other, which one bulk copy stores.  The next tile's input is this one's spare, its scratch the Z
// buffer, its spare the buffer being stored.  Whole tiles only (the host runs the remainder with k_r2c).  A
// wait that runs out sets *err and the CTA returns.
// ---------------------------------------------------------------------------------------------------
template <typename T, class F>
__host__ __device__ constexpr int r2c_stage_elems(int spc)
{
    // the input tile (spc c complex), the padded work layout, the output tile (up to c + 1 bins per signal)
    const int a = spc * (F::n + 1), b = spc * F::gstride(F::n);
    return ((a > b ? a : b) + 15) / 16 * 16;
}

template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1)
    k_r2c_pipe(const real_args a, const long long ntiles, const int spc, int* err)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int C      = F::n;
    constexpr int STRIDE = F::gstride(C);
    const F fft(nullptr, a.d, F::ts);
    const int slen       = r2c_stage_elems<T, F>(spc);
    const int olen       = a.ccs ? C + 1 : C;
    cpx<T>* const tiles  = reinterpret_cast<cpx<T>*>(smem_raw);
    uint64_t* bars       = reinterpret_cast<uint64_t*>(tiles + 3 * slen);
    const uint32_t ibytes = uint32_t(spc) * uint32_t(C) * uint32_t(sizeof(cpx<T>));
    const uint32_t obytes = uint32_t(spc) * uint32_t(olen) * uint32_t(sizeof(cpx<T>));
    const cpx<T>* in     = reinterpret_cast<const cpx<T>*>(a.in);
    cpx<T>* out          = reinterpret_cast<cpx<T>*>(a.out);
    const cpx<T>* tw     = reinterpret_cast<const cpx<T>*>(a.tw);
    const cpx<T>* __restrict__ rtw = reinterpret_cast<const cpx<T>*>(a.rtw);
    const group_map gm(F::ts, spc);
    if (threadIdx.x == 0)
    {
        for (int b = 0; b < 3; b++)
            mbar_init(&bars[b], 1);
        mbar_fence_init();
    }
    __syncthreads();
    long long t = blockIdx.x;
    if (threadIdx.x == 0 && t < ntiles)
    {
        mbar_arrive_expect_tx(&bars[0], ibytes);
        bulk_g2s(tiles, in + t * spc * C, ibytes, &bars[0]);
    }
    uint32_t phase = 0;         // bit b: parity to wait for on tile buffer b
    int bi = 0, bs = 1, bn = 2; // input, scratch and spare tile buffers
    for (; t < ntiles; t += gridDim.x)
    {
        cpx<T>* in_t   = tiles + bi * slen;
        cpx<T>* scr_t  = tiles + bs * slen;
        const bool got = mbar_wait(&bars[bi], (phase >> bi) & 1, a.wait_spins);
        if (!__syncthreads_and(got))
        {
            if (threadIdx.x == 0)
            {
                atomicExch(err, 1);
                // the copy waited for is the only load in flight (the next one is issued after this wait):
                // give it a bounded chance to land in this CTA's shared memory before the CTA exits
                mbar_wait(&bars[bi], (phase >> bi) & 1);
                bulk_wait_all();
            }
            return;
        }
        phase ^= 1u << bi;
        const long long tn  = t + gridDim.x;
        const auto prefetch = [&]()
        {
            if (threadIdx.x == 0 && tn < ntiles)
            {
                // the spare buffer holds the previous tile's spectrum: wait until its bulk store has read it
                bulk_wait_read();
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(&bars[bn], ibytes);
                bulk_g2s(tiles + bn * slen, in + tn * spc * C, ibytes, &bars[bn]);
            }
        };
        // pass i writes B (i even) or A (i odd): with an odd pass count the last pass reads A
        constexpr bool odd = F::npass % 2 == 1;
        cpx<T>* zb         = odd ? scr_t : in_t; // Z in natural order
        cpx<T>* xb         = odd ? in_t : scr_t; // the tile's spectrum
        const cpx<T>* src  = in_t + gm.g * C;
        cpx<T>* zsig       = zb + gm.g * C;
        const auto nothing = []() {};
        fft.run_pp([&](int p) { return src[p]; }, [&](int q, cpx<T> x) { zsig[q] = x; }, prefetch, nothing,
                   in_t + gm.g * STRIDE, scr_t + gm.g * STRIDE, tw, gm.lt);
        // the split: bin k of signal s from Z[k] and Z[c - k]
        for (int i = threadIdx.x; i < spc * olen; i += blockDim.x)
        {
            const int s     = int(div_by(uint32_t(i), a.div_out));
            const int k     = i - s * olen;
            const cpx<T>* z = zb + s * C;
            cpx<T> v;
            if (k == 0)
            {
                const cpx<T> z0 = z[0];
                v = a.ccs ? mk<T>(z0.x + z0.y, 0) : mk<T>(z0.x + z0.y, z0.x - z0.y);
            }
            else if (k == C)
            {
                const cpx<T> z0 = z[0];
                v               = mk<T>(z0.x - z0.y, 0);
            }
            else
            {
                const cpx<T> zk  = z[k];
                const cpx<T> znk = conj(z[C - k]);
                const cpx<T> e   = scale(zk + znk, T(0.5));
                const cpx<T> o   = scale(mul_mi(zk - znk), T(0.5));
                v                = e + ldg(rtw + k) * o;
            }
            xb[i] = v;
        }
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0)
        {
            bulk_s2g(out + t * spc * olen, xb, obytes);
            bulk_commit();
        }
        const int zi = odd ? bs : bi, xi = odd ? bi : bs;
        bi = bn;
        bs = zi;
        bn = xi;
    }
    if (threadIdx.x == 0)
        bulk_wait_all();
}

// ---------------------------------------------------------------------------------------------------
// Real inverse DFT: the merge of from_fmt (src/dft/fft-impl.hpp:1852-1896) fused into the load, then an
// unscaled inverse c-point complex DFT whose output is the 2c reals.  Only the real parts of the DC and
// Nyquist bins are read, as in the reference.
// ---------------------------------------------------------------------------------------------------
template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1) k_c2r(const real_args a, const int ts, const int spc)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ pass_desc sp[kMaxPasses];
    const F fft(sp, a.d, ts);
    cpx<T>* sm        = reinterpret_cast<cpx<T>*>(smem_raw);
    const int c       = fft.n;
    const int stride  = F::gstride(c);
    const long long s0 = (long long)blockIdx.x * spc;
    const cpx<T>* __restrict__ in  = reinterpret_cast<const cpx<T>*>(a.in);
    T* __restrict__ outr           = reinterpret_cast<T*>(a.out);
    const cpx<T>* __restrict__ rtw = reinterpret_cast<const cpx<T>*>(a.rtw);
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * c; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_n));
        const int k = i - s * c;
        const long long sig = s0 + s;
        if (sig >= a.batch)
            continue;
        const cpx<T>* X = in + sig * a.istride;
        cpx<T> z;
        if (k == 0)
        {
            const T x0 = X[0].x;
            const T xn = a.ccs ? X[c].x : X[0].y;
            z          = mk<T>(x0 + xn, x0 - xn);
        }
        else
        {
            const cpx<T> xk  = X[k];
            const cpx<T> xnk = conj(X[c - k]);
            const cpx<T> f1  = xk + xnk;
            const cpx<T> f2  = xk - xnk;
            z                = f1 + mul_pi(conj(ldg(rtw + k)) * f2);
        }
        sm[s * stride + F::pi(k)] = conj(z);
    }
    __syncthreads();
    const group_map gm(ts, spc);
    fft.run(sm + gm.g * stride, reinterpret_cast<const cpx<T>*>(a.tw), gm.lt);
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * c; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_n));
        const int e = i - s * c;
        const long long sig = s0 + s;
        if (sig < a.batch)
        {
            T* yr          = outr + sig * a.ostride + 2 * e;
            const cpx<T> v = conj(sm[s * stride + F::pi(e)]);
            // reals at an odd element offset store one by one
            if ((reinterpret_cast<uintptr_t>(yr) % sizeof(cpx<T>)) == 0)
                *reinterpret_cast<cpx<T>*>(yr) = v;
            else
            {
                yr[0] = v.x;
                yr[1] = v.y;
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------------
// Real inverse DFT, contiguous batch, persistent and pipelined (compile-time c): tiles of `spc` signals (spc
// even: each tile's input, ilen complex bins per signal, and output, 2c reals per signal, are whole 16-byte
// units).  Three tile buffers rotate as in k_r2c_pipe: the input tile arrives by bulk copy; the merge
// (from_fmt, src/dft/fft-impl.hpp:1852-1896) writes conj(Z) in natural order into the scratch tile; the
// passes ping-pong between the scratch and input tiles, the last one writing the conjugated output (the 2c
// reals as c complex values) into the buffer it does not read, which one bulk copy stores.  The next tile's
// copy is issued after the first pass.  Whole tiles only (the host runs the remainder with k_c2r).  A wait
// that runs out sets *err and the CTA returns.
// ---------------------------------------------------------------------------------------------------
template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1)
    k_c2r_pipe(const real_args a, const long long ntiles, const int spc, int* err)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int C      = F::n;
    constexpr int STRIDE = F::gstride(C);
    const F fft(nullptr, a.d, F::ts);
    const int slen       = r2c_stage_elems<T, F>(spc);
    const int ilen       = a.ccs ? C + 1 : C;
    cpx<T>* const tiles  = reinterpret_cast<cpx<T>*>(smem_raw);
    uint64_t* bars       = reinterpret_cast<uint64_t*>(tiles + 3 * slen);
    const uint32_t ibytes = uint32_t(spc) * uint32_t(ilen) * uint32_t(sizeof(cpx<T>));
    const uint32_t obytes = uint32_t(spc) * uint32_t(C) * uint32_t(sizeof(cpx<T>));
    const cpx<T>* in     = reinterpret_cast<const cpx<T>*>(a.in);
    cpx<T>* out          = reinterpret_cast<cpx<T>*>(a.out);
    const cpx<T>* tw     = reinterpret_cast<const cpx<T>*>(a.tw);
    const cpx<T>* __restrict__ rtw = reinterpret_cast<const cpx<T>*>(a.rtw);
    const group_map gm(F::ts, spc);
    if (threadIdx.x == 0)
    {
        for (int b = 0; b < 3; b++)
            mbar_init(&bars[b], 1);
        mbar_fence_init();
    }
    __syncthreads();
    long long t = blockIdx.x;
    if (threadIdx.x == 0 && t < ntiles)
    {
        mbar_arrive_expect_tx(&bars[0], ibytes);
        bulk_g2s(tiles, in + t * spc * ilen, ibytes, &bars[0]);
    }
    uint32_t phase = 0;         // bit b: parity to wait for on tile buffer b
    int bi = 0, bs = 1, bn = 2; // input, scratch and spare tile buffers
    for (; t < ntiles; t += gridDim.x)
    {
        cpx<T>* in_t   = tiles + bi * slen;
        cpx<T>* scr_t  = tiles + bs * slen;
        const bool got = mbar_wait(&bars[bi], (phase >> bi) & 1, a.wait_spins);
        if (!__syncthreads_and(got))
        {
            if (threadIdx.x == 0)
            {
                atomicExch(err, 1);
                // the copy waited for is the only load in flight (the next one is issued after this wait):
                // give it a bounded chance to land in this CTA's shared memory before the CTA exits
                mbar_wait(&bars[bi], (phase >> bi) & 1);
                bulk_wait_all();
            }
            return;
        }
        phase ^= 1u << bi;
        // the merge: conj(Z[k]) of signal s from bins k and c - k
        for (int i = threadIdx.x; i < spc * C; i += blockDim.x)
        {
            const int s     = int(div_by(uint32_t(i), a.div_n));
            const int k     = i - s * C;
            const cpx<T>* X = in_t + s * ilen;
            cpx<T> z;
            if (k == 0)
            {
                const T x0 = X[0].x;
                const T xn = a.ccs ? X[C].x : X[0].y;
                z          = mk<T>(x0 + xn, x0 - xn);
            }
            else
            {
                const cpx<T> xk  = X[k];
                const cpx<T> xnk = conj(X[C - k]);
                z                = (xk + xnk) + mul_pi(conj(ldg(rtw + k)) * (xk - xnk));
            }
            scr_t[i] = conj(z);
        }
        __syncthreads();
        const long long tn  = t + gridDim.x;
        const auto prefetch = [&]()
        {
            if (threadIdx.x == 0 && tn < ntiles)
            {
                // the spare buffer holds the previous tile's output: wait until its bulk store has read it
                bulk_wait_read();
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(&bars[bn], ibytes);
                bulk_g2s(tiles + bn * slen, in + tn * spc * ilen, ibytes, &bars[bn]);
            }
        };
        // passes: A = scratch (holding conj(Z)), B = input tile; pass i writes B (i even) or A (i odd), so
        // with an odd pass count the last pass reads A and writes the output into the input tile
        constexpr bool odd = F::npass % 2 == 1;
        cpx<T>* ob         = odd ? in_t : scr_t;
        const cpx<T>* zsig = scr_t + gm.g * C;
        cpx<T>* osig       = ob + gm.g * C;
        const auto nothing = []() {};
        fft.run_pp([&](int p) { return zsig[p]; }, [&](int q, cpx<T> x) { osig[q] = conj(x); }, prefetch, nothing,
                   scr_t + gm.g * STRIDE, in_t + gm.g * STRIDE, tw, gm.lt);
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0)
        {
            bulk_s2g(out + t * spc * C, ob, obytes);
            bulk_commit();
        }
        const int oi = odd ? bi : bs, fi = odd ? bs : bi;
        bi = bn;
        bs = fi;
        bn = oi;
    }
    if (threadIdx.x == 0)
        bulk_wait_all();
}

// ---------------------------------------------------------------------------------------------------
// DCT-II (dct_plan::execute, include/kfr/dft/fft.hpp:938-950): even/odd mirror on load, n-point DFT,
// Re*cos + Im*sin on store.
// ---------------------------------------------------------------------------------------------------
template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1) k_dct2(const dct_args a, const int ts, const int spc)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ pass_desc sp[kMaxPasses];
    const F fft(sp, a.d, ts);
    cpx<T>* sm        = reinterpret_cast<cpx<T>*>(smem_raw);
    const int n       = fft.n;
    const int stride  = F::gstride(n);
    const long long s0 = (long long)blockIdx.x * spc;
    const T* __restrict__ in       = reinterpret_cast<const T*>(a.in);
    T* __restrict__ out            = reinterpret_cast<T*>(a.out);
    const cpx<T>* __restrict__ dtw = reinterpret_cast<const cpx<T>*>(a.dtw);
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * n; i += blockDim.x)
    {
        const int s   = int(div_by(uint32_t(i), a.div_n));
        const int src = i - s * n;
        const long long sig = s0 + s;
        if (sig >= a.batch)
            continue;
        const int pos = (src & 1) ? n - 1 - (src >> 1) : (src >> 1);
        sm[s * stride + F::pi(pos)] = mk<T>(in[sig * a.stride + src], T(0));
    }
    __syncthreads();
    const group_map gm(ts, spc);
    fft.run(sm + gm.g * stride, reinterpret_cast<const cpx<T>*>(a.tw), gm.lt);
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * n; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_n));
        const int k = i - s * n;
        const long long sig = s0 + s;
        if (sig >= a.batch)
            continue;
        const cpx<T> y = sm[s * stride + F::pi(k)];
        const cpx<T> w = ldg(dtw + k);
        out[sig * a.stride + k] = y.x * w.x + y.y * w.y;
    }
}

// DCT-III, the reference's "inverse" (include/kfr/dft/fft.hpp:951-969): x_k * e^{-i pi k / 2n}, X0 halved,
// forward n-point DFT, un-mirror the real parts.
template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1) k_dct3(const dct_args a, const int ts, const int spc)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ pass_desc sp[kMaxPasses];
    const F fft(sp, a.d, ts);
    cpx<T>* sm        = reinterpret_cast<cpx<T>*>(smem_raw);
    const int n       = fft.n;
    const int stride  = F::gstride(n);
    const long long s0 = (long long)blockIdx.x * spc;
    const T* __restrict__ in       = reinterpret_cast<const T*>(a.in);
    T* __restrict__ out            = reinterpret_cast<T*>(a.out);
    const cpx<T>* __restrict__ dtw = reinterpret_cast<const cpx<T>*>(a.dtw);
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * n; i += blockDim.x)
    {
        const int s = int(div_by(uint32_t(i), a.div_n));
        const int k = i - s * n;
        const long long sig = s0 + s;
        if (sig >= a.batch)
            continue;
        const T x      = in[sig * a.stride + k];
        const cpx<T> w = ldg(dtw + k);
        cpx<T> v       = mk<T>(x * w.x, -(x * w.y));
        if (k == 0)
            v = scale(v, T(0.5));
        sm[s * stride + F::pi(k)] = v;
    }
    __syncthreads();
    const group_map gm(ts, spc);
    fft.run(sm + gm.g * stride, reinterpret_cast<const cpx<T>*>(a.tw), gm.lt);
#pragma unroll 4
    for (int i = threadIdx.x; i < spc * n; i += blockDim.x)
    {
        const int s   = int(div_by(uint32_t(i), a.div_n));
        const int dst = i - s * n;
        const long long sig = s0 + s;
        if (sig >= a.batch)
            continue;
        const int pos = (dst & 1) ? n - 1 - (dst >> 1) : (dst >> 1);
        out[sig * a.stride + dst] = sm[s * stride + F::pi(pos)].x;
    }
}

// ---------------------------------------------------------------------------------------------------
// DCT-II / DCT-III, contiguous batch, persistent and pipelined (compile-time n): tiles of `spc` signals of n
// reals.  Three tile buffers rotate as in k_r2c_pipe: the input tile (bulk copy of spc n reals, then the
// passes' A buffer), the scratch tile (B) and the spare tile, into which the next tile's copy is issued
// after the first pass.  DCT-II (include/kfr/dft/fft.hpp:938-950): the first pass reads the even/odd mirror
// of the reals straight from the input tile, the last pass writes Re(V[k]) cos + Im(V[k]) sin as reals into
// the buffer it does not read.  DCT-III (fft.hpp:951-969): the first pass reads x[k] e^{-i pi k / 2n} (x[0]
// halved), the last pass un-mirrors the real parts.  One bulk copy stores the tile.  Whole tiles only (the
// host runs the remainder with k_dct2 / k_dct3).  A wait that runs out sets *err and the CTA returns.
// ---------------------------------------------------------------------------------------------------
template <typename T, class F>
__host__ __device__ constexpr int dct_stage_elems(int spc)
{
    // complex elements: the real tiles (spc n / 2) and the padded work layout
    const int a = spc * F::n / 2, b = spc * F::gstride(F::n);
    return ((a > b ? a : b) + 15) / 16 * 16;
}

template <typename T, class F, bool INV>
__global__ void __launch_bounds__(F::max_threads, 1)
    k_dct_pipe(const dct_args a, const long long ntiles, const int spc, int* err)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int N      = F::n;
    constexpr int STRIDE = F::gstride(N);
    const F fft(nullptr, a.d, F::ts);
    const int slen       = dct_stage_elems<T, F>(spc);
    cpx<T>* const tiles  = reinterpret_cast<cpx<T>*>(smem_raw);
    uint64_t* bars       = reinterpret_cast<uint64_t*>(tiles + 3 * slen);
    const uint32_t bytes = uint32_t(spc) * uint32_t(N) * uint32_t(sizeof(T));
    const T* in          = reinterpret_cast<const T*>(a.in);
    T* out               = reinterpret_cast<T*>(a.out);
    const cpx<T>* tw     = reinterpret_cast<const cpx<T>*>(a.tw);
    const cpx<T>* __restrict__ dtw = reinterpret_cast<const cpx<T>*>(a.dtw);
    const group_map gm(F::ts, spc);
    if (threadIdx.x == 0)
    {
        for (int b = 0; b < 3; b++)
            mbar_init(&bars[b], 1);
        mbar_fence_init();
    }
    __syncthreads();
    long long t = blockIdx.x;
    if (threadIdx.x == 0 && t < ntiles)
    {
        mbar_arrive_expect_tx(&bars[0], bytes);
        bulk_g2s(tiles, in + t * spc * N, bytes, &bars[0]);
    }
    uint32_t phase = 0;         // bit b: parity to wait for on tile buffer b
    int bi = 0, bs = 1, bn = 2; // input, scratch and spare tile buffers
    for (; t < ntiles; t += gridDim.x)
    {
        cpx<T>* in_t   = tiles + bi * slen;
        cpx<T>* scr_t  = tiles + bs * slen;
        const bool got = mbar_wait(&bars[bi], (phase >> bi) & 1, a.wait_spins);
        if (!__syncthreads_and(got))
        {
            if (threadIdx.x == 0)
            {
                atomicExch(err, 1);
                // the copy waited for is the only load in flight (the next one is issued after this wait):
                // give it a bounded chance to land in this CTA's shared memory before the CTA exits
                mbar_wait(&bars[bi], (phase >> bi) & 1);
                bulk_wait_all();
            }
            return;
        }
        phase ^= 1u << bi;
        const long long tn  = t + gridDim.x;
        const auto prefetch = [&]()
        {
            if (threadIdx.x == 0 && tn < ntiles)
            {
                // the spare buffer holds the previous tile's output: wait until its bulk store has read it
                bulk_wait_read();
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(&bars[bn], bytes);
                bulk_g2s(tiles + bn * slen, in + tn * spc * N, bytes, &bars[bn]);
            }
        };
        // pass i writes B (i even) or A (i odd): with an odd pass count the last pass reads A and writes B
        constexpr bool odd = F::npass % 2 == 1;
        T* ob              = reinterpret_cast<T*>(odd ? scr_t : in_t);
        const T* xs        = reinterpret_cast<const T*>(in_t) + gm.g * N;
        T* os              = ob + gm.g * N;
        const auto nothing = []() {};
        if constexpr (!INV)
            fft.run_pp(
                [&](int p)
                {
                    const int i = p < N / 2 ? 2 * p : 2 * (N - 1 - p) + 1;
                    return mk<T>(xs[i], T(0));
                },
                [&](int q, cpx<T> x)
                {
                    const cpx<T> w = ldg(dtw + q);
                    os[q]          = x.x * w.x + x.y * w.y;
                },
                prefetch, nothing, in_t + gm.g * STRIDE, scr_t + gm.g * STRIDE, tw, gm.lt);
        else
            fft.run_pp(
                [&](int p)
                {
                    const T x      = xs[p];
                    const cpx<T> w = ldg(dtw + p);
                    const cpx<T> v = mk<T>(x * w.x, -(x * w.y));
                    return p == 0 ? scale(v, T(0.5)) : v;
                },
                [&](int q, cpx<T> x) { os[q < N / 2 ? 2 * q : 2 * (N - 1 - q) + 1] = x.x; }, prefetch, nothing,
                in_t + gm.g * STRIDE, scr_t + gm.g * STRIDE, tw, gm.lt);
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0)
        {
            bulk_s2g(out + t * spc * N, ob, bytes);
            bulk_commit();
        }
        // next: input = spare, scratch = the buffer the last pass read, spare = the buffer being stored
        const int oi = odd ? bs : bi, ri = odd ? bi : bs;
        bi = bn;
        bs = ri;
        bn = oi;
    }
    if (threadIdx.x == 0)
        bulk_wait_all();
}

// ---------------------------------------------------------------------------------------------------
// Four-step passes for lengths beyond one CTA (N = n1 * n2).  grid = (tiles, batch).
// ---------------------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ cpx<T> twiddle_2level(const cpx<T>* __restrict__ A, const cpx<T>* __restrict__ B,
                                                 long long m, int lbits)
{
    return ldg(A + (m >> lbits)) * ldg(B + (m & ((1LL << lbits) - 1)));
}

template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1) k_fs_cols(const fourstep_args a, const int ts)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ pass_desc sp[kMaxPasses];
    const F fft(sp, a.d, ts);
    cpx<T>* sm       = reinterpret_cast<cpx<T>*>(smem_raw);
    const int n1     = fft.n, n2 = a.n2, S = a.tile, sh = a.tile_shift;
    const int stride = F::gstride(n1);
    const int c0     = blockIdx.x * S;
    const long long sig = blockIdx.y;
    const cpx<T>* __restrict__ x = reinterpret_cast<const cpx<T>*>(a.in) + sig * a.sig_stride;
    cpx<T>* __restrict__ y       = reinterpret_cast<cpx<T>*>(a.out) + sig * a.sig_stride;
    const bool cin  = a.conj_in != 0;
    const int total = S * n1;
    copy_batched<8>(
        total,
        [&](int i)
        {
            const int n1i = i >> sh; // S is a power of two
            const int c   = i & (S - 1);
            return c0 + c < n2 ? x[(long long)n1i * n2 + c0 + c] : mk<T>(0, 0);
        },
        [&](int i, cpx<T> v)
        {
            const int n1i = i >> sh;
            const int c   = i & (S - 1);
            sm[c * stride + F::pi(n1i)] = conj_if(v, cin);
        });
    __syncthreads();
    const group_map gm(ts, S);
    const cpx<T>* twA = reinterpret_cast<const cpx<T>*>(a.twA);
    const cpx<T>* twB = reinterpret_cast<const cpx<T>*>(a.twB);
    if constexpr (F::compile_time)
    {
        if (a.pingpong && !a.same_layout)
        {
            // ping-pong passes with a second buffer after the tile; the last pass applies W_N^{col k1} and
            // stores the column contiguously (stride one across a signal's threads)
            const int col      = c0 + gm.g;
            const bool cout    = a.conj_out != 0;
            const auto nothing = []() {};
            fft.run_pp([&](int p) { return sm[gm.g * stride + F::pi(p)]; },
                       [&](int k1, cpx<T> v)
                       {
                           if (col < n2)
                               y[(long long)col * n1 + k1] =
                                   conj_if(v * twiddle_2level(twA, twB, (long long)col * k1, a.lbits), cout);
                       },
                       nothing, nothing, sm + gm.g * stride, sm + (S + gm.g) * stride,
                       reinterpret_cast<const cpx<T>*>(a.tw), gm.lt);
            return;
        }
    }
    fft.run(sm + gm.g * stride, reinterpret_cast<const cpx<T>*>(a.tw), gm.lt);
    if (a.same_layout)
    {
        // an axis of a multi-dimensional transform: no twiddle, back to the input's own layout
#pragma unroll 4
        for (int i = threadIdx.x; i < total; i += blockDim.x)
        {
            const int k1 = i >> sh;
            const int c  = i & (S - 1);
            if (c0 + c < n2)
                y[(long long)k1 * n2 + c0 + c] = conj_if(sm[c * stride + F::pi(k1)], a.conj_out != 0);
        }
        return;
    }
#pragma unroll 4
    for (int i = threadIdx.x; i < total; i += blockDim.x)
    {
        const int c  = int(div_by(uint32_t(i), a.div_n));
        const int k1 = i - c * n1;
        const int col = c0 + c;
        if (col < n2)
        {
            cpx<T> v = sm[c * stride + F::pi(k1)];
            v        = v * twiddle_2level(twA, twB, (long long)col * k1, a.lbits);
            y[(long long)col * n1 + k1] = conj_if(v, a.conj_out != 0);
        }
    }
}

template <typename T, class F>
__global__ void __launch_bounds__(F::max_threads, 1) k_fs_rows(const fourstep_args a, const int ts)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ pass_desc sp[kMaxPasses];
    const F fft(sp, a.d, ts);
    cpx<T>* sm       = reinterpret_cast<cpx<T>*>(smem_raw);
    const int n1     = a.n1, n2 = fft.n, S = a.tile, sh = a.tile_shift;
    const int stride = F::gstride(n2);
    const int r0     = blockIdx.x * S;
    const long long sig = blockIdx.y;
    const cpx<T>* __restrict__ y = reinterpret_cast<const cpx<T>*>(a.in) + sig * a.sig_stride;
    cpx<T>* __restrict__ X       = reinterpret_cast<cpx<T>*>(a.out) + sig * a.sig_stride;
    const int total = S * n2;
    const bool cin  = a.conj_in != 0;
    copy_batched<8>(
        total,
        [&](int i)
        {
            const int n2i = i >> sh;
            const int r   = i & (S - 1);
            return r0 + r < n1 ? y[(long long)n2i * n1 + r0 + r] : mk<T>(0, 0);
        },
        [&](int i, cpx<T> v)
        {
            const int n2i = i >> sh;
            const int r   = i & (S - 1);
            sm[r * stride + F::pi(n2i)] = conj_if(v, cin);
        });
    __syncthreads();
    const group_map gm(ts, S);
    const bool cout = a.conj_out != 0;
    if constexpr (F::compile_time)
    {
        if (a.pingpong)
        {
            // ping-pong passes with a second buffer after the tile; the last pass stages its output as
            // [k2][row] (rows XOR-swizzled by k2) in the buffer it does not read, for row-contiguous stores
            cpx<T>* B          = sm + S * stride;
            cpx<T>* stg        = F::npass % 2 == 0 ? sm : B;
            const auto nothing = []() {};
            fft.run_pp([&](int p) { return sm[gm.g * stride + F::pi(p)]; },
                       [&](int k2, cpx<T> v) { stg[k2 * S + (gm.g ^ (k2 & (S - 1)))] = v; }, nothing, nothing,
                       sm + gm.g * stride, B + gm.g * stride, reinterpret_cast<const cpx<T>*>(a.tw), gm.lt);
#pragma unroll 4
            for (int i = threadIdx.x; i < total; i += blockDim.x)
            {
                const int k2 = i >> sh;
                const int r  = i & (S - 1);
                if (r0 + r < n1)
                    X[(long long)(r0 + r) + (long long)n1 * k2] = conj_if(stg[k2 * S + (r ^ (k2 & (S - 1)))], cout);
            }
            return;
        }
    }
    fft.run(sm + gm.g * stride, reinterpret_cast<const cpx<T>*>(a.tw), gm.lt);
#pragma unroll 4
    for (int i = threadIdx.x; i < total; i += blockDim.x)
    {
        const int k2 = i >> sh;
        const int r  = i & (S - 1);
        if (r0 + r < n1)
            X[(long long)(r0 + r) + (long long)n1 * k2] = conj_if(sm[r * stride + F::pi(k2)], cout);
    }
}

// ---------------------------------------------------------------------------------------------------
// Four-step passes with both lengths, the tile and the twiddle split known at compile time (KFR_CT_FSPAIR):
// the same work as the ping-pong branches of k_fs_cols / k_fs_rows with every index folded to constants.
// ---------------------------------------------------------------------------------------------------
template <int N>
__host__ __device__ constexpr int lbits_for()
{
    int lb = 0;
    while ((1LL << (2 * lb)) < (long long)N)
        lb++;
    return lb;
}

template <typename T, class FA, int N2>
__global__ void __launch_bounds__(1024, 1) k_fsp_cols(const fourstep_args a)
{
    constexpr int N1 = FA::n, GA = FA::gstride(), TS = FA::ts;
    constexpr int S  = fsp_tile(N1, TS, kFspSmem), SH = S == 16 ? 4 : 3;
    constexpr long long N = (long long)N1 * N2;
    constexpr int LB      = lbits_for<N1 * N2>();
    static_assert(S >= 8, "pair kernels need a tile of at least 8");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<T>* sm      = reinterpret_cast<cpx<T>*>(smem_raw);
    const int c0    = blockIdx.x * S;
    const cpx<T>* __restrict__ x = reinterpret_cast<const cpx<T>*>(a.in) + blockIdx.y * N;
    cpx<T>* __restrict__ y       = reinterpret_cast<cpx<T>*>(a.out) + blockIdx.y * N;
    const bool cin = a.conj_in != 0, cout = a.conj_out != 0;
    copy_batched<8>(
        S * N1,
        [&](int i)
        {
            const int c = i & (S - 1);
            return (N2 % S == 0 || c0 + c < N2) ? x[(i >> SH) * N2 + c0 + c] : mk<T>(0, 0);
        },
        [&](int i, cpx<T> v) { sm[(i & (S - 1)) * GA + FA::pi(i >> SH)] = conj_if(v, cin); });
    __syncthreads();
    const int g  = int(threadIdx.x) / TS;
    const int lt = g < S ? int(threadIdx.x) - g * TS : TS;
    const int gg = g < S ? g : 0;
    const int col = c0 + gg;
    const cpx<T>* twA  = reinterpret_cast<const cpx<T>*>(a.twA);
    const cpx<T>* twB  = reinterpret_cast<const cpx<T>*>(a.twB);
    const auto nothing = []() {};
    const FA fa(nullptr, a.d, TS);
    fa.run_pp([&](int p) { return sm[gg * GA + FA::pi(p)]; },
              [&](int k1, cpx<T> v)
              {
                  if (N2 % S == 0 || col < N2)
                      y[col * N1 + k1] = conj_if(v * twiddle_2level(twA, twB, (long long)(col * k1), LB), cout);
              },
              nothing, nothing, sm + gg * GA, sm + (S + gg) * GA, reinterpret_cast<const cpx<T>*>(a.tw), lt);
}

template <typename T, class FB, int N1>
__global__ void __launch_bounds__(1024, 1) k_fsp_rows(const fourstep_args a)
{
    constexpr int N2 = FB::n, GB = FB::gstride(), TS = FB::ts;
    constexpr int S  = fsp_tile(N2, TS, kFspSmem), SH = S == 16 ? 4 : 3;
    constexpr long long N = (long long)N1 * N2;
    static_assert(S >= 8, "pair kernels need a tile of at least 8");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<T>* sm      = reinterpret_cast<cpx<T>*>(smem_raw);
    const int r0    = blockIdx.x * S;
    const cpx<T>* __restrict__ y = reinterpret_cast<const cpx<T>*>(a.in) + blockIdx.y * N;
    cpx<T>* __restrict__ X       = reinterpret_cast<cpx<T>*>(a.out) + blockIdx.y * N;
    const bool cin = a.conj_in != 0, cout = a.conj_out != 0;
    copy_batched<8>(
        S * N2,
        [&](int i)
        {
            const int r = i & (S - 1);
            return (N1 % S == 0 || r0 + r < N1) ? y[(i >> SH) * N1 + r0 + r] : mk<T>(0, 0);
        },
        [&](int i, cpx<T> v) { sm[(i & (S - 1)) * GB + FB::pi(i >> SH)] = conj_if(v, cin); });
    __syncthreads();
    const int g  = int(threadIdx.x) / TS;
    const int lt = g < S ? int(threadIdx.x) - g * TS : TS;
    const int gg = g < S ? g : 0;
    cpx<T>* B          = sm + S * GB;
    cpx<T>* stg        = FB::npass % 2 == 0 ? sm : B;
    const auto nothing = []() {};
    const FB fb(nullptr, a.d, TS);
    fb.run_pp([&](int p) { return sm[gg * GB + FB::pi(p)]; },
              [&](int k2, cpx<T> v) { stg[k2 * S + (gg ^ (k2 & (S - 1)))] = v; }, nothing, nothing, sm + gg * GB,
              B + gg * GB, reinterpret_cast<const cpx<T>*>(a.tw), lt);
#pragma unroll 4
    for (int i = threadIdx.x; i < S * N2; i += blockDim.x)
    {
        const int k2 = i >> SH, r = i & (S - 1);
        if (N1 % S == 0 || r0 + r < N1)
            X[(r0 + r) + N1 * k2] = conj_if(stg[k2 * S + (r ^ (k2 & (S - 1)))], cout);
    }
}

// ---------------------------------------------------------------------------------------------------
// Four-step pair kernels, persistent, with 2-D tensor copies (TMA).  Same transforms as k_fsp_cols /
// k_fsp_rows for lengths of two or three passes: a tile is S columns (rows) of the signal, S = 16, 8, 4 or 2
// contiguous 8-byte elements (128 to 16 bytes) per row, loaded as one box per 256 rows with the matching
// swizzle (128, 64, 32 bytes; none for 16) and double buffered: the next tile streams in while the CTA
// transforms the current one.  Waits are bounded; one that runs out sets *err and the CTA returns.
//   column pass: the four-step twiddle per butterfly of the last pass; two passes: the tile's S output
//     columns (contiguous in the intermediate) are written over the box and stored by one bulk copy; three
//     passes (the box is the ping-pong A buffer): stored straight from the last pass;
//   row pass: two passes: the output is written back into the swizzled box and stored by tensor copies;
//     three passes: threads are ordered row-fastest, so the last pass stores S consecutive outputs per
//     column index straight to global memory.
//   in map (columns): x viewed as (2 N2 floats) x (N1 * batch) rows, box (2 S floats, min(N1, 256))
//   in / out maps (rows): y and X viewed as (2 N1 floats) x (N2 * batch) rows, box (2 S floats, min(N2, 256))
// ---------------------------------------------------------------------------------------------------
template <class F>
__host__ __device__ constexpr int fspt_stage_elems(int S)
{
    // the box, or (three passes) the padded A buffer of S signals, rounded to 1024 bytes
    const int e = F::npass == 3 && S * F::gstride() > S * F::n ? S * F::gstride() : S * F::n;
    return (e * 8 + 1023) / 1024 * 128;
}

// shared memory of a tensor-copy pair kernel: two stage tiles, the B buffer, two mbarriers, alignment slack
template <class F>
__host__ __device__ constexpr int fspt_smem_s(int S)
{
    return 2 * fspt_stage_elems<F>(S) * 8 + S * F::gstride() * 8 + 16 + 1024;
}

// tile width: the widest of 16, 8, 4 and 2 whose threads and shared memory fit (0: none)
template <class F>
__host__ __device__ constexpr int fspt_tile()
{
    if (!(F::npass == 2 || F::npass == 3) || !(F::n <= 256 || F::n % 256 == 0))
        return 0;
    for (int S = 16; S >= 2; S /= 2)
        if (S * F::ts <= 1024 && fspt_smem_s<F>(S) <= kFspSmem)
            return S;
    return 0;
}

template <class F>
__host__ __device__ constexpr bool fspt_ok()
{
    return fspt_tile<F>() != 0;
}

template <class F>
__host__ __device__ constexpr int fspt_smem()
{
    return fspt_smem_s<F>(fspt_tile<F>());
}

template <class F>
__host__ __device__ constexpr int fspt_threads()
{
    return fspt_tile<F>() * F::ts;
}

// CTAs per SM the launch bound asks registers for: three small CTAs, or one of up to 1024 threads
template <class F>
__host__ __device__ constexpr int fspt_min_ctas()
{
    return fspt_threads<F>() <= 256 ? 3 : 1;
}

// loads the S x N box of tile coordinates (x floats, y0 rows) as boxes of at most 256 rows
template <int S, int N>
__device__ __forceinline__ void fspt_load(void* dst, const tensor_map* tm, int x, int y0, uint64_t* bar)
{
    constexpr int BR = N < 256 ? N : 256;
    mbar_arrive_expect_tx(bar, uint32_t(S * N * 8));
#pragma unroll 1
    for (int b = 0; b < N / BR; b++)
        tensor_g2s_2d(static_cast<char*>(dst) + b * BR * S * 8, tm, x, y0 + b * BR, bar);
}

// Position of column output k1 in the real-fused layout (RP): k1 and N1 - k1 side by side at 2j and 2j + 1
// (j = min(k1, N1 - k1) >= 1), row 0 at 0, row N1/2 (N1 even) at 1; N1 odd leaves position 1 unused.
template <int N1>
__device__ __forceinline__ int rp_pos(int k1)
{
    return k1 == 0 ? 0 : (2 * k1 < N1 ? 2 * k1 : (2 * k1 == N1 ? 1 : 2 * (N1 - k1) + 1));
}

template <typename T, class FA, int N2, bool RP = false>
__global__ void __launch_bounds__(fspt_threads<FA>(), fspt_min_ctas<FA>())
    k_fspt_cols(const fourstep_args a, const __grid_constant__ tensor_map tm_in, const long long ntiles, int* err)
{
    static_assert(fspt_ok<FA>(), "two or three passes on tiles of 16 to 2 columns");
    constexpr int N1 = FA::n, GA = FA::gstride(), TS = FA::ts, S = fspt_tile<FA>();
    // RP: the real-fused layout, columns P1 apart (N1 rounded up to even) with outputs at rp_pos(k1)
    constexpr int P1 = RP ? N1 + (N1 & 1) : N1;
    const auto pos   = [](int k1) { return RP ? rp_pos<N1>(k1) : k1; };
    constexpr int NTC = (N2 + S - 1) / S;
    constexpr int SE  = fspt_stage_elems<FA>(S);
    constexpr int LB  = lbits_for<N1 * N2>();
    constexpr int NSL = N1 / FA::rlast; // last pass: butterfly j makes outputs j + r NSL
    constexpr bool three = FA::npass == 3;
    static_assert(three || (P1 * 8) % 16 == 0, "whole columns are bulk-copied");
    static_assert(three || S * P1 <= SE, "the tile's output columns fit the stage");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<T>* st0    = reinterpret_cast<cpx<T>*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    cpx<T>* B      = st0 + 2 * SE;
    uint64_t* bars = reinterpret_cast<uint64_t*>(B + S * GA);
    const bool cin = a.conj_in != 0, cout = a.conj_out != 0;
    const int g    = int(threadIdx.x) / TS;
    const int lt   = int(threadIdx.x) - g * TS;
    const cpx<T>* twA = reinterpret_cast<const cpx<T>*>(a.twA);
    const cpx<T>* twB = reinterpret_cast<const cpx<T>*>(a.twB);
    const cpx<T>* tw  = reinterpret_cast<const cpx<T>*>(a.tw);
    const FA fa(nullptr, a.d, TS);
    if (threadIdx.x == 0)
    {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    long long t = blockIdx.x;
    if (threadIdx.x == 0 && t < ntiles)
        fspt_load<S, N1>(st0, &tm_in, int(t % NTC) * 2 * S, int(t / NTC) * N1, &bars[0]);
    for (int it = 0; t < ntiles; t += gridDim.x, it++)
    {
        const int s    = it & 1;
        cpx<T>* stage  = st0 + s * SE;
        const bool got = mbar_wait(&bars[s], (it >> 1) & 1, a.wait_spins);
        if (!__syncthreads_and(got))
        {
            if (threadIdx.x == 0)
            {
                atomicExch(err, 1);
                // the copy waited for is the only load in flight (the next one is issued after this wait):
                // give it a bounded chance to land before the CTA exits
                mbar_wait(&bars[s], (it >> 1) & 1);
                bulk_wait_all();
            }
            return;
        }
        const long long tn = t + gridDim.x;
        if (threadIdx.x == 0 && tn < ntiles)
        {
            // the other stage holds the previous tile's output (or its A buffer): once its bulk store, if
            // any, has read it, stream the next tile in
            bulk_wait_read();
            fence_proxy_async_smem();
            fspt_load<S, N1>(st0 + (s ^ 1) * SE, &tm_in, int(tn % NTC) * 2 * S, int(tn / NTC) * N1, &bars[s ^ 1]);
        }
        const long long b = t / NTC;
        const int c0      = int(t % NTC) * S;
        const int col     = c0 + g;
        cpx<T>* y         = reinterpret_cast<cpx<T>*>(a.out) + b * (long long)P1 * N2;
        // four-step twiddle W_N^{col k1} on the last pass's outputs k1 = j + r NSL: W_N^{col j} times powers
        // of the tile's step W_N^{col NSL}
        const cpx<T> step = twiddle_2level(twA, twB, (long long)(col * NSL), LB);
        const auto post   = [&](int j, auto& o)
        {
            twiddle_powers<T, FA::rlast>(o, step);
            const cpx<T> w = twiddle_2level(twA, twB, (long long)(col * j), LB);
#pragma unroll
            for (int r = 0; r < FA::rlast; r++)
                o[r] = o[r] * w;
        };
        const auto ld = [&](int p) { return conj_if(stage[swz_8b<S>(p, g)], cin); };
        if constexpr (three)
        {
            // the box (consumed by pass 1) is the A buffer of pass 2; the last pass stores to global memory
            fa.run_pp_post(ld, post,
                           [&](int k1, cpx<T> v)
                           {
                               if (N2 % S == 0 || col < N2)
                                   y[(long long)col * P1 + pos(k1)] = conj_if(v, cout);
                           },
                           stage + g * GA, B + g * GA, tw, lt);
        }
        else
        {
            // pass 1 reads the box; pass 2 writes the tile's S output columns (contiguous in y) over it
            fa.run_pp_post(ld, post, [&](int k1, cpx<T> v) { stage[g * P1 + pos(k1)] = conj_if(v, cout); }, stage,
                           B + g * GA, tw, lt);
            fence_proxy_async_smem();
            __syncthreads();
            if (threadIdx.x == 0)
            {
                const int ncols = N2 % S == 0 ? S : (N2 - c0 < S ? N2 - c0 : S);
                bulk_s2g(y + (long long)c0 * P1, stage, uint32_t(ncols * P1 * 8));
                bulk_commit();
            }
        }
    }
    if (threadIdx.x == 0)
        bulk_wait_all();
}

template <typename T, class FB, int N1>
__global__ void __launch_bounds__(fspt_threads<FB>(), fspt_min_ctas<FB>())
    k_fspt_rows(const fourstep_args a, const __grid_constant__ tensor_map tm_in,
                const __grid_constant__ tensor_map tm_out, const long long ntiles, int* err)
{
    static_assert(fspt_ok<FB>(), "two or three passes on tiles of 16 to 2 rows");
    constexpr int N2 = FB::n, GB = FB::gstride(), TS = FB::ts, S = fspt_tile<FB>();
    constexpr int NTR = (N1 + S - 1) / S;
    constexpr int SE  = fspt_stage_elems<FB>(S);
    constexpr int BR  = N2 < 256 ? N2 : 256;
    constexpr bool three = FB::npass == 3;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<T>* st0    = reinterpret_cast<cpx<T>*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    cpx<T>* B      = st0 + 2 * SE;
    uint64_t* bars = reinterpret_cast<uint64_t*>(B + S * GB);
    const bool cin = a.conj_in != 0, cout = a.conj_out != 0;
    // two passes: the S threads' groups are contiguous (each row's TS threads together); three passes: rows
    // fastest, so that a warp's last-pass stores cover S consecutive outputs
    const int g  = three ? int(threadIdx.x) % S : int(threadIdx.x) / TS;
    const int lt = three ? int(threadIdx.x) / S : int(threadIdx.x) - g * TS;
    const cpx<T>* tw = reinterpret_cast<const cpx<T>*>(a.tw);
    const auto nothing = []() {};
    const FB fb(nullptr, a.d, TS);
    if (threadIdx.x == 0)
    {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    long long t = blockIdx.x;
    if (threadIdx.x == 0 && t < ntiles)
        fspt_load<S, N2>(st0, &tm_in, int(t % NTR) * 2 * S, int(t / NTR) * N2, &bars[0]);
    for (int it = 0; t < ntiles; t += gridDim.x, it++)
    {
        const int s    = it & 1;
        cpx<T>* stage  = st0 + s * SE;
        const bool got = mbar_wait(&bars[s], (it >> 1) & 1, a.wait_spins);
        if (!__syncthreads_and(got))
        {
            if (threadIdx.x == 0)
            {
                atomicExch(err, 1);
                // the copy waited for is the only load in flight (the next one is issued after this wait):
                // give it a bounded chance to land before the CTA exits
                mbar_wait(&bars[s], (it >> 1) & 1);
                bulk_wait_all();
            }
            return;
        }
        const long long tn = t + gridDim.x;
        if (threadIdx.x == 0 && tn < ntiles)
        {
            // the other stage holds the previous tile's output (or its A buffer): once its store, if any, has
            // read it, stream the next tile in
            bulk_wait_read();
            fence_proxy_async_smem();
            fspt_load<S, N2>(st0 + (s ^ 1) * SE, &tm_in, int(tn % NTR) * 2 * S, int(tn / NTR) * N2, &bars[s ^ 1]);
        }
        const auto ld = [&](int p) { return conj_if(stage[swz_8b<S>(p, g)], cin); };
        if constexpr (three)
        {
            const long long b = t / NTR;
            const int r       = int(t % NTR) * S + g;
            cpx<T>* X         = reinterpret_cast<cpx<T>*>(a.out) + b * (long long)N1 * N2;
            fb.run_pp(ld,
                      [&](int k2, cpx<T> v)
                      {
                          if (N1 % S == 0 || r < N1)
                              X[r + (long long)N1 * k2] = conj_if(v, cout);
                      },
                      nothing, nothing, stage + g * GB, B + g * GB, tw, lt);
        }
        else
        {
            // pass 1 reads the box, pass 2 writes the transformed rows back into it (same swizzled layout)
            fb.run_pp(ld, [&](int k2, cpx<T> v) { stage[swz_8b<S>(k2, g)] = conj_if(v, cout); }, nothing, nothing,
                      stage, B + g * GB, tw, lt);
            fence_proxy_async_smem();
            __syncthreads();
            if (threadIdx.x == 0)
            {
#pragma unroll 1
                for (int bx = 0; bx < N2 / BR; bx++)
                    tensor_s2g_2d(&tm_out, int(t % NTR) * 2 * S, int(t / NTR) * N2 + bx * BR, stage + bx * BR * S);
                bulk_commit();
            }
        }
    }
    if (threadIdx.x == 0)
        bulk_wait_all();
}

// The row pass of a real forward DFT on the real-fused column layout (k_fspt_cols with RP): a tile is S
// positions of the P1 per column, that is S/2 mirror pairs of rows k1 and N1 - k1 (or rows 0 and N1/2), so
// after the row FFTs Z[k] and Z[c - k] (c = N1 N2) of every output lie in the same tile and the split
//   X[k] = (Z[k] + conj Z[c-k]) / 2 - i W_2c^k (Z[k] - conj Z[c-k]) / 2
// writes the real spectrum directly: X[k] for row k1 at k2 and X[c - k] for row N1 - k1 at N2 - 1 - k2.
// Two passes only (the row FFT writes back into the box, the split reads it).
template <typename T, class FB, int N1>
__global__ void __launch_bounds__(fspt_threads<FB>(), fspt_min_ctas<FB>())
    k_fspt_rows_r2c(const fourstep_args a, const __grid_constant__ tensor_map tm_in, const long long ntiles, int* err)
{
    static_assert(fspt_ok<FB>() && FB::npass == 2, "two passes on tiles of 16 to 2 rows");
    constexpr int N2 = FB::n, GB = FB::gstride(), TS = FB::ts, S = fspt_tile<FB>();
    static_assert(S % 2 == 0, "whole mirror pairs per tile");
    constexpr int P1  = N1 + (N1 & 1);
    constexpr int NTR = (P1 + S - 1) / S;
    constexpr int SE  = fspt_stage_elems<FB>(S);
    constexpr int THREADS = fspt_threads<FB>();
    constexpr long long C = (long long)N1 * N2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cpx<T>* st0    = reinterpret_cast<cpx<T>*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    cpx<T>* B      = st0 + 2 * SE;
    uint64_t* bars = reinterpret_cast<uint64_t*>(B + S * GB);
    const int g    = int(threadIdx.x) / TS;
    const int lt   = int(threadIdx.x) - g * TS;
    const cpx<T>* tw  = reinterpret_cast<const cpx<T>*>(a.tw);
    // W_2c^k for k = k1 + N1 k2 as W_2c^k1 (rtw[k1]) times W_2c^(N1 k2) (rtw[N1 + k2]); W_2c^(c - k) is
    // -conj(W_2c^k)
    const cpx<T>* rtw = reinterpret_cast<const cpx<T>*>(a.rtw);
    const bool ccs    = a.ccs != 0;
    const long long olen = ccs ? C + 1 : C;
    const auto nothing = []() {};
    const FB fb(nullptr, a.d, TS);
    // X[k] from Z[k] = u and Z[c - k] = v, w = W_2c^k
    const auto split = [](cpx<T> u, cpx<T> v, cpx<T> w)
    { return scale(u + conj(v), T(0.5)) + w * scale(mul_mi(u - conj(v)), T(0.5)); };
    const auto mirror = [](cpx<T> w) { return mk<T>(-w.x, w.y); }; // W_2c^(c - k) = -conj(W_2c^k)
    if (threadIdx.x == 0)
    {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    long long t = blockIdx.x;
    if (threadIdx.x == 0 && t < ntiles)
        fspt_load<S, N2>(st0, &tm_in, int(t % NTR) * 2 * S, int(t / NTR) * N2, &bars[0]);
    for (int it = 0; t < ntiles; t += gridDim.x, it++)
    {
        const int s    = it & 1;
        cpx<T>* stage  = st0 + s * SE;
        const bool got = mbar_wait(&bars[s], (it >> 1) & 1, a.wait_spins);
        if (!__syncthreads_and(got))
        {
            if (threadIdx.x == 0)
            {
                atomicExch(err, 1);
                // the copy waited for is the only load in flight (the next one is issued after this wait):
                // give it a bounded chance to land before the CTA exits
                mbar_wait(&bars[s], (it >> 1) & 1);
            }
            return;
        }
        const long long tn = t + gridDim.x;
        if (threadIdx.x == 0 && tn < ntiles)
        {
            // the other stage was last read by the previous tile's split, before this tile's first barrier
            fence_proxy_async_smem();
            fspt_load<S, N2>(st0 + (s ^ 1) * SE, &tm_in, int(tn % NTR) * 2 * S, int(tn / NTR) * N2, &bars[s ^ 1]);
        }
        // pass 1 reads the box, pass 2 writes the transformed rows back into it (same swizzled layout)
        fb.run_pp([&](int p) { return stage[swz_8b<S>(p, g)]; },
                  [&](int k2, cpx<T> v) { stage[swz_8b<S>(k2, g)] = v; }, nothing, nothing, stage, B + g * GB, tw, lt);
        // run_pp ends with a barrier: every row of the tile is transformed
        const long long b = t / NTR;
        const int pb      = int(t % NTR) * S;
        cpx<T>* X         = reinterpret_cast<cpx<T>*>(a.out) + b * olen;
        for (int i = threadIdx.x; i < (S / 2) * N2; i += THREADS)
        {
            const int q = i % (S / 2), k2 = i / (S / 2);
            const int p0 = pb + 2 * q; // even position: rows p0 / 2 and N1 - p0 / 2, or rows 0 and N1 / 2
            if (p0 >= P1)
                continue;
            if (p0 > 0)
            {
                const long long ka = p0 / 2 + (long long)N1 * k2;
                const cpx<T> u     = stage[swz_8b<S>(k2, 2 * q)];
                const cpx<T> v     = stage[swz_8b<S>(N2 - 1 - k2, 2 * q + 1)];
                const cpx<T> w     = ldg(rtw + p0 / 2) * ldg(rtw + N1 + k2);
                X[ka]              = split(u, v, w);
                X[C - ka]          = split(v, u, mirror(w));
                continue;
            }
            // row 0: Z[N1 k2] pairs with Z[N1 (N2 - k2)] in the same row; Z[0] gives X[0] and X[c]
            if (2 * k2 <= N2)
            {
                const cpx<T> u = stage[swz_8b<S>(k2, 2 * q)];
                if (k2 == 0)
                {
                    X[0] = ccs ? mk<T>(u.x + u.y, T(0)) : mk<T>(u.x + u.y, u.x - u.y);
                    if (ccs)
                        X[C] = mk<T>(u.x - u.y, T(0));
                }
                else
                {
                    const cpx<T> v     = stage[swz_8b<S>(N2 - k2, 2 * q)];
                    const long long ka = (long long)N1 * k2;
                    const cpx<T> w     = ldg(rtw + N1 + k2);
                    X[ka]              = split(u, v, w);
                    if (2 * k2 != N2)
                        X[C - ka] = split(v, u, mirror(w));
                }
            }
            // row N1/2 (N1 even, position 1): Z[N1/2 + N1 k2] pairs with k2' = N2 - 1 - k2 in the same row
            if (N1 % 2 == 0 && 2 * k2 <= N2 - 1)
            {
                const cpx<T> u     = stage[swz_8b<S>(k2, 2 * q + 1)];
                const cpx<T> v     = stage[swz_8b<S>(N2 - 1 - k2, 2 * q + 1)];
                const long long ka = N1 / 2 + (long long)N1 * k2;
                const cpx<T> w     = ldg(rtw + N1 / 2) * ldg(rtw + N1 + k2);
                X[ka]              = split(u, v, w);
                if (2 * k2 != N2 - 1)
                    X[C - ka] = split(v, u, mirror(w));
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------------
// Launchers.  A block_cfg with ct != 0 selects the compile-time kernel of that length (single precision,
// launched by the launch_ct_* functions of kernels_ct_*.cu); otherwise cfg.ept picks the runtime kernel.
// ---------------------------------------------------------------------------------------------------

template <typename K, typename... Args>
static cudaError_t go(K kernel, dim3 grid, const block_cfg& c, cudaStream_t st, Args... args)
{
    if (c.smem > 48 * 1024)
    {
        const cudaError_t e = prepare_launch(reinterpret_cast<const void*>(kernel), c.threads, c.smem);
        if (e != cudaSuccess)
            return e;
    }
    kernel<<<grid, c.threads, c.smem, st>>>(args...);
    return cudaGetLastError();
}

#define KFR_GPU_RUNTIME_DISPATCH(KERNEL, GRID, ...)                                                        \
    switch (c.ept)                                                                                         \
    {                                                                                                      \
    case 16: return go(KERNEL<T, rt_fft<T, 16>>, GRID, c, st, __VA_ARGS__);                                \
    case 32: return go(KERNEL<T, rt_fft<T, 32>>, GRID, c, st, __VA_ARGS__);                                \
    default: return cudaErrorInvalidValue;                                                                 \
    }

#define KFR_GPU_CT_HOOK(CTFN)                                                                              \
    if (c.ct)                                                                                              \
    {                                                                                                      \
        if constexpr (std::is_same<T, float>::value)                                                       \
            return CTFN(a, c, st);                                                                         \
        else                                                                                               \
            return cudaErrorInvalidValue;                                                                  \
    }

#define KFR_GPU_GRID1 dim3(unsigned(c.grid))
#define KFR_GPU_GRID2 dim3(unsigned(c.grid), unsigned(a.batch))

template <typename T>
cudaError_t launch_c2c(const c2c_args& a, const block_cfg& c, cudaStream_t st)
{
    KFR_GPU_CT_HOOK(launch_ct_c2c_f32)
    KFR_GPU_RUNTIME_DISPATCH(k_c2c, KFR_GPU_GRID1, a, c.ts, c.spc)
}
template <typename T>
cudaError_t launch_bluestein(const bluestein_args& a, const block_cfg& c, cudaStream_t st)
{
    KFR_GPU_CT_HOOK(launch_ct_bluestein_f32)
    KFR_GPU_RUNTIME_DISPATCH(k_bluestein, KFR_GPU_GRID1, a, c.ts, c.spc)
}
template <typename T>
cudaError_t launch_rader(const rader_args& a, const block_cfg& c, cudaStream_t st)
{
    KFR_GPU_CT_HOOK(launch_ct_rader_f32)
    KFR_GPU_RUNTIME_DISPATCH(k_rader, KFR_GPU_GRID1, a, c.ts, c.spc)
}
template <typename T>
cudaError_t launch_r2c(const real_args& a, const block_cfg& c, cudaStream_t st)
{
    KFR_GPU_CT_HOOK(launch_ct_r2c_f32)
    KFR_GPU_RUNTIME_DISPATCH(k_r2c, KFR_GPU_GRID1, a, c.ts, c.spc)
}
template <typename T>
cudaError_t launch_c2r(const real_args& a, const block_cfg& c, cudaStream_t st)
{
    KFR_GPU_CT_HOOK(launch_ct_c2r_f32)
    KFR_GPU_RUNTIME_DISPATCH(k_c2r, KFR_GPU_GRID1, a, c.ts, c.spc)
}
template <typename T>
cudaError_t launch_dct2(const dct_args& a, const block_cfg& c, cudaStream_t st)
{
    KFR_GPU_CT_HOOK(launch_ct_dct2_f32)
    KFR_GPU_RUNTIME_DISPATCH(k_dct2, KFR_GPU_GRID1, a, c.ts, c.spc)
}
template <typename T>
cudaError_t launch_dct3(const dct_args& a, const block_cfg& c, cudaStream_t st)
{
    KFR_GPU_CT_HOOK(launch_ct_dct3_f32)
    KFR_GPU_RUNTIME_DISPATCH(k_dct3, KFR_GPU_GRID1, a, c.ts, c.spc)
}
template <typename T>
cudaError_t launch_fs_cols(const fourstep_args& a, const block_cfg& c, cudaStream_t st)
{
    KFR_GPU_CT_HOOK(launch_ct_fs_cols_f32)
    KFR_GPU_RUNTIME_DISPATCH(k_fs_cols, KFR_GPU_GRID2, a, c.ts)
}
template <typename T>
cudaError_t launch_fs_rows(const fourstep_args& a, const block_cfg& c, cudaStream_t st)
{
    KFR_GPU_CT_HOOK(launch_ct_fs_rows_f32)
    KFR_GPU_RUNTIME_DISPATCH(k_fs_rows, KFR_GPU_GRID2, a, c.ts)
}

// Compile-time kernel cases for the launch_ct_* functions: CT_KERNEL and CT_ARGS are defined by the caller.
#define KFR_GPU_CT_CASE(N, TS, ...)                                                                        \
    case N: return go(CT_KERNEL<float, ct_fft<float, N, TS, __VA_ARGS__>>, CT_GRID, c, st, CT_ARGS);

#define KFR_GPU_INSTANTIATE(T)                                                                             \
    template cudaError_t launch_c2c<T>(const c2c_args&, const block_cfg&, cudaStream_t);                   \
    template cudaError_t launch_bluestein<T>(const bluestein_args&, const block_cfg&, cudaStream_t);       \
    template cudaError_t launch_rader<T>(const rader_args&, const block_cfg&, cudaStream_t);               \
    template cudaError_t launch_r2c<T>(const real_args&, const block_cfg&, cudaStream_t);                  \
    template cudaError_t launch_c2r<T>(const real_args&, const block_cfg&, cudaStream_t);                  \
    template cudaError_t launch_dct2<T>(const dct_args&, const block_cfg&, cudaStream_t);                  \
    template cudaError_t launch_dct3<T>(const dct_args&, const block_cfg&, cudaStream_t);                  \
    template cudaError_t launch_fs_cols<T>(const fourstep_args&, const block_cfg&, cudaStream_t);          \
    template cudaError_t launch_fs_rows<T>(const fourstep_args&, const block_cfg&, cudaStream_t);

} // namespace kfr_gpu
