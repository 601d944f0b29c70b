// Rader's algorithm with prime-factor (Good-Thomas) convolution DFTs, for primes N whose L = N - 1 splits
// into pairwise coprime compile-time radices (8191: 8190 = 13 * 5 * 9 * 14; 127: 126 = 14 * 9).
//
// Rader (as in the per-signal kernel k_rader): a[p] = x[g^p] (p < L), A = DFT_L(a), A'[k] = conj(A[k] bhat[k]) with
// bhat = DFT_L(b) / L, b[m] = W_N^{g^-m}; C = DFT_L(A'); X[g^-q] = x[0] + conj(C[q]); X[0] = x[0] + A[0].
//
// Prime-factor form of the two L-point DFTs (Good 1958, Thomas 1963): with L = r_0 r_1 ... r_{d-1} pairwise
// coprime and L_i = L / r_i, write an index n either by its residues (CRT map: n_i = n mod r_i) or as
// n = sum_i n_i L_i mod L (Ruritanian map).  If the input index is mapped one way and the output index the
// other, n k = sum_i n_i k_i L_i (mod L), so W_L^{n k} = prod_i W_{r_i}^{n_i k_i}: the DFT is a
// d-dimensional array of plain r_i-point DFTs, one pass per axis, with no twiddle factors.  The first DFT
// takes its input by the CRT map and leaves its output by the Ruritanian map; the second takes that layout
// as its (Ruritanian) input and leaves its output by the CRT map.  So nothing is permuted between the two,
// and the input gather x[g^p] and the output scatter X[g^-q] fold into two index tables over the array:
//   tin[pos]  = g^p mod N,   p = the index whose residues are pos's coordinates,
//   tout[pos] = g^-p mod N,
//   bphys[pos] = bhat[k],    k = sum_i c_i L_i mod L for pos's coordinates c_i.
// The array is row-major over the axes r_0 (outermost) ... r_{d-1}.  A pass along axis i runs each
// butterfly in place (it reads and writes its own r_i elements only), so one buffer per signal suffices and
// only the gather and the scatter need a barrier between their reads and their writes.
//
// Kernel: persistent over tiles of SPC contiguous signals; a shared buffer per tile in flight (NBUF = 2: the
// next tile's copy lands in the second buffer while this one is transformed).  A bulk copy brings the tile's
// enclosing 16-byte range in; pass 1 (axis 0) gathers into registers, a barrier, then writes the array; the
// middle axes run in place; the last axis of the first DFT and the same axis of the second are fused around
// the multiplication by bphys; the second DFT's axis-0 pass reads into registers, a barrier, then scatters X
// in natural order into the buffer, which one bulk copy stores (the tile's edge elements beyond the 16-byte
// interior by plain stores).  The three tables (bphys, and tin / tout as 16-bit indices) are copied into
// shared memory once per CTA.  Measured on 256 MiB batches (N=8191: 640 threads, one CTA per SM; N=127: 24
// signals per tile, four CTAs per SM), two buffers beat one by 16% to 20%, an earlier tiled ping-pong kernel
// (three buffers, twiddled passes) by 12% (8191) and 22% (127), and the shared-memory tables the same tables
// read through L1 by 6.5% (8191: 96 KB of tables beside 128 KB of tile buffers) and 4.5% (127).
#include "kernels.cuh"

namespace kfr_gpu
{

namespace
{

template <int... R>
struct axes
{
    static constexpr int d    = sizeof...(R);
    static constexpr int r[d] = { R... };
    __host__ __device__ static constexpr int len()
    {
        int l = 1;
        for (int i = 0; i < d; i++)
            l *= r[i];
        return l;
    }
    // stride of axis i in the row-major array
    __host__ __device__ static constexpr int stride(int i)
    {
        int s = 1;
        for (int j = i + 1; j < d; j++)
            s *= r[j];
        return s;
    }
};

// A pass along one axis (R points, stride S) over `nsig` signals of L points: butterflies j = tid,
// tid + THREADS, ...; each loads its R elements, runs DFT_R and stores in place.  TWICE (the fused axis):
// between two DFT_R, `mid(pos, signal, value)` maps each output.
template <typename T, int R, int S, int L, int THREADS, bool TWICE, class MID>
__device__ __forceinline__ void axis_pass(cpx<T>* buf, const int nsig, const MID& mid)
{
    constexpr int NB = L / R;
    for (int j = threadIdx.x; j < nsig * NB; j += THREADS)
    {
        const int s    = j / NB;
        const int b    = j - s * NB;
        const int base = s * L + (b / S) * (S * R) + (b % S);
        cpx<T> v[R];
#pragma unroll
        for (int t = 0; t < R; t++)
            v[t] = buf[base + t * S];
        dft_codelet<T, R>(v);
        if constexpr (TWICE)
        {
            cpx<T> w[R];
#pragma unroll
            for (int t = 0; t < R; t++)
                w[t] = mid(base + t * S - s * L, s, v[codelet_out<R>(t)]);
            dft_codelet<T, R>(w);
#pragma unroll
            for (int t = 0; t < R; t++)
                buf[base + t * S] = w[codelet_out<R>(t)];
        }
        else
        {
#pragma unroll
            for (int t = 0; t < R; t++)
                buf[base + t * S] = v[codelet_out<R>(t)];
        }
    }
}

// The passes along the middle axes I .. LAST (ascending, STEP = 1, or descending, STEP = -1), in place.
template <typename T, class AX, int I, int LAST, int STEP, int THREADS>
__device__ __forceinline__ void middle_passes(cpx<T>* buf, const int nsig)
{
    if constexpr ((STEP > 0 && I <= LAST) || (STEP < 0 && I >= LAST))
    {
        constexpr int R = AX::r[I], S = AX::stride(I), L = AX::len();
        const auto keep = [](int, int, cpx<T> x) { return x; };
        axis_pass<T, R, S, L, THREADS, false>(buf, nsig, keep);
        __syncthreads();
        middle_passes<T, AX, I + STEP, LAST, STEP, THREADS>(buf, nsig);
    }
}

template <int N, int SPC>
__host__ __device__ constexpr int pfa_buflen()
{
    // the tile in natural order (plus the enclosing 16-byte range's slack) and the array of SPC (N - 1) points
    return ((SPC * N + 2 > SPC * (N - 1) ? SPC * N + 2 : SPC * (N - 1)) + 15) / 16 * 16;
}

template <typename T, int N, int SPC, int THREADS, int MINB, int NBUF, int... R>
__global__ void __launch_bounds__(THREADS, MINB) k_rader_pfa(const rader_pfa_args a, const long long ntiles)
{
    using AX          = axes<R...>;
    constexpr int L   = N - 1;
    constexpr int D   = AX::d;
    constexpr int R0  = AX::r[0];
    constexpr int S0  = AX::stride(0);
    constexpr int NB0 = L / R0;
    constexpr int RF  = AX::r[D - 1]; // the fused axis
    constexpr int ESZ = int(sizeof(cpx<T>));
    static_assert(AX::len() == L, "the axes multiply to N - 1");
    static_assert(SPC * NB0 <= THREADS, "one axis-0 butterfly per thread in the gather and scatter passes");
    static_assert(D >= 2, "at least the gather axis and the fused axis");
    static_assert(NBUF == 1 || NBUF == 2, "one buffer, or two with the next tile's copy overlapping");
    extern __shared__ __align__(128) unsigned char smem_raw[];
    cpx<T>* const bufs = reinterpret_cast<cpx<T>*>(smem_raw);
    cpx<T>* x0s        = bufs + NBUF * pfa_buflen<N, SPC>();
    cpx<T>* a0s        = x0s + SPC;
    uint64_t* bars     = reinterpret_cast<uint64_t*>(a0s + SPC);
    // the kernel-spectrum and index tables, copied once per CTA into shared memory (for N = 8191 they are
    // 96 KB, which the L1 left beside the tile buffers does not hold)
    static_assert(N <= 65536, "16-bit index tables");
    cpx<T>* const sbph    = reinterpret_cast<cpx<T>*>(bars + NBUF);
    uint16_t* const stin  = reinterpret_cast<uint16_t*>(sbph + L);
    uint16_t* const stout = stin + L;
    for (int i = threadIdx.x; i < L; i += THREADS)
    {
        sbph[i]  = ldg(reinterpret_cast<const cpx<T>*>(a.bphys) + i);
        stin[i]  = uint16_t(__ldg(a.tin + i));
        stout[i] = uint16_t(__ldg(a.tout + i));
    }
    // kernel parameters are read where they are used (from the parameter bank), and the tile's byte range is
    // recomputed after the passes, so that little stays live across the passes' register-heavy codelets
    constexpr long long tile_bytes = (long long)SPC * N * ESZ;
    // thread 0 issues tile tt's copy into buffer b (after the store that last read it, which is the only
    // store outstanding then); the final 8-byte element of the last tile, beyond its 16-byte interior (the
    // enclosing range could reach past the batch), is loaded by a plain load
    const auto load = [&](long long tt, int b)
    {
        const int nt       = int(a.batch - tt * SPC < SPC ? a.batch - tt * SPC : SPC);
        const long long s0 = tt * tile_bytes, e = s0 + (long long)nt * N * ESZ;
        const long long a0 = s0 & ~15LL;
        const long long a1 = tt == ntiles - 1 ? (e & ~15LL) : ((e + 15) & ~15LL);
        const char* inb    = reinterpret_cast<const char*>(a.in);
        cpx<T>* dst        = bufs + b * pfa_buflen<N, SPC>();
        bulk_wait_read();
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bars[b], uint32_t(a1 - a0));
        bulk_g2s(dst, inb + a0, uint32_t(a1 - a0), &bars[b]);
        if (a1 < e)
            *reinterpret_cast<cpx<T>*>(reinterpret_cast<char*>(dst) + (e - ESZ - a0)) =
                *reinterpret_cast<const cpx<T>*>(inb + e - ESZ);
    };
    if (threadIdx.x == 0)
    {
        for (int b = 0; b < NBUF; b++)
            mbar_init(&bars[b], 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0 && blockIdx.x < ntiles)
        load(blockIdx.x, 0);
    uint32_t phase   = 0; // bit b: parity to wait for on buffer b
    uint32_t pending = blockIdx.x < ntiles ? 1u : 0u; // bit b: a copy into buffer b is in flight
    int cur          = 0;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x)
    {
        const int ns      = int(a.batch - t * SPC < SPC ? a.batch - t * SPC : SPC);
        cpx<T>* const buf = bufs + cur * pfa_buflen<N, SPC>();
        const bool got    = mbar_wait(&bars[cur], (phase >> cur) & 1, a.wait_spins);
        if (!__syncthreads_and(got))
        {
            if (threadIdx.x == 0)
            {
                atomicExch(a.err, 1);
                // give every copy in flight into this CTA's shared memory a bounded chance to land before the
                // CTA exits
                for (int b = 0; b < NBUF; b++)
                    if ((pending >> b) & 1)
                        mbar_wait(&bars[b], (phase >> b) & 1);
                bulk_wait_all();
            }
            return;
        }
        phase ^= 1u << cur;
        pending &= ~(1u << cur);
        const long long tn = t + gridDim.x;
        if constexpr (NBUF == 2)
        {
            // the next tile streams into the other buffer while this one is transformed
            if (tn < ntiles)
            {
                pending |= 1u << (cur ^ 1);
                if (threadIdx.x == 0)
                    load(tn, cur ^ 1);
            }
        }
        const int off = int(((t * tile_bytes) & 15) / ESZ); // the tile's first element in the buffer
        const bool inv = a.inverse != 0;
        if (int(threadIdx.x) < ns)
            x0s[threadIdx.x] = conj_if(buf[off + threadIdx.x * N], inv);
        // pass 1, axis 0 of the first DFT: gather a[p] = x[g^p] into registers
        const int gs    = int(threadIdx.x) / NB0, gb = int(threadIdx.x) - gs * NB0;
        const bool gact = gs < ns;
        cpx<T> v[R0];
        if (gact)
        {
#pragma unroll
            for (int q = 0; q < R0; q++)
                v[q] = conj_if(buf[off + gs * N + stin[gb + q * S0]], inv);
            dft_codelet<T, R0>(v);
        }
        __syncthreads(); // every gather is done before the array overwrites the input
        if (gact)
        {
#pragma unroll
            for (int q = 0; q < R0; q++)
                buf[gs * L + gb + q * S0] = v[codelet_out<R0>(q)];
        }
        __syncthreads();
        // the first DFT's middle axes
        middle_passes<T, AX, 1, D - 2, 1, THREADS>(buf, ns);
        // the fused axis: last pass of the first DFT, conj(A bhat), first pass of the second DFT
        {
            constexpr int SF = AX::stride(D - 1);
            const auto mul   = [&](int pos, int s, cpx<T> x)
            {
                if (pos == 0)
                    a0s[s] = x; // A[0]: the sum of x[1..N-1]
                return conj(x * sbph[pos]);
            };
            axis_pass<T, RF, SF, L, THREADS, true>(buf, ns, mul);
        }
        __syncthreads();
        // the second DFT's middle axes, in reverse order
        middle_passes<T, AX, D - 2, 1, -1, THREADS>(buf, ns);
        // last pass, axis 0 of the second DFT: into registers, then X[g^-q] = x[0] + conj(C[q]) in natural order
        if (gact)
        {
#pragma unroll
            for (int q = 0; q < R0; q++)
                v[q] = buf[gs * L + gb + q * S0];
            dft_codelet<T, R0>(v);
        }
        __syncthreads(); // every read of the array is done before the output overwrites it
        if (gact)
        {
            const cpx<T> x0 = x0s[gs];
#pragma unroll
            for (int q = 0; q < R0; q++)
                buf[off + gs * N + stout[gb + q * S0]] = conj_if(x0 + conj(v[codelet_out<R0>(q)]), a.inverse != 0);
        }
        if (int(threadIdx.x) < ns)
            buf[off + threadIdx.x * N] = conj_if(x0s[threadIdx.x] + a0s[threadIdx.x], a.inverse != 0);
        fence_proxy_async_smem();
        __syncthreads();
        // the tile's output: its 16-byte-aligned interior by a bulk store, the (at most two) 8-byte edge
        // elements by plain stores
        const long long s0 = t * tile_bytes, e = s0 + (long long)ns * N * ESZ, a0 = s0 & ~15LL;
        const long long c0 = (s0 + 15) & ~15LL, c1 = e & ~15LL;
        char* outb         = reinterpret_cast<char*>(a.out);
        if (threadIdx.x == 0)
        {
            if (c1 > c0)
                bulk_s2g(outb + c0, reinterpret_cast<const char*>(buf) + (c0 - a0), uint32_t(c1 - c0));
            bulk_commit();
        }
        if (threadIdx.x == 32 % THREADS && c0 != s0)
            *reinterpret_cast<cpx<T>*>(outb + s0) = buf[off];
        if (threadIdx.x == 64 % THREADS && c1 != e)
            *reinterpret_cast<cpx<T>*>(outb + e - ESZ) = buf[off + ns * N - 1];
        __syncthreads(); // the edge stores have read the buffer before a later copy overwrites it
        if constexpr (NBUF == 1)
        {
            if (tn < ntiles)
            {
                pending |= 1u;
                if (threadIdx.x == 0)
                    load(tn, 0);
            }
        }
        else
            cur ^= 1;
    }
    if (threadIdx.x == 0)
        bulk_wait_all();
}

template <int N, int SPC, int NBUF>
constexpr int pfa_smem()
{
    // tile buffers, x[0] and A[0] per signal, mbarriers, the spectrum table and the two 16-bit index tables
    return (NBUF * pfa_buflen<N, SPC>() + 2 * SPC) * 8 + NBUF * 8 + (N - 1) * (8 + 2 + 2);
}

template <class K>
cudaError_t go_pfa(K kernel, int threads, int smem, long long ntiles, const rader_pfa_args& a, cudaStream_t st)
{
    int per_sm    = 0;
    cudaError_t e = prepare_launch(reinterpret_cast<const void*>(kernel), threads, smem, &per_sm);
    if (e != cudaSuccess)
        return e;
    const int sms = device_sm_count();
    if (per_sm < 1 || sms < 1)
        return cudaErrorInvalidConfiguration;
    const long long grid = std::min<long long>(ntiles, (long long)per_sm * sms);
    kernel<<<unsigned(grid), threads, smem, st>>>(a, ntiles);
    return cudaGetLastError();
}

// The compile-time instances: X(N, signals per tile, threads, CTAs per SM, buffers, axes: gather axis first,
// fused axis last)
#define KFR_RADER_PFA_F32(X)                                                                               \
    X(8191, 1, 640, 1, 2, 13, 5, 9, 14)                                                                      \
    X(127, 24, 224, 4, 2, 14, 9)

} // namespace

bool rader_pfa_shape(long long n, std::vector<int>& axes_out, int& spc)
{
#define KFR_RADER_PFA_SHAPE(N, SPC, TH, MB, NB, ...)                                                           \
    if (n == N)                                                                                            \
    {                                                                                                      \
        axes_out = { __VA_ARGS__ };                                                                        \
        spc      = SPC;                                                                                    \
        return true;                                                                                       \
    }
    KFR_RADER_PFA_F32(KFR_RADER_PFA_SHAPE)
#undef KFR_RADER_PFA_SHAPE
    return false;
}

cudaError_t launch_rader_pfa_f32(const rader_pfa_args& a0, long long n, cudaStream_t st)
{
    rader_pfa_args a = a0;
    a.wait_spins     = wait_limit();
#define KFR_RADER_PFA_CASE(N, SPC, TH, MB, NB, ...)                                                        \
    if (n == N)                                                                                            \
        return go_pfa(k_rader_pfa<float, N, SPC, TH, MB, NB, __VA_ARGS__>, TH, pfa_smem<N, SPC, NB>(),    \
                      (a.batch + SPC - 1) / SPC, a, st);
    KFR_RADER_PFA_F32(KFR_RADER_PFA_CASE)
#undef KFR_RADER_PFA_CASE
    return cudaErrorInvalidValue;
}

} // namespace kfr_gpu
