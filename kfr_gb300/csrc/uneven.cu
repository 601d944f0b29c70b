// Uneven batch: persistent dependency-aware work-queue kernel, plan, autotuner and graph capture
// (uneven.hpp).
#include "uneven.hpp"
#include "kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <sstream>

namespace kfr_gpu
{

// ------------------------------------------------------------------------------------------------------
// kernel
// ------------------------------------------------------------------------------------------------------

__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// L2 load (bypasses L1): data another CTA wrote during this launch
__device__ __forceinline__ cpx<float> ld_cg(const cpx<float>* p)
{
    const float2 v = __ldcg(reinterpret_cast<const float2*>(p));
    return mk<float>(v.x, v.y);
}
__device__ __forceinline__ cpx<double> ld_cg(const cpx<double>* p)
{
    const double2 v = __ldcg(reinterpret_cast<const double2*>(p));
    return mk<double>(v.x, v.y);
}

template <typename T>
__global__ void __launch_bounds__(kUnevenThreads, 1) k_uneven(const uneven_launch a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ pass_desc sp[kMaxPasses];
    __shared__ long long s_off[kUnevenMaxSpc];
    __shared__ uneven_job J;
    __shared__ int s_item, s_count, s_first, s_fft, s_m, s_ts, s_stride, s_npass;
    __shared__ fast_div s_div;
    __shared__ const cpx<T>* s_tw;
    cpx<T>* sm = reinterpret_cast<cpx<T>*>(smem_raw);
    const cpx<T>* gin = reinterpret_cast<const cpx<T>*>(a.in);
    cpx<T>* gout      = reinterpret_cast<cpx<T>*>(a.out);
    cpx<T>* gscr      = reinterpret_cast<cpx<T>*>(a.scratch);
    const bool inv    = a.inverse != 0;
    if (threadIdx.x == 0)
        s_fft = -1;
    for (;;)
    {
        __syncthreads();
        if (threadIdx.x == 0)
        {
            const int it = atomicAdd(a.queue, 1);
            s_item       = it;
            if (it < a.nitems)
            {
                const uneven_item w = a.items[it];
                J                   = a.jobs[w.job];
                s_count             = w.count;
                s_first             = w.first;
                if (J.fft != s_fft)
                {
                    const uneven_fft& F = a.ffts[J.fft];
                    s_fft    = J.fft;
                    s_m      = F.m;
                    s_ts     = F.ts;
                    s_stride = F.stride;
                    s_npass  = F.d.npass;
                    s_div    = F.div_m;
                    s_tw     = reinterpret_cast<const cpx<T>*>(F.tw);
                    for (int p = 0; p < F.d.npass; p++)
                        sp[p] = F.d.pass[p];
                }
                if (J.wait >= 0)
                {
                    // every tile of the stage waited for was dequeued before this one and runs on a resident
                    // CTA, so the counter reaches `need`; the bound only guards against a fault elsewhere
                    uint32_t spins = 0;
                    while (ld_acquire(a.counters + J.wait) < J.need + a.stage_bias)
                    {
                        if (spins++ >= a.wait_spins)
                        {
                            atomicExch(a.err, 1); // carry on: the tile's loads stay inside its buffers
                            break;
                        }
                        __nanosleep(256);
                    }
                }
            }
        }
        __syncthreads();
        const int it = s_item;
        if (it >= a.nitems)
            break;
        const int mode = J.mode, cnt = s_count, m = s_m, stride = s_stride;
        if (mode <= UM_BLUE1)
        {
            if (int(threadIdx.x) < cnt)
                s_off[threadIdx.x] = a.offsets[s_first + threadIdx.x];
            __syncthreads();
            const int n = J.n;
            const fast_div dm   = s_div;
            const cpx<T>* chirp = mode == UM_BLUE1 ? reinterpret_cast<const cpx<T>*>(J.chirp) : nullptr;
#pragma unroll 4
            for (int i = threadIdx.x; i < cnt * m; i += blockDim.x)
            {
                const int s = int(fdiv(uint32_t(i), dm));
                const int e = i - s * m;
                cpx<T> v    = mk<T>(0, 0);
                if (e < n)
                {
                    v = conj_if(gin[s_off[s] + e], inv);
                    if (chirp)
                        v = v * ldg(chirp + e);
                }
                sm[s * stride + pidx<T>(e)] = v;
            }
        }
        else
        {
            // a tile of `cnt` (a power of two) columns (COL) or rows (ROW) of a four-step transform
            const int S = cnt, sh = 31 - __clz(cnt);
            const int n1 = J.n1, n2 = J.n2, c0 = s_first;
            const cpx<T>* src = (J.src == 0 ? gin : J.src == 1 ? gout : gscr) + J.src_off;
            const bool cj     = J.first && inv;
            if (mode == UM_COL)
            {
                const cpx<T>* chirp = J.pre ? reinterpret_cast<const cpx<T>*>(J.chirp) : nullptr;
                const long long nv  = J.nvalid;
#pragma unroll 4
                for (int i = threadIdx.x; i < S * m; i += blockDim.x)
                {
                    const int j1 = i >> sh, c = i & (S - 1), col = c0 + c;
                    const long long g = (long long)j1 * n2 + col;
                    cpx<T> v          = mk<T>(0, 0);
                    if (col < n2 && (!chirp || g < nv))
                    {
                        v = J.src == 2 ? ld_cg(src + g) : src[g];
                        v = conj_if(v, cj);
                        if (chirp)
                            v = v * ldg(chirp + g);
                    }
                    sm[c * stride + pidx<T>(j1)] = v;
                }
            }
            else
            {
#pragma unroll 4
                for (int i = threadIdx.x; i < S * m; i += blockDim.x)
                {
                    const int n2i = i >> sh, r = i & (S - 1), row = c0 + r;
                    cpx<T> v      = mk<T>(0, 0);
                    if (row < n1)
                    {
                        const long long g = (long long)n2i * n1 + row;
                        v = J.src == 2 ? ld_cg(src + g) : src[g];
                        v = conj_if(v, cj);
                    }
                    sm[r * stride + pidx<T>(n2i)] = v;
                }
            }
        }
        // one FFT call site, run twice for a one-CTA Bluestein tile (times the kernel spectrum in between)
        for (int round = 0;; round++)
        {
            __syncthreads();
            {
                const group_map gm(s_ts, cnt);
                block_fft<T, 16>(sm + gm.g * s_stride, sp, s_npass, s_m, s_tw, gm.lt, s_ts);
            }
            if (J.mode != UM_BLUE1 || round == 1)
                break;
            const int mm = s_m, st = s_stride;
            const fast_div dm  = s_div;
            const cpx<T>* bhat = reinterpret_cast<const cpx<T>*>(J.bhat);
            for (int i = threadIdx.x; i < cnt * mm; i += blockDim.x)
            {
                const int s = int(fdiv(uint32_t(i), dm));
                const int e = i - s * mm;
                cpx<T>& r   = sm[s * st + pidx<T>(e)];
                r           = conj(r * ldg(bhat + e));
            }
        }
        if (mode <= UM_BLUE1)
        {
            const int n = J.n;
            const fast_div dm   = s_div;
            const cpx<T>* chirp = mode == UM_BLUE1 ? reinterpret_cast<const cpx<T>*>(J.chirp) : nullptr;
#pragma unroll 4
            for (int i = threadIdx.x; i < cnt * m; i += blockDim.x)
            {
                const int s = int(fdiv(uint32_t(i), dm));
                const int e = i - s * m;
                if (e < n)
                {
                    const cpx<T> r     = sm[s * stride + pidx<T>(e)];
                    gout[s_off[s] + e] = chirp ? conj_if(conj(r) * ldg(chirp + e), inv) : conj_if(r, inv);
                }
            }
        }
        else
        {
            const int S = cnt, sh = 31 - __clz(cnt);
            const int n1 = J.n1, n2 = J.n2, c0 = s_first;
            cpx<T>* dst   = (J.dst == 1 ? gout : gscr) + J.dst_off;
            const bool cj = J.last && inv;
            if (mode == UM_COL)
            {
                const cpx<T>* twA = reinterpret_cast<const cpx<T>*>(J.twA);
                const cpx<T>* twB = reinterpret_cast<const cpx<T>*>(J.twB);
                const fast_div dm = s_div;
#pragma unroll 4
                for (int i = threadIdx.x; i < S * m; i += blockDim.x)
                {
                    const int c = int(fdiv(uint32_t(i), dm)), k1 = i - c * m, col = c0 + c;
                    if (col < n2)
                    {
                        const cpx<T> v = sm[c * stride + pidx<T>(k1)] *
                                         twiddle_2level(twA, twB, (long long)col * k1, J.lbits);
                        dst[(long long)col * n1 + k1] = conj_if(v, cj);
                    }
                }
            }
            else
            {
                const cpx<T>* chirp = reinterpret_cast<const cpx<T>*>(J.chirp);
                const cpx<T>* bhat  = reinterpret_cast<const cpx<T>*>(J.bhat);
                const int post      = J.post;
                const long long nv  = J.nvalid;
#pragma unroll 4
                for (int i = threadIdx.x; i < S * m; i += blockDim.x)
                {
                    const int k2 = i >> sh, r = i & (S - 1), row = c0 + r;
                    if (row >= n1)
                        continue;
                    const long long k = row + (long long)n1 * k2;
                    const cpx<T> v    = sm[r * stride + pidx<T>(k2)];
                    if (post == 0)
                        dst[k] = conj_if(v, cj);
                    else if (post == 1)
                        dst[k] = conj(v * ldg(bhat + k));
                    else if (k < nv)
                        dst[k] = conj_if(conj(v) * ldg(chirp + k), inv);
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0 && J.done >= 0)
        {
            __threadfence();
            atomicAdd(a.counters + J.done, 1);
        }
    }
}

cudaError_t launch_uneven_f32(const uneven_launch& a, int smem, int grid, cudaStream_t st)
{
    const cudaError_t e = prepare_launch(reinterpret_cast<const void*>(k_uneven<float>), kUnevenThreads, smem);
    if (e != cudaSuccess)
        return e;
    k_uneven<float><<<unsigned(grid), kUnevenThreads, smem, st>>>(a);
    return cudaGetLastError();
}

int uneven_max_smem()
{
    // dynamic shared memory beside the kernel's static pass list, offsets and job
    return max_smem_bytes() - int(sizeof(pass_desc)) * kMaxPasses - int(sizeof(long long)) * kUnevenMaxSpc -
           int(sizeof(uneven_job)) - 1024;
}

// ------------------------------------------------------------------------------------------------------
// plan
// ------------------------------------------------------------------------------------------------------

namespace
{

std::mutex g_tune_mu;
std::map<long long, std::pair<std::vector<int>, int>> g_tune; // length -> fastest radix order and tile

bool fits_one_cta(long long m, const std::vector<int>& order, int& ts)
{
    if (order.empty() || m > 8192)
        return false;
    ts = threads_needed(m, order, 16);
    return ts > 0 && ts <= kUnevenThreads && padded_len_host<float>(int(m)) * 8 <= uneven_max_smem();
}

std::vector<std::vector<int>> candidate_orders(long long m)
{
    std::vector<std::vector<int>> c;
    const auto a = factor_radices(m);
    if (a.empty())
        return c;
    auto add = [&](std::vector<int> v)
    {
        if (std::find(c.begin(), c.end(), v) == c.end())
            c.push_back(v);
    };
    add(a);
    add(std::vector<int>(a.rbegin(), a.rend()));
    auto d = a;
    std::sort(d.begin(), d.end(), std::greater<int>());
    add(d);
    std::sort(d.begin(), d.end());
    add(d);
    return c;
}

// largest power-of-two tile (<= 16) of columns / rows of an m-point FFT of `ts` threads within one CTA
int tile_of(int m, int ts)
{
    int s = 16;
    while (s > 1 && (s * ts > kUnevenThreads || s * padded_len_host<float>(m) * 8 > uneven_max_smem()))
        s /= 2;
    return s;
}

// four-step split n = n1 * n2 with both factors one-CTA lengths, as balanced as possible
bool split_of(long long n, int& n1, int& n2)
{
    long long best = 0;
    for (long long a = 2; a * a <= n; a++)
    {
        if (n % a)
            continue;
        const long long b = n / a;
        int t1 = 0, t2 = 0;
        if (fits_one_cta(a, factor_radices(a), t1) && fits_one_cta(b, factor_radices(b), t2))
            best = a;
    }
    if (!best)
        return false;
    n1 = int(best);
    n2 = int(n / best);
    return true;
}

} // namespace

int uneven_plan::get_shape(long long m, int, const std::vector<int>* order)
{
    std::vector<int> o = order ? *order : factor_radices(m);
    if (!order)
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto f = g_tune.find(m);
        if (f != g_tune.end())
            o = f->second.first;
    }
    const std::pair<long long, int> key(m, 0);
    auto f = shape_of_.find(key);
    if (f != shape_of_.end() && !order)
        return f->second;
    std::unique_ptr<shape> s(new shape);
    if (m == 1)
    {
        // length 1: no passes (the transform is the identity); a one-element table keeps tw valid
        std::memset(&s->prog.desc, 0, sizeof(s->prog.desc));
        s->prog.desc.n = 1;
        s->prog.n      = 1;
        s->prog.gstride = padded_len_host<float>(1);
        const std::complex<float> one(1, 0);
        s->prog.tw.upload(&one, sizeof(one));
        s->ts = 1;
    }
    else
    {
        int ts = 0;
        if (!fits_one_cta(m, o, ts))
            throw std::invalid_argument("internal: uneven batch shape exceeds one CTA");
        s->prog.build(int(m), CT_NONE, &o, 16);
        s->ts = s->prog.ts;
    }
    const int idx = int(shapes_.size());
    shapes_.push_back(std::move(s));
    if (!order)
        shape_of_[key] = idx;
    return idx;
}

uneven_plan::uneven_plan(const std::vector<long long>& lengths, bool autotune) : lengths_(lengths)
{
    offsets_.resize(lengths.size());
    for (size_t i = 0; i < lengths.size(); i++)
    {
        if (lengths[i] < 1)
            throw std::invalid_argument("every signal length must be at least 1");
        offsets_[i] = total_;
        total_ += lengths[i];
    }
    check(cudaStreamCreateWithFlags(&cap_, cudaStreamNonBlocking), "create stream");
    derr_.alloc(sizeof(int));
    check(cudaMemset(derr_.get(), 0, sizeof(int)), "clear error flag");

    // autotuner for the one-CTA lengths present: time candidate radix orders and tiles on a synthetic batch
    // of that length alone, keep the fastest for the process
    if (autotune)
    {
        std::vector<long long> todo;
        for (long long n : lengths)
        {
            int ts = 0;
            if (n > 1 && fits_one_cta(n, factor_radices(n), ts))
                todo.push_back(n);
        }
        std::sort(todo.begin(), todo.end());
        todo.erase(std::unique(todo.begin(), todo.end()), todo.end());
        dbuf tin, tout, tffts, tjobs, titems, toffs, tq;
        const long long tune_elems = 1 << 20;
        tin.alloc(size_t(tune_elems) * 8);
        tout.alloc(size_t(tune_elems) * 8);
        check(cudaMemset(tin.get(), 0, tin.size()), "clear tuning input");
        tq.alloc(sizeof(int));
        cudaEvent_t e0, e1;
        check(cudaEventCreate(&e0), "event");
        check(cudaEventCreate(&e1), "event");
        for (long long n : todo)
        {
            {
                std::lock_guard<std::mutex> g(g_tune_mu);
                if (g_tune.count(n))
                    continue;
            }
            float best = 1e30f;
            std::pair<std::vector<int>, int> best_cfg(factor_radices(n), 0);
            for (const auto& order : candidate_orders(n))
            {
                int ts = 0;
                if (!fits_one_cta(n, order, ts))
                    continue;
                block_program<float> p;
                p.build(int(n), CT_NONE, &order, 16);
                const int smax = std::max(1, std::min({ kUnevenThreads / p.ts, uneven_max_smem() / (p.gstride * 8),
                                                        kUnevenMaxSpc }));
                for (int spc : { smax, std::max(1, smax / 2) })
                {
                    const long long nsig = std::max<long long>(spc, std::min<long long>(4096, tune_elems / n));
                    std::vector<long long> offs(nsig);
                    for (long long s = 0; s < nsig; s++)
                        offs[s] = s * n;
                    std::vector<uneven_item> its;
                    for (long long s = 0; s < nsig; s += spc)
                        its.push_back({ 0, int(s), int(std::min<long long>(spc, nsig - s)) });
                    uneven_fft f{ p.desc, p.tw.get(), int(n), p.ts, p.gstride, make_fast_div(uint32_t(n)) };
                    uneven_job j{};
                    j.mode = UM_DIRECT;
                    j.fft  = 0;
                    j.n    = int(n);
                    j.wait = -1;
                    j.done = -1;
                    tffts.upload(&f, sizeof(f));
                    tjobs.upload(&j, sizeof(j));
                    titems.upload(its.data(), its.size() * sizeof(uneven_item));
                    toffs.upload(offs.data(), offs.size() * sizeof(long long));
                    uneven_launch L{ static_cast<uneven_fft*>(tffts.get()), static_cast<uneven_job*>(tjobs.get()),
                                     static_cast<uneven_item*>(titems.get()), static_cast<long long*>(toffs.get()),
                                     int(its.size()), static_cast<int*>(tq.get()), nullptr,
                                     static_cast<int*>(derr_.get()), tin.get(), tout.get(), nullptr, 0 };
                    const int smem = spc * p.gstride * 8;
                    const int grid = std::min<int>(int(its.size()), 152);
                    for (int rep = 0; rep < 4; rep++)
                    {
                        check(cudaMemset(tq.get(), 0, sizeof(int)), "clear queue");
                        if (rep == 1)
                            check(cudaEventRecord(e0), "event");
                        check(launch_uneven_f32(L, smem, grid, nullptr), "tune");
                    }
                    float ms = 0;
                    check(cudaEventRecord(e1), "event");
                    check(cudaEventSynchronize(e1), "tune");
                    check(cudaEventElapsedTime(&ms, e0, e1), "tune");
                    if (ms / float(nsig) < best)
                    {
                        best     = ms / float(nsig);
                        best_cfg = { order, spc };
                    }
                }
            }
            std::lock_guard<std::mutex> g(g_tune_mu);
            g_tune[n] = best_cfg;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }

    // jobs and items.  Stage s of every signal is listed after all of stage s-1 (stage 0: whole signals and
    // first column passes), each stage heaviest first.
    std::vector<uneven_job> jobs;
    std::vector<std::vector<uneven_item>> stage_items(4);
    std::vector<std::vector<double>> stage_cost(4);
    std::vector<long long> offs;
    long long scratch_elems = 0;
    auto add_item = [&](int stage, const uneven_item& it, double cost)
    {
        stage_items[stage].push_back(it);
        stage_cost[stage].push_back(cost);
    };
    auto tables = [&]() -> dbuf&
    {
        tables_.emplace_back(new dbuf);
        return *tables_.back();
    };
    // one-CTA lengths: a job per length over its signals
    std::map<long long, std::vector<int>> by_len;
    for (size_t i = 0; i < lengths.size(); i++)
        by_len[lengths[i]].push_back(int(i));
    for (auto& kv : by_len)
    {
        const long long n = kv.first;
        const auto& sig   = kv.second;
        const auto rad    = factor_radices(n);
        int ts            = 0;
        const bool direct = n == 1 || fits_one_cta(n, rad, ts);
        long long m       = n;
        if (!direct && rad.empty())
        {
            // Bluestein convolution length: the smallest power of two >= 2n - 1 (the smallest 7-smooth one
            // is up to 2x shorter, but its radix-3/5/7 passes cost as much in this kernel: measured the same)
            m = 1;
            while (m < 2 * n - 1)
                m <<= 1;
        }
        if (direct || (rad.empty() && fits_one_cta(m, factor_radices(m), ts)))
        {
            uneven_job j{};
            j.mode  = direct ? UM_DIRECT : UM_BLUE1;
            j.fft   = get_shape(m, kUnevenThreads);
            j.n     = int(n);
            j.wait  = -1;
            j.done  = -1;
            if (!direct)
            {
                dbuf& ch = tables();
                dbuf& bh = tables();
                bluestein_tables<float>(n, m, ch, bh);
                j.chirp = ch.get();
                j.bhat  = bh.get();
                n_blue1_ += int(sig.size());
            }
            else
                n_direct_ += int(sig.size());
            const shape& sh = *shapes_[j.fft];
            int spc = std::max(1, std::min({ kUnevenThreads / sh.ts, uneven_max_smem() / (sh.prog.gstride * 8),
                                             kUnevenMaxSpc }));
            {
                std::lock_guard<std::mutex> g(g_tune_mu);
                auto f = g_tune.find(m);
                if (f != g_tune.end() && f->second.second > 0)
                    spc = std::min(spc, f->second.second);
            }
            const int jid   = int(jobs.size());
            jobs.push_back(j);
            const int first = int(offs.size());
            for (int i : sig)
                offs.push_back(offsets_[i]);
            for (int s = 0; s < int(sig.size()); s += spc)
            {
                const int c = std::min(spc, int(sig.size()) - s);
                add_item(0, { jid, first + s, c }, double(c) * double(m) * std::log2(double(std::max<long long>(m, 2))) *
                                                       (direct ? 1.0 : 2.0));
            }
            smem_ = std::max(smem_, spc * sh.prog.gstride * 8);
            continue;
        }
        // long signals: four-step (smooth lengths) or four-step Bluestein (a large prime factor), per signal
        const bool blue = rad.empty();
        int n1 = 0, n2 = 0;
        if (!split_of(m, n1, n2))
            throw std::invalid_argument("uneven batch: length " + std::to_string(n) + " is not supported");
        const int f1 = get_shape(n1, kUnevenThreads), f2 = get_shape(n2, kUnevenThreads);
        const int S1 = tile_of(n1, shapes_[f1]->ts), S2 = tile_of(n2, shapes_[f2]->ts);
        smem_        = std::max({ smem_, S1 * shapes_[f1]->prog.gstride * 8, S2 * shapes_[f2]->prog.gstride * 8 });
        // W_m^k two-level table
        int lb = 0;
        while ((1LL << (2 * lb)) < m)
            lb++;
        const long long nb = 1LL << lb, na = (m + nb - 1) / nb;
        std::vector<std::complex<float>> A(na), B(nb);
        for (long long i = 0; i < na; i++)
        {
            const auto w = twiddle(i * nb, m);
            A[i]         = { float(w.real()), float(w.imag()) };
        }
        for (long long i = 0; i < nb; i++)
        {
            const auto w = twiddle(i, m);
            B[i]         = { float(w.real()), float(w.imag()) };
        }
        dbuf& tA = tables();
        dbuf& tB = tables();
        tA.upload(A.data(), A.size() * sizeof(A[0]));
        tB.upload(B.data(), B.size() * sizeof(B[0]));
        const void *chirp = nullptr, *bhat = nullptr;
        if (blue)
        {
            dbuf& ch = tables();
            dbuf& bh = tables();
            bluestein_tables<float>(n, m, ch, bh);
            chirp = ch.get();
            bhat  = bh.get();
        }
        const int ncol = (n2 + S1 - 1) / S1, nrow = (n1 + S2 - 1) / S2;
        const double c1 = double(S1) * n1 * std::log2(double(n1)), c2 = double(S2) * n2 * std::log2(double(n2));
        for (int i : sig)
        {
            const int base = ncounters_;
            ncounters_ += blue ? 3 : 1;
            const long long sc = scratch_elems;
            scratch_elems += blue ? 2 * m : m;
            auto stage_job = [&](int mode, int src, long long soff, int dst, long long doff, int pre, int post,
                                 bool first, bool last, int wait, int need, int done)
            {
                uneven_job j{};
                j.mode    = mode;
                j.fft     = mode == UM_COL ? f1 : f2;
                j.n       = mode == UM_COL ? n1 : n2;
                j.n1      = n1;
                j.n2      = n2;
                j.src     = src;
                j.dst     = dst;
                j.src_off = soff;
                j.dst_off = doff;
                j.pre     = pre;
                j.post    = post;
                j.first   = first;
                j.last    = last;
                j.nvalid  = n;
                j.chirp   = chirp;
                j.bhat    = bhat;
                j.twA     = tA.get();
                j.twB     = tB.get();
                j.lbits   = lb;
                j.wait    = wait;
                j.need    = need;
                j.done    = done;
                jobs.push_back(j);
                return int(jobs.size()) - 1;
            };
            const long long off = offsets_[i];
            if (!blue)
            {
                const int jc = stage_job(UM_COL, 0, off, 2, sc, 0, 0, true, false, -1, 0, base);
                const int jr = stage_job(UM_ROW, 2, sc, 1, off, 0, 0, false, true, base, ncol, -1);
                for (int c = 0; c < ncol; c++)
                    add_item(0, { jc, c * S1, S1 }, c1);
                for (int r = 0; r < nrow; r++)
                    add_item(1, { jr, r * S2, S2 }, c2);
                n_fourstep_++;
            }
            else
            {
                // convolution: (x chirp) -> FFT_m -> conj(. bhat) -> FFT_m -> conj(.) chirp, in four stages
                const int j0 = stage_job(UM_COL, 0, off, 2, sc, 1, 0, true, false, -1, 0, base);
                const int j1 = stage_job(UM_ROW, 2, sc, 2, sc + m, 0, 1, false, false, base, ncol, base + 1);
                const int j2 = stage_job(UM_COL, 2, sc + m, 2, sc, 0, 0, false, false, base + 1, nrow, base + 2);
                const int j3 = stage_job(UM_ROW, 2, sc, 1, off, 0, 2, false, true, base + 2, ncol, -1);
                for (int c = 0; c < ncol; c++)
                {
                    add_item(0, { j0, c * S1, S1 }, c1);
                    add_item(2, { j2, c * S1, S1 }, c1);
                }
                for (int r = 0; r < nrow; r++)
                {
                    add_item(1, { j1, r * S2, S2 }, c2);
                    add_item(3, { j3, r * S2, S2 }, c2);
                }
                n_blue_fs_++;
            }
        }
    }
    std::vector<uneven_item> items;
    for (int s = 0; s < 4; s++)
    {
        std::vector<size_t> idx(stage_items[s].size());
        for (size_t i = 0; i < idx.size(); i++)
            idx[i] = i;
        std::stable_sort(idx.begin(), idx.end(),
                         [&](size_t x, size_t y) { return stage_cost[s][x] > stage_cost[s][y]; });
        for (size_t i : idx)
            items.push_back(stage_items[s][i]);
    }
    nitems_ = int(items.size());
    std::vector<uneven_fft> ffts;
    for (auto& sp : shapes_)
        ffts.push_back({ sp->prog.desc, sp->prog.tw.get(), sp->prog.n, sp->ts, sp->prog.gstride,
                         make_fast_div(uint32_t(std::max(1, sp->prog.n))) });
    if (!ffts.empty())
        dffts_.upload(ffts.data(), ffts.size() * sizeof(uneven_fft));
    if (!jobs.empty())
        djobs_.upload(jobs.data(), jobs.size() * sizeof(uneven_job));
    if (!items.empty())
        ditems_.upload(items.data(), items.size() * sizeof(uneven_item));
    if (!offs.empty())
        doffsets_.upload(offs.data(), offs.size() * sizeof(long long));
    dqueue_.alloc(sizeof(int));
    dcounters_.alloc(size_t(std::max(1, ncounters_)) * sizeof(int));
    if (scratch_elems)
        scratch_.alloc(size_t(scratch_elems) * 8);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    grid_ = std::max(1, std::min(nitems_, sms));
    smem_ = std::max(smem_, 1024);
}

uneven_plan::~uneven_plan()
{
    if (gexec_)
        cudaGraphExecDestroy(gexec_);
    if (cap_)
        cudaStreamDestroy(cap_);
}

void uneven_plan::enqueue(void* out, const void* in, bool inverse, cudaStream_t st)
{
    if (!nitems_)
        return;
    check(cudaMemsetAsync(dqueue_.get(), 0, sizeof(int), st), "clear work queue");
    if (ncounters_)
        check(cudaMemsetAsync(dcounters_.get(), 0, size_t(ncounters_) * sizeof(int), st), "clear stage counters");
    uneven_launch L{ static_cast<uneven_fft*>(dffts_.get()), static_cast<uneven_job*>(djobs_.get()),
                     static_cast<uneven_item*>(ditems_.get()), static_cast<long long*>(doffsets_.get()), nitems_,
                     static_cast<int*>(dqueue_.get()), static_cast<int*>(dcounters_.get()),
                     static_cast<int*>(derr_.get()), in, out, scratch_.get(), inverse ? 1 : 0, wait_limit(),
                     unreachable_ ? 1 : 0 };
    check(launch_uneven_f32(L, smem_, grid_, st), "launch uneven batch");
}

void uneven_plan::execute(void* out, const void* in, bool inverse, cudaStream_t st)
{
    if (!gexec_ || gin_ != in || gout_ != out || ginv_ != inverse || gspins_ != wait_limit() ||
        gunreach_ != unreachable_)
    {
        if (gexec_)
        {
            cudaGraphExecDestroy(gexec_);
            gexec_ = nullptr;
        }
        // the kernel's attributes are set outside the capture by one eager run
        enqueue(out, in, inverse, cap_);
        check(cudaStreamSynchronize(cap_), "uneven batch");
        cudaGraph_t g = nullptr;
        check(cudaStreamBeginCapture(cap_, cudaStreamCaptureModeThreadLocal), "begin capture");
        try
        {
            enqueue(out, in, inverse, cap_);
        }
        catch (...)
        {
            cudaStreamEndCapture(cap_, &g);
            if (g)
                cudaGraphDestroy(g);
            throw;
        }
        check(cudaStreamEndCapture(cap_, &g), "end capture");
        const cudaError_t e = cudaGraphInstantiate(&gexec_, g, 0);
        cudaGraphDestroy(g);
        check(e, "instantiate graph");
        gin_      = in;
        gout_     = out;
        ginv_     = inverse;
        gspins_   = wait_limit();
        gunreach_ = unreachable_;
    }
    check(cudaGraphLaunch(gexec_, st), "launch graph");
}

void uneven_plan::check_device_error() const
{
    int v = 0;
    check(cudaMemcpy(&v, derr_.get(), sizeof(int), cudaMemcpyDeviceToHost), "read error flag");
    if (v)
    {
        cudaMemset(derr_.get(), 0, sizeof(int));
        throw cuda_error("an uneven-batch tile gave up waiting for the stage it depends on (device error flag)");
    }
}

void uneven_plan::execute_per_signal(void* out, const void* in, bool inverse, cudaStream_t st)
{
    // the plain form: a regular plan per distinct length, one execution per signal
    for (size_t i = 0; i < lengths_.size(); i++)
    {
        const long long n = lengths_[i];
        auto f            = engines_.find(n);
        if (f == engines_.end())
            f = engines_.emplace(n, std::unique_ptr<complex_engine<float>>(new complex_engine<float>(n))).first;
        const long long need = f->second->scratch_elems(1);
        if (need * 8 > (long long)plain_scratch_.size())
        {
            check(cudaStreamSynchronize(st), "plain form");
            plain_scratch_.alloc(size_t(need) * 8);
        }
        f->second->execute(static_cast<char*>(out) + offsets_[i] * 8, static_cast<const char*>(in) + offsets_[i] * 8, 1,
                           n, n, inverse, plain_scratch_.get(), st);
    }
}

std::string uneven_plan::describe() const
{
    std::ostringstream s;
    s << "uneven batch: " << lengths_.size() << " signals in " << nitems_ << " work items on " << grid_
      << " persistent CTAs (" << n_direct_ << " one-CTA, " << n_blue1_ << " one-CTA Bluestein, " << n_fourstep_
      << " four-step, " << n_blue_fs_ << " four-step Bluestein)";
    return s.str();
}

} // namespace kfr_gpu
