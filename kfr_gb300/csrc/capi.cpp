// extern "C" layer: the reference's C API (include/kfr/capi.h, implemented in src/capi/capi.cpp) over the GPU
// engines.  Error convention of src/capi/capi.cpp:36-91: every entry point runs inside try_fn, which stores
// the exception text in a thread-local 256-byte buffer and returns the fallback (NULL / 0).
#include "kfr_capi.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <new>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>
#include <stdexcept>
#include <string>

#include "adjoint.hpp"
#include "conv.hpp"
#include "convolve.hpp"
#include "md.hpp"
#include "uneven.hpp"
#include "plan.hpp"

using namespace kfr_gpu;

namespace
{

thread_local std::array<char, 256> g_last_error{};

void reset_error() { g_last_error.fill(0); }

void set_error(const char* s)
{
    const size_t n = std::min(std::strlen(s), g_last_error.size() - 1);
    std::memcpy(g_last_error.data(), s, n);
    std::fill(g_last_error.begin() + n, g_last_error.end(), 0);
}

template <typename Fn, typename R>
R try_fn(Fn&& fn, R fallback)
{
    try
    {
        R r = fn();
        reset_error();
        return r;
    }
    catch (std::exception& e)
    {
        set_error(e.what());
    }
    catch (...)
    {
        set_error("(unknown exception)");
    }
    return fallback;
}

template <typename Fn>
void try_void(Fn&& fn)
{
    try
    {
        fn();
        reset_error();
    }
    catch (std::exception& e)
    {
        set_error(e.what());
    }
    catch (...)
    {
        set_error("(unknown exception)");
    }
}

// ---------------------------------------------------------------------------------------------------
// Plan objects behind the opaque handles.  A tag word guards against NULL or mismatched handles.
// ---------------------------------------------------------------------------------------------------

enum : uint32_t
{
    TAG_DFT_F32  = 0x31465444u,
    TAG_DFT_F64  = 0x32465444u,
    TAG_REAL_F32 = 0x31455244u,
    TAG_REAL_F64 = 0x32455244u,
    TAG_DCT_F32  = 0x31544344u,
    TAG_DCT_F64  = 0x32544344u,
    TAG_FLT_F32  = 0x31544c46u,
    TAG_FLT_F64  = 0x32544c46u,
    TAG_UNEVEN   = 0x31564e55u,
};

// Streams and per-stream buffers of the pipelined host-to-host path (see run_chunked).
constexpr int kPipeStreams = 3;
struct pipe_set
{
    cudaStream_t s[kPipeStreams] = {};
    dbuf in[kPipeStreams], out[kPipeStreams], scr[kPipeStreams];
    pipe_set()
    {
        for (auto& x : s)
            check(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking), "create stream");
    }
    ~pipe_set()
    {
        for (auto x : s)
            if (x)
                cudaStreamDestroy(x);
    }
};

struct plan_base
{
    uint32_t tag;
    std::mutex mu;     // guards the plan-owned staging and scratch buffers
    dbuf stage_in, stage_out, scratch;
    std::unique_ptr<pipe_set> pipes;
    explicit plan_base(uint32_t t) : tag(t) {}
    virtual ~plan_base() { tag = 0; }
};

template <typename T>
struct tags;
template <>
struct tags<float>
{
    static constexpr uint32_t dft = TAG_DFT_F32, real = TAG_REAL_F32, dct = TAG_DCT_F32, flt = TAG_FLT_F32;
};
template <>
struct tags<double>
{
    static constexpr uint32_t dft = TAG_DFT_F64, real = TAG_REAL_F64, dct = TAG_DCT_F64, flt = TAG_FLT_F64;
};

// Progressive execution (include/kfr/dft/fft.hpp:393-439; src/dft/fft-impl.hpp:2025-2064): the reference
// runs one stage per step; here a step is one kernel launch of the plan.  progressive_start records one
// execution with the given buffers by stream capture (nothing runs) and orders the recorded nodes; step i
// replays the i-th kernel launch (and any copy or memset recorded before it) and waits for it.
struct recorded_launches
{
    cudaGraph_t graph = nullptr;
    std::vector<std::vector<cudaGraphNode_t>> steps; // per step: the nodes before a kernel, then the kernel

    recorded_launches() = default;
    recorded_launches(const recorded_launches&) = delete;
    recorded_launches& operator=(const recorded_launches&) = delete;
    ~recorded_launches()
    {
        if (graph)
            cudaGraphDestroy(graph);
    }

    // Records fn(stream) by capture on `st` and splits the nodes (a chain) into steps.
    template <typename Fn>
    void record(cudaStream_t st, Fn&& fn)
    {
        check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
        try
        {
            fn(st);
        }
        catch (...)
        {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(st, &g);
            if (g)
                cudaGraphDestroy(g);
            throw;
        }
        check(cudaStreamEndCapture(st, &graph), "end capture");
        size_t count = 0;
        check(cudaGraphGetNodes(graph, nullptr, &count), "graph nodes");
        std::vector<cudaGraphNode_t> nodes(count);
        if (count)
            check(cudaGraphGetNodes(graph, nodes.data(), &count), "graph nodes");
        // topological order of the recorded chain
        std::vector<cudaGraphNode_t> order;
        std::vector<char> done(count, 0);
        while (order.size() < count)
        {
            bool progress = false;
            for (size_t i = 0; i < count; i++)
            {
                if (done[i])
                    continue;
                size_t nd = 0;
                check(cudaGraphNodeGetDependencies(nodes[i], nullptr, nullptr, &nd), "graph dependencies");
                std::vector<cudaGraphNode_t> deps(nd);
                if (nd)
                    check(cudaGraphNodeGetDependencies(nodes[i], deps.data(), nullptr, &nd), "graph dependencies");
                bool ready = true;
                for (auto d : deps)
                    ready = ready && std::find(order.begin(), order.end(), d) != order.end();
                if (ready)
                {
                    order.push_back(nodes[i]);
                    done[i]  = 1;
                    progress = true;
                }
            }
            if (!progress)
                throw std::logic_error("progressive execution: recorded launches are not ordered");
        }
        std::vector<cudaGraphNode_t> cur;
        for (auto nd : order)
        {
            cur.push_back(nd);
            cudaGraphNodeType t;
            check(cudaGraphNodeGetType(nd, &t), "graph node type");
            if (t == cudaGraphNodeTypeKernel)
            {
                steps.push_back(cur);
                cur.clear();
            }
        }
        if (!cur.empty())
        {
            if (steps.empty())
                steps.push_back(cur);
            else
                steps.back().insert(steps.back().end(), cur.begin(), cur.end());
        }
        if (steps.empty())
            steps.emplace_back();
    }

    // Runs step i's nodes on st.
    void replay(size_t i, cudaStream_t st) const
    {
        for (auto nd : steps.at(i))
        {
            cudaGraphNodeType t;
            check(cudaGraphNodeGetType(nd, &t), "graph node type");
            if (t == cudaGraphNodeTypeKernel)
            {
                cudaKernelNodeParams p{};
                check(cudaGraphKernelNodeGetParams(nd, &p), "kernel node");
                check(cudaLaunchKernel(p.func, p.gridDim, p.blockDim, p.kernelParams, p.sharedMemBytes, st),
                      "progressive step launch");
            }
            else if (t == cudaGraphNodeTypeMemcpy)
            {
                cudaMemcpy3DParms p{};
                check(cudaGraphMemcpyNodeGetParams(nd, &p), "copy node");
                check(cudaMemcpy3DAsync(&p, st), "progressive step copy");
            }
            else if (t == cudaGraphNodeTypeMemset)
            {
                cudaMemsetParams p{};
                check(cudaGraphMemsetNodeGetParams(nd, &p), "memset node");
                if (p.elementSize != 1 && p.value != 0)
                    throw std::logic_error("progressive execution: unsupported memset");
                check(cudaMemset2DAsync(p.dst, p.pitch, int(p.value), p.width * p.elementSize, p.height, st),
                      "progressive step memset");
            }
            else if (t != cudaGraphNodeTypeEmpty)
                throw std::logic_error("progressive execution: unsupported recorded operation");
        }
    }
};

struct progressive_run
{
    cudaStream_t st = nullptr;
    recorded_launches rec;
    void* host_out = nullptr; // where the last step copies the result (host output), else null
    const void* dev_out = nullptr;
    size_t out_bytes = 0;
    progressive_run() { check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "create stream"); }
    ~progressive_run()
    {
        if (st)
            cudaStreamDestroy(st);
    }
};

// A complex plan is one-dimensional (complex_engine) or multi-dimensional (md_engine), like the reference's
// var_dft_plan over dft_plan / dft_plan_md (src/capi/capi.cpp:93-156).
template <typename T>
struct dft_obj : plan_base
{
    size_t n; // total number of complex values
    std::unique_ptr<complex_engine<T>> eng1;
    std::unique_ptr<md_engine<T>> md;
    std::unique_ptr<progressive_run> prog; // the progressive execution in progress, if any
    size_t prog_steps = 0;                 // steps of a progressive execution (0: not counted yet)
    explicit dft_obj(size_t n_) : plan_base(tags<T>::dft), n(n_), eng1(new complex_engine<T>((long long)n_)) {}
    dft_obj(size_t n_, int tensor_mode)
        : plan_base(tags<T>::dft), n(n_), eng1(new complex_engine<T>((long long)n_, tensor_mode))
    {
    }
    explicit dft_obj(const std::vector<long long>& shape) : plan_base(tags<T>::dft), n(0)
    {
        if (shape.size() == 1)
            eng1.reset(new complex_engine<T>(shape[0]));
        else
            md.reset(new md_engine<T>(shape));
        n = eng1 ? size_t(eng1->size()) : size_t(md->size());
    }
    long long scratch_elems(long long b) const { return eng1 ? eng1->scratch_elems(b) : md->scratch_elems(b); }
    void execute(void* o, const void* i, long long b, bool inv, void* s, cudaStream_t st) const
    {
        if (eng1)
            eng1->execute(o, i, b, (long long)n, (long long)n, inv, s, st);
        else
            md->execute(o, i, b, inv, s, st);
    }
    std::string describe() const { return eng1 ? eng1->describe() : md->describe(); }
    int launches(long long b) const { return eng1 ? eng1->launches(b) : md->launches(b); }
    void check_device_error() const
    {
        if (eng1)
            eng1->check_device_error();
        else
            md->check_device_error();
    }
};

// A real plan: one-dimensional (real_engine, CCs or Perm) or multi-dimensional (md_real_engine, CCs).
template <typename T>
struct real_obj : plan_base
{
    size_t n; // total number of reals
    bool ccs;
    std::unique_ptr<real_engine<T>> eng1;
    std::unique_ptr<md_real_engine<T>> md;
    real_obj(size_t n_, bool ccs_) : plan_base(tags<T>::real), n(n_), ccs(ccs_)
    {
        if (n_ % 2 != 0)
            throw std::logic_error("dft_plan_real requires size to be even");
        eng1.reset(new real_engine<T>((long long)n_));
    }
    real_obj(const std::vector<long long>& shape, bool real_out_is_enough) : plan_base(tags<T>::real), n(0), ccs(true)
    {
        if (shape.size() == 1)
        {
            if (shape[0] % 2 != 0)
                throw std::logic_error("dft_plan_real requires size to be even");
            eng1.reset(new real_engine<T>(shape[0]));
            n = size_t(shape[0]);
        }
        else
        {
            md.reset(new md_real_engine<T>(shape, real_out_is_enough));
            n = size_t(md->size());
        }
    }
    size_t clen() const { return md ? size_t(md->complex_size()) : (ccs ? n / 2 + 1 : n / 2); }
    long long scratch_elems(long long b) const { return eng1 ? eng1->scratch_elems(b) : md->scratch_elems(b); }
    void forward(void* o, const void* i, long long b, void* s, cudaStream_t st) const
    {
        if (eng1)
            eng1->forward(o, i, b, ccs, s, st);
        else
            md->forward(o, i, b, s, st);
    }
    void inverse(void* o, const void* i, long long b, void* s, cudaStream_t st) const
    {
        if (eng1)
            eng1->inverse(o, i, b, ccs, s, st);
        else
            md->inverse(o, i, b, s, st);
    }
    std::string describe() const { return eng1 ? eng1->describe() : md->describe(); }
    void check_device_error() const
    {
        if (eng1)
            eng1->check_device_error();
        else
            md->check_device_error();
    }
};

template <typename T>
struct dct_obj : plan_base
{
    size_t n;
    dct_engine<T> eng;
    explicit dct_obj(size_t n_) : plan_base(tags<T>::dct), n(n_), eng((long long)n_) {}
};

template <typename T>
struct filter_obj : plan_base
{
    conv_filter<T> f;
    filter_obj(const T* taps, size_t ntaps, size_t block, int channels = 1)
        : plan_base(tags<T>::flt), f(taps, ntaps, block, channels)
    {
    }
};

template <typename Obj>
Obj* as(void* h, uint32_t tag)
{
    if (!h)
        throw std::invalid_argument("plan is NULL");
    plan_base* b = static_cast<plan_base*>(h);
    if (b->tag != tag)
        throw std::invalid_argument("invalid or mismatched plan handle");
    return static_cast<Obj*>(b);
}

bool is_device_ptr(const void* p)
{
    if (!p)
        return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Page-locked host memory mapped into the device's address space (cudaHostAlloc / cudaHostRegister): its
// device-side address, or nullptr for any other pointer.
void* host_mapped(const void* p)
{
    if (!p)
        return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

bool overlap(const void* a, size_t an, const void* b, size_t bn)
{
    const char* x = static_cast<const char*>(a);
    const char* y = static_cast<const char*>(b);
    return x < y + bn && y < x + an;
}

// Runs `fn(dout, din, scratch, stream)` with host buffers staged through plan-owned device memory.
// stream == nullptr: synchronous on the legacy default stream, host or device pointers.
// stream != nullptr: enqueued only; in/out must be device pointers.
template <typename Fn>
void run(plan_base& pl, void* out, size_t out_bytes, const void* in, size_t in_bytes, uint8_t* temp,
         size_t scratch_bytes, void* stream, bool copy_aliased_input, Fn&& fn)
{
    if ((!out && out_bytes) || (!in && in_bytes))
        throw std::invalid_argument("NULL data pointer");
    const bool in_dev  = is_device_ptr(in);
    const bool out_dev = is_device_ptr(out);
    cudaStream_t st    = static_cast<cudaStream_t>(stream);
    if (stream && (!in_dev || !out_dev))
        throw std::invalid_argument("stream-ordered execution needs device pointers for in and out");
    std::unique_lock<std::mutex> lock(pl.mu);
    const void* din = in;
    void* dout      = out;
    if (!in_dev)
    {
        pl.stage_in.ensure(in_bytes);
        check(cudaMemcpyAsync(pl.stage_in.get(), in, in_bytes, cudaMemcpyHostToDevice, st), "copy input to device");
        din = pl.stage_in.get();
    }
    else if (copy_aliased_input && out_dev && overlap(in, in_bytes, out, out_bytes))
    {
        pl.stage_in.ensure(in_bytes);
        check(cudaMemcpyAsync(pl.stage_in.get(), in, in_bytes, cudaMemcpyDeviceToDevice, st), "copy aliased input");
        din = pl.stage_in.get();
    }
    if (!out_dev)
    {
        pl.stage_out.ensure(out_bytes);
        dout = pl.stage_out.get();
    }
    void* scr = nullptr;
    if (scratch_bytes)
    {
        if (temp && is_device_ptr(temp))
            scr = temp;
        else
        {
            pl.scratch.ensure(scratch_bytes);
            scr = pl.scratch.get();
        }
    }
    fn(dout, din, scr, st);
    check(cudaGetLastError(), "kernel launch");
    if (!out_dev)
        check(cudaMemcpyAsync(out, dout, out_bytes, cudaMemcpyDeviceToHost, st), "copy result to host");
    if (!stream)
        check(cudaStreamSynchronize(st), "execute");
}

// Host buffers on both sides of a synchronous call of a batch-separable transform: the batch runs as a
// pipeline of chunks (up to about 16 MiB of input each) over kPipeStreams streams, so that copying chunk c+1
// in, transforming chunk c and copying chunk c-1 out overlap (the two copy directions and the kernels run
// concurrently).  The first chunks grow from a quarter of that size and the last ones shrink back to it, so
// that the copy-in before the first transform and the copy-out after the last one (when only one link
// direction is busy) stay short.  exec(dout, din, nb, scratch, stream) transforms nb signals; scr_bytes(nb)
// is its scratch.  Returns false (nothing done) when the call does not qualify: device pointers, a caller
// stream, or a batch too small to split.
template <typename Exec, typename Scr>
bool run_chunked(plan_base& pl, void* out, size_t out_per, const void* in, size_t in_per, size_t batch, void* stream,
                 Scr&& scr_bytes, Exec&& exec)
{
    if (stream || !out || !in || batch < 2 || is_device_ptr(in) || is_device_ptr(out))
        return false;
    const size_t per   = std::max(in_per, out_per);
    const size_t chunk = std::max<size_t>(1, std::min<size_t>(batch, (size_t(16) << 20) / std::max<size_t>(per, 1)));
    if ((batch + chunk - 1) / chunk < 2)
        return false;
    // chunk boundaries: sizes chunk/4, chunk/2, chunk, ..., chunk, chunk/2, chunk/4 (each at least one signal)
    std::vector<size_t> bounds{ 0 };
    {
        const size_t q = std::max<size_t>(1, chunk / 4), h = std::max<size_t>(1, chunk / 2);
        const size_t ramp = 2 * (q + h);
        std::vector<size_t> sizes;
        if (batch >= 2 * ramp + chunk)
        {
            sizes = { q, h };
            size_t mid = batch - 2 * (q + h);
            for (; mid > 0; mid -= std::min(mid, chunk))
                sizes.push_back(std::min(mid, chunk));
            sizes.push_back(h);
            sizes.push_back(q);
        }
        else
            for (size_t left = batch; left > 0; left -= std::min(left, chunk))
                sizes.push_back(std::min(left, chunk));
        for (size_t z : sizes)
            bounds.push_back(bounds.back() + z);
    }
    const size_t nchunks = bounds.size() - 1;
    std::unique_lock<std::mutex> lock(pl.mu);
    if (!pl.pipes)
        pl.pipes.reset(new pipe_set());
    pipe_set& P      = *pl.pipes;
    const size_t scr = scr_bytes((long long)chunk);
    for (int k = 0; k < kPipeStreams; k++)
    {
        P.in[k].ensure(chunk * in_per);
        P.out[k].ensure(chunk * out_per);
        if (scr)
            P.scr[k].ensure(scr);
    }
    const char* hin = static_cast<const char*>(in);
    char* hout      = static_cast<char*>(out);
    for (size_t c = 0; c < nchunks; c++)
    {
        const int k       = int(c % kPipeStreams);
        const size_t b0   = bounds[c];
        const size_t nb   = bounds[c + 1] - bounds[c];
        cudaStream_t st   = P.s[k];
        check(cudaMemcpyAsync(P.in[k].get(), hin + b0 * in_per, nb * in_per, cudaMemcpyHostToDevice, st),
              "copy input to device");
        exec(P.out[k].get(), P.in[k].get(), (long long)nb, scr ? P.scr[k].get() : nullptr, st);
        check(cudaGetLastError(), "kernel launch");
        check(cudaMemcpyAsync(hout + b0 * out_per, P.out[k].get(), nb * out_per, cudaMemcpyDeviceToHost, st),
              "copy result to host");
    }
    for (auto st : P.s)
        check(cudaStreamSynchronize(st), "execute");
    return true;
}

template <typename T>
void* create_dft(size_t n)
{
    return static_cast<plan_base*>(new dft_obj<T>(n));
}

// Synchronous call of a one-dimensional complex plan with page-locked host input and output: the kernels
// read the input and write the output across the host link themselves (zero-copy), so the link's two
// directions stay busy for the whole call with no staging, no chunk pipeline to fill and drain, and no
// device copy of the data.  Taken for the one-CTA lengths up to 4096 points, whose plain-load kernels hold
// many signals per CTA and keep the link busy (measured 256 -> 318 GB/s in + out at N=1000, 234 -> 273 at
// 2187, 238 -> 285 at 127); longer lengths (the one-signal-per-CTA kernels, Rader at 8191, the four-step's
// strided column reads) ran slower zero-copy than through the chunk pipeline and keep it.  False (nothing
// done) when the call does not qualify.
template <typename T>
bool run_zero_copy(dft_obj<T>& p, void* out, const void* in, size_t batch, uint8_t* temp, bool inverse, void* stream)
{
    using kind = typename complex_engine<T>::kind;
    if (stream || !p.eng1 || p.n < 2 || p.n > 4096)
        return false;
    const kind k = p.eng1->strategy();
    if (k != kind::smem && k != kind::rader_smem && k != kind::bluestein_smem)
        return false;
    void* dout      = host_mapped(out);
    const void* din = dout ? host_mapped(in) : nullptr;
    if (!dout || !din)
        return false;
    std::unique_lock<std::mutex> lock(p.mu);
    const size_t scr_bytes = size_t(p.scratch_elems((long long)batch)) * 2 * sizeof(T);
    void* scr              = nullptr;
    if (scr_bytes)
    {
        if (temp && is_device_ptr(temp))
            scr = temp;
        else
        {
            p.scratch.ensure(scr_bytes);
            scr = p.scratch.get();
        }
    }
    struct host_io_scope
    {
        const complex_engine<T>& e;
        explicit host_io_scope(const complex_engine<T>& x) : e(x) { e.set_host_io(true); }
        ~host_io_scope() { e.set_host_io(false); }
    } scope(*p.eng1);
    p.eng1->execute(dout, din, (long long)batch, (long long)p.n, (long long)p.n, inverse, scr, nullptr);
    check(cudaGetLastError(), "kernel launch");
    check(cudaStreamSynchronize(nullptr), "execute");
    return true;
}

template <typename T>
void exec_dft(void* h, size_t batch, void* out, const void* in, uint8_t* temp, bool inverse, void* stream)
{
    auto* p = as<dft_obj<T>>(h, tags<T>::dft);
    if (batch == 0 || p->n == 0)
        return;
    const size_t per   = p->n * 2 * sizeof(T);
    const size_t bytes = batch * per;
    const size_t scr   = size_t(p->scratch_elems((long long)batch)) * 2 * sizeof(T);
    if (run_zero_copy(*p, out, in, batch, temp, inverse, stream))
    {
        p->check_device_error();
        return;
    }
    if (!run_chunked(
            *p, out, per, in, per, batch, stream,
            [&](long long nb) { return size_t(p->scratch_elems(nb)) * 2 * sizeof(T); },
            [&](void* o, const void* i, long long nb, void* s, cudaStream_t st) { p->execute(o, i, nb, inverse, s, st); }))
        run(*p, out, bytes, in, bytes, temp, scr, stream, false,
            [&](void* o, const void* i, void* s, cudaStream_t st) { p->execute(o, i, (long long)batch, inverse, s, st); });
    if (!stream)
        p->check_device_error();
}

template <typename T>
void exec_real(void* h, size_t batch, void* out, const void* in, uint8_t* temp, bool inverse, void* stream)
{
    auto* p = as<real_obj<T>>(h, tags<T>::real);
    if (batch == 0)
        return;
    const size_t rbytes = batch * p->n * sizeof(T);
    const size_t cbytes = batch * p->clen() * 2 * sizeof(T);
    const size_t scr    = size_t(p->scratch_elems((long long)batch)) * 2 * sizeof(T);
    const bool alias    = batch > 1 || p->md != nullptr;
    const auto scr_of   = [&](long long nb) { return size_t(p->scratch_elems(nb)) * 2 * sizeof(T); };
    if (!inverse)
    {
        if (!run_chunked(*p, out, cbytes / batch, in, rbytes / batch, batch, stream, scr_of,
                         [&](void* o, const void* i, long long nb, void* s, cudaStream_t st) { p->forward(o, i, nb, s, st); }))
            run(*p, out, cbytes, in, rbytes, temp, scr, stream, alias,
                [&](void* o, const void* i, void* s, cudaStream_t st) { p->forward(o, i, (long long)batch, s, st); });
    }
    else
    {
        if (!run_chunked(*p, out, rbytes / batch, in, cbytes / batch, batch, stream, scr_of,
                         [&](void* o, const void* i, long long nb, void* s, cudaStream_t st) { p->inverse(o, i, nb, s, st); }))
            run(*p, out, rbytes, in, cbytes, temp, scr, stream, alias,
                [&](void* o, const void* i, void* s, cudaStream_t st) { p->inverse(o, i, (long long)batch, s, st); });
    }
    if (!stream)
        p->check_device_error();
}

template <typename T>
void exec_dct(void* h, size_t batch, void* out, const void* in, uint8_t* temp, bool inverse, void* stream)
{
    auto* p = as<dct_obj<T>>(h, tags<T>::dct);
    if (batch == 0 || p->n == 0)
        return;
    const size_t per   = p->n * sizeof(T);
    const size_t bytes = batch * per;
    const size_t scr   = size_t(p->eng.scratch_elems((long long)batch)) * 2 * sizeof(T);
    if (!run_chunked(
            *p, out, per, in, per, batch, stream,
            [&](long long nb) { return size_t(p->eng.scratch_elems(nb)) * 2 * sizeof(T); },
            [&](void* o, const void* i, long long nb, void* s, cudaStream_t st) { p->eng.execute(o, i, nb, inverse, s, st); }))
        run(*p, out, bytes, in, bytes, temp, scr, stream, false,
            [&](void* o, const void* i, void* s, cudaStream_t st) { p->eng.execute(o, i, (long long)batch, inverse, s, st); });
    if (!stream)
        p->eng.check_device_error();
}

// ---------------------------------------------------------------------------------------------------
// Adjoints (adjoint.hpp): the same kernels as the transforms plus elementwise weighting.
// ---------------------------------------------------------------------------------------------------

template <typename T>
void adj_real(void* h, size_t batch, void* grad_in, const void* grad_out, bool of_inverse, void* stream)
{
    auto* p = as<real_obj<T>>(h, tags<T>::real);
    if (batch == 0)
        return;
    if (!p->eng1)
        throw std::invalid_argument("adjoints are provided for one-dimensional real plans");
    const long long b    = (long long)batch;
    const size_t rbytes  = batch * p->n * sizeof(T);
    const size_t spec    = batch * p->clen() * 2 * sizeof(T);
    const size_t escr    = size_t(p->scratch_elems(b)) * 2 * sizeof(T);
    if (!of_inverse)
    {
        // adjoint of r2c: c2r of the gradient with the interior bins halved (into scratch: the caller's
        // gradient stays untouched)
        run(*p, grad_in, rbytes, grad_out, spec, nullptr, spec + escr, stream, false,
            [&](void* o, const void* i, void* s, cudaStream_t st)
            {
                check(launch_spectrum_weight<T>(s, i, b, (long long)p->clen(), p->ccs, T(0.5), st), "weight spectrum");
                p->inverse(o, s, b, escr ? static_cast<char*>(s) + spec : nullptr, st);
            });
    }
    else
    {
        // adjoint of c2r: r2c of the gradient with the interior bins doubled
        run(*p, grad_in, spec, grad_out, rbytes, nullptr, escr, stream, true,
            [&](void* o, const void* i, void* s, cudaStream_t st)
            {
                p->forward(o, i, b, s, st);
                check(launch_spectrum_weight<T>(o, o, b, (long long)p->clen(), p->ccs, T(2), st), "weight spectrum");
            });
    }
}

template <typename T>
void adj_dct(void* h, size_t batch, T* grad_in, const T* grad_out, bool of_inverse, void* stream)
{
    auto* p = as<dct_obj<T>>(h, tags<T>::dct);
    if (batch == 0 || p->n == 0)
        return;
    const long long b   = (long long)batch, n = (long long)p->n;
    const size_t bytes  = batch * p->n * sizeof(T);
    const size_t escr   = size_t(p->eng.scratch_elems(b)) * 2 * sizeof(T);
    if (!of_inverse)
    {
        // DCT-II^T = DCT-III with X0 at full weight = the reference's inverse of g with g[0] doubled
        const size_t wb = (bytes + 255) / 256 * 256;
        run(*p, grad_in, bytes, grad_out, bytes, nullptr, wb + escr, stream, false,
            [&](void* o, const void* i, void* s, cudaStream_t st)
            {
                T* w = static_cast<T*>(s);
                check(launch_scale_first<T>(w, static_cast<const T*>(i), b, n, T(2), st), "scale X0");
                p->eng.execute(o, w, b, true, escr ? static_cast<char*>(s) + wb : nullptr, st);
            });
    }
    else
    {
        // (DCT-III with X0 halved)^T = DCT-II, then element 0 halved
        run(*p, grad_in, bytes, grad_out, bytes, nullptr, escr, stream, false,
            [&](void* o, const void* i, void* s, cudaStream_t st)
            {
                p->eng.execute(o, i, b, false, s, st);
                check(launch_scale_first<T>(static_cast<T*>(o), static_cast<const T*>(o), b, n, T(0.5), st), "scale X0");
            });
    }
}

template <typename T>
void fir_bwd(const T* taps, size_t ntaps, size_t channels, size_t n, const T* x, const T* grad_y, T* grad_x,
             T* grad_taps, void* stream)
{
    if (!taps || !x || !grad_y)
        throw std::invalid_argument("NULL data pointer");
    for (const void* q : { (const void*)taps, (const void*)x, (const void*)grad_y, (const void*)grad_x,
                           (const void*)grad_taps })
        if (q && !is_device_ptr(q))
            throw std::invalid_argument("FIR backward needs device pointers");
    fir_backward<T>(taps, (long long)ntaps, (long long)channels, (long long)n, x, grad_y, grad_x, grad_taps,
                    static_cast<cudaStream_t>(stream));
}

struct uneven_obj : plan_base
{
    uneven_plan plan;
    uneven_obj(const std::vector<long long>& lengths, bool tune) : plan_base(TAG_UNEVEN), plan(lengths, tune) {}
};

void exec_uneven(void* h, void* out, const void* in, bool inverse, void* stream, bool per_signal)
{
    auto* p = as<uneven_obj>(h, TAG_UNEVEN);
    if (p->plan.total() == 0)
        return;
    if (!out || !in || !is_device_ptr(out) || !is_device_ptr(in))
        throw std::invalid_argument("uneven batch execution needs device pointers");
    std::unique_lock<std::mutex> lock(p->mu);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (per_signal)
        p->plan.execute_per_signal(out, in, inverse, st);
    else
        p->plan.execute(out, in, inverse, st);
    check(cudaGetLastError(), "uneven batch");
    if (!stream)
    {
        check(cudaStreamSynchronize(st), "uneven batch");
        p->plan.check_device_error();
    }
}

template <typename T>
void filter_process(void* h, T* out, const T* in, size_t n)
{
    auto* p = as<filter_obj<T>>(h, tags<T>::flt);
    if (n == 0)
        return;
    const size_t bytes = n * size_t(p->f.channels()) * sizeof(T);
    run(*p, out, bytes, in, bytes, nullptr, 0, nullptr, true,
        [&](void* o, const void* i, void*, cudaStream_t st)
        { p->f.process(static_cast<T*>(o), static_cast<const T*>(i), n, st); });
}

void print_line(const std::string& s)
{
    std::printf("%s\n", s.c_str());
    std::fflush(stdout);
}

std::string& version_string()
{
    static std::string s = [] {
        int rt = 0;
        cudaRuntimeGetVersion(&rt);
        char buf[160];
        std::snprintf(buf, sizeof(buf), "KFR 7.0.1 gb300 sm_103a 64-bit (CUDA runtime %d.%d)", rt / 1000,
                      (rt % 1000) / 10);
        return std::string(buf);
    }();
    return s;
}

// Host allocations carry a small header: the pointer returned by malloc, the requested size, a reference
// count and whether the block is pinned.  The counting follows the reference's managed allocation
// (include/kfr/meta/memory.hpp:58-140): a block starts with one reference and is freed when the last one is
// released.
struct alloc_header
{
    void* base;
    size_t size;
    std::atomic<unsigned> refs;
    int pinned;
    int magic;
};
constexpr int kAllocMagic = 0x6b667241;

alloc_header* header_of(void* p)
{
    alloc_header* h = reinterpret_cast<alloc_header*>(p) - 1;
    if (h->magic != kAllocMagic)
        throw std::invalid_argument("pointer was not allocated by kfr_allocate");
    return h;
}

void* host_alloc(size_t size, size_t alignment)
{
    // the reference returns NULL for alignments of 0 or above 32768 (include/kfr/meta/memory.hpp:64-65)
    if (alignment == 0 || alignment > 32768 || (alignment & (alignment - 1)))
        throw std::invalid_argument("alignment must be a power of two between 1 and 32768");
    alignment         = std::max(alignment, alignof(alloc_header));
    const size_t total = size + alignment + sizeof(alloc_header);
    void* base         = std::malloc(total);
    if (!base)
        throw std::bad_alloc();
    uintptr_t p = (reinterpret_cast<uintptr_t>(base) + sizeof(alloc_header) + alignment - 1) & ~(uintptr_t(alignment) - 1);
    alloc_header* h = new (reinterpret_cast<alloc_header*>(p) - 1) alloc_header;
    h->base         = base;
    h->size         = size;
    h->refs.store(1);
    h->magic        = kAllocMagic;
    h->pinned       = 0;
    int ndev        = 0;
    if (size >= 4096 && cudaGetDeviceCount(&ndev) == cudaSuccess && ndev > 0)
    {
        if (cudaHostRegister(reinterpret_cast<void*>(p), size, cudaHostRegisterDefault) == cudaSuccess)
            h->pinned = 1;
        else
            cudaGetLastError();
    }
    else
        cudaGetLastError();
    return reinterpret_cast<void*>(p);
}

// Drops one reference; frees the block at zero.
void host_free(void* p)
{
    if (!p)
        return;
    alloc_header* h = header_of(p);
    if (--h->refs != 0)
        return;
    if (h->pinned)
    {
        cudaHostUnregister(p);
        cudaGetLastError();
    }
    h->magic = 0;
    void* base = h->base;
    h->~alloc_header();
    std::free(base);
}

// include/kfr/meta/memory.hpp:120-140
void* host_realloc(void* p, size_t new_size, size_t alignment)
{
    if (!p)
        return new_size ? host_alloc(new_size, alignment) : nullptr;
    const size_t old_size = header_of(p)->size;
    if (!new_size)
    {
        host_free(p);
        return nullptr;
    }
    void* q = host_alloc(new_size, alignment);
    std::memcpy(q, p, std::min(old_size, new_size));
    host_free(p);
    return q;
}

// init_shape (src/capi/capi.cpp:106-114)
std::vector<long long> to_shape(size_t dims, const unsigned* shape)
{
    if (dims && !shape)
        throw std::invalid_argument("shape is NULL");
    std::vector<long long> s(dims);
    for (size_t i = 0; i < dims; i++)
        s[i] = shape[i];
    return s;
}

// Whole-signal convolution with host or device pointers: host inputs and outputs are staged through
// stream-ordered device allocations on the legacy default stream, and the call synchronises.
template <typename T>
size_t convolve_any(void* out, const void* a, size_t na, const void* b, size_t nb, bool is_complex, int mode)
{
    if (na == 0 || nb == 0)
        return 0;
    if (!out || !a || !b)
        throw std::invalid_argument("NULL data pointer");
    const size_t esz  = (is_complex ? 2 : 1) * sizeof(T);
    const size_t olen = na + nb - 1;
    cudaStream_t st   = nullptr;
    const void* da    = a;
    const void* db    = b;
    void* dout        = out;
    std::vector<void*> owned;
    struct guard_t
    {
        std::vector<void*>& v;
        ~guard_t()
        {
            for (void* p : v)
                cudaFreeAsync(p, nullptr);
        }
    } guard{ owned };
    auto stage = [&](const void* src, size_t bytes) -> const void*
    {
        if (is_device_ptr(src))
            return src;
        void* d = nullptr;
        check(cudaMallocAsync(&d, bytes, st), "cudaMallocAsync");
        owned.push_back(d);
        check(cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, st), "copy input to device");
        return d;
    };
    da                 = stage(a, na * esz);
    db                 = stage(b, nb * esz);
    const bool out_dev = is_device_ptr(out);
    if (!out_dev)
    {
        void* d = nullptr;
        check(cudaMallocAsync(&d, olen * esz, st), "cudaMallocAsync");
        owned.push_back(d);
        dout = d;
    }
    convolve_device<T>(dout, da, (long long)na, db, (long long)nb, is_complex, mode, st);
    if (!out_dev)
        check(cudaMemcpyAsync(out, dout, olen * esz, cudaMemcpyDeviceToHost, st), "copy result to host");
    check(cudaStreamSynchronize(st), "convolve");
    return olen;
}

// autocorrelate: the upper half of correlate(a, a), lags 0 .. n-1 (include/kfr/dft/convolution.hpp:69-76)
template <typename T>
size_t autocorrelate_any(T* out, const T* a, size_t n)
{
    if (n == 0)
        return 0;
    std::vector<T> full;
    const bool out_dev = is_device_ptr(out);
    void* tmp          = nullptr;
    if (out_dev)
    {
        check(cudaMallocAsync(&tmp, (2 * n - 1) * sizeof(T), nullptr), "cudaMallocAsync");
        convolve_any<T>(tmp, a, n, a, n, false, 1);
        check(cudaMemcpy(out, static_cast<T*>(tmp) + (n - 1), n * sizeof(T), cudaMemcpyDeviceToDevice), "copy");
        cudaFreeAsync(tmp, nullptr);
        check(cudaStreamSynchronize(nullptr), "autocorrelate");
    }
    else
    {
        full.resize(2 * n - 1);
        convolve_any<T>(full.data(), a, n, a, n, false, 1);
        std::memcpy(out, full.data() + (n - 1), n * sizeof(T));
    }
    return n;
}

[[noreturn]] void not_built(const char* what)
{
    throw std::logic_error(std::string(what) + " is not part of the GPU DFT path in this build");
}

} // namespace

namespace
{
// A device address that is never dereferenced: progressive_total_steps records one execution with it to
// count the launches (recording runs nothing).  Aligned like a cudaMalloc allocation.
void* unused_device_address(int i) { return reinterpret_cast<void*>((uintptr_t(0x7f00) + uintptr_t(i)) << 32); }

template <typename T>
size_t progressive_total(void* plan)
{
    auto* p = as<dft_obj<T>>(plan, tags<T>::dft);
    std::unique_lock<std::mutex> lock(p->mu);
    if (!p->prog_steps)
    {
        cudaStream_t st = nullptr;
        check(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "create stream");
        try
        {
            recorded_launches rec;
            void* scr = p->scratch_elems(1) ? unused_device_address(2) : nullptr;
            rec.record(st, [&](cudaStream_t s)
                       { p->execute(unused_device_address(0), unused_device_address(1), 1, false, scr, s); });
            p->prog_steps = rec.steps.size();
        }
        catch (...)
        {
            cudaStreamDestroy(st);
            throw;
        }
        cudaStreamDestroy(st);
    }
    return p->prog_steps;
}

template <typename T>
size_t progressive_start(void* plan, void* out, const void* in, uint8_t* temp, bool inverse)
{
    auto* p = as<dft_obj<T>>(plan, tags<T>::dft);
    if (!out || !in)
        throw std::invalid_argument("NULL data pointer");
    const size_t bytes = p->n * 2 * sizeof(T);
    std::unique_lock<std::mutex> lock(p->mu);
    p->prog.reset(new progressive_run);
    progressive_run& r = *p->prog;
    const void* din    = in;
    void* dout         = out;
    if (!is_device_ptr(in))
    {
        p->stage_in.ensure(bytes);
        check(cudaMemcpy(p->stage_in.get(), in, bytes, cudaMemcpyHostToDevice), "copy input to device");
        din = p->stage_in.get();
    }
    if (!is_device_ptr(out))
    {
        p->stage_out.ensure(bytes);
        dout        = p->stage_out.get();
        r.host_out  = out;
        r.dev_out   = dout;
        r.out_bytes = bytes;
    }
    void* scr = nullptr;
    if (const size_t sb = size_t(p->scratch_elems(1)) * 2 * sizeof(T))
    {
        if (temp && is_device_ptr(temp))
            scr = temp;
        else
        {
            p->scratch.ensure(sb);
            scr = p->scratch.get();
        }
    }
    r.rec.record(r.st, [&](cudaStream_t st) { p->execute(dout, din, 1, inverse, scr, st); });
    return r.rec.steps.size();
}

template <typename T>
bool progressive_step(void* plan, size_t step)
{
    auto* p = as<dft_obj<T>>(plan, tags<T>::dft);
    std::unique_lock<std::mutex> lock(p->mu);
    if (!p->prog)
        throw std::logic_error("progressive_step before progressive_start");
    progressive_run& r = *p->prog;
    if (step >= r.rec.steps.size())
        throw std::invalid_argument("progressive step " + std::to_string(step) + " of " +
                                    std::to_string(r.rec.steps.size()));
    r.rec.replay(step, r.st);
    check(cudaStreamSynchronize(r.st), "progressive step");
    const bool more = step + 1 < r.rec.steps.size();
    if (!more)
    {
        if (r.host_out)
            check(cudaMemcpy(r.host_out, r.dev_out, r.out_bytes, cudaMemcpyDeviceToHost), "copy result to host");
        p->prog.reset();
        lock.unlock();
        p->check_device_error();
    }
    return more;
}

template <typename T>
void fft_multiply_dev(void* dest, const void* acc, const void* src1, const void* src2, size_t size, size_t batch,
                      bool shared, bool perm, void* stream)
{
    if (!size || !batch)
        return;
    for (const void* p : { (const void*)dest, acc, src1, src2 })
        if (p && !is_device_ptr(p))
            throw std::invalid_argument("fft_multiply needs device pointers");
    if (!dest || !src1 || !src2)
        throw std::invalid_argument("fft_multiply: NULL buffer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    check(launch_fft_multiply<T>(dest, acc, src1, src2, (long long)size, (long long)batch,
                                 shared ? 0LL : (long long)size, perm, st),
          "fft_multiply");
    if (!stream)
        check(cudaStreamSynchronize(st), "fft_multiply");
}

template <typename T>
size_t describe_into(void* plan, unsigned tag, char* buf, size_t size)
{
    return try_fn(
        [&]
        {
            const std::string d = as<dft_obj<T>>(plan, tag)->describe();
            if (buf && size)
            {
                const size_t n = std::min(size - 1, d.size());
                std::memcpy(buf, d.data(), n);
                buf[n] = 0;
            }
            return d.size();
        },
        size_t(0));
}
} // namespace

extern "C"
{

// ---- information ---------------------------------------------------------------------------------
KFR_API_SPEC const char* kfr_version_string(void) { return version_string().c_str(); }
KFR_API_SPEC uint32_t kfr_version(void) { return 70001; }
KFR_API_SPEC const char* kfr_enabled_archs(void) { return "sm_103a"; }
KFR_API_SPEC int kfr_current_arch(void)
{
    return try_fn(
        []
        {
            int dev = 0, ma = 0, mi = 0;
            check(cudaGetDevice(&dev), "cudaGetDevice");
            check(cudaDeviceGetAttribute(&ma, cudaDevAttrComputeCapabilityMajor, dev), "attribute");
            check(cudaDeviceGetAttribute(&mi, cudaDevAttrComputeCapabilityMinor, dev), "attribute");
            return ma * 10 + mi;
        },
        -1);
}
KFR_API_SPEC const char* kfr_last_error(void) { return g_last_error.data(); }

KFR_API_SPEC void* kfr_allocate(size_t size)
{
    return try_fn([&] { return host_alloc(size, KFR_DEFAULT_ALIGNMENT); }, (void*)nullptr);
}
KFR_API_SPEC void* kfr_allocate_aligned(size_t size, size_t alignment)
{
    return try_fn([&] { return host_alloc(size, alignment); }, (void*)nullptr);
}
KFR_API_SPEC void kfr_deallocate(void* ptr)
{
    try_void([&] { host_free(ptr); });
}
KFR_API_SPEC void* kfr_reallocate(void* ptr, size_t new_size)
{
    return try_fn([&] { return host_realloc(ptr, new_size, KFR_DEFAULT_ALIGNMENT); }, (void*)nullptr);
}
KFR_API_SPEC void* kfr_reallocate_aligned(void* ptr, size_t new_size, size_t alignment)
{
    return try_fn([&] { return host_realloc(ptr, new_size, alignment); }, (void*)nullptr);
}
KFR_API_SPEC void* kfr_add_ref(void* ptr)
{
    return try_fn(
        [&]
        {
            if (ptr)
                header_of(ptr)->refs++;
            return ptr;
        },
        (void*)nullptr);
}
KFR_API_SPEC void kfr_release(void* ptr)
{
    try_void([&] { host_free(ptr); });
}
KFR_API_SPEC size_t kfr_allocated_size(void* ptr)
{
    return try_fn([&] { return ptr ? header_of(ptr)->size : size_t(0); }, size_t(0));
}

// ---- complex DFT ---------------------------------------------------------------------------------
KFR_API_SPEC KFR_DFT_PLAN_F32* kfr_dft_create_plan_f32(size_t size)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_PLAN_F32*>(create_dft<float>(size)); },
                  (KFR_DFT_PLAN_F32*)nullptr);
}
KFR_API_SPEC KFR_DFT_PLAN_F64* kfr_dft_create_plan_f64(size_t size)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_PLAN_F64*>(create_dft<double>(size)); },
                  (KFR_DFT_PLAN_F64*)nullptr);
}
KFR_API_SPEC KFR_DFT_PLAN_F32* kfr_dft_create_2d_plan_f32(size_t size1, size_t size2)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_PLAN_F32*>(static_cast<plan_base*>(new dft_obj<float>(std::vector<long long>{ (long long)size1, (long long)size2 }))); },
                  (KFR_DFT_PLAN_F32*)nullptr);
}
KFR_API_SPEC KFR_DFT_PLAN_F32* kfr_dft_create_3d_plan_f32(size_t size1, size_t size2, size_t size3)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_PLAN_F32*>(static_cast<plan_base*>(new dft_obj<float>(std::vector<long long>{ (long long)size1, (long long)size2, (long long)size3 }))); },
                  (KFR_DFT_PLAN_F32*)nullptr);
}
KFR_API_SPEC KFR_DFT_PLAN_F32* kfr_dft_create_md_plan_f32(size_t dims, const unsigned* shape)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_PLAN_F32*>(static_cast<plan_base*>(new dft_obj<float>(to_shape(dims, shape)))); },
                  (KFR_DFT_PLAN_F32*)nullptr);
}
KFR_API_SPEC KFR_DFT_PLAN_F64* kfr_dft_create_2d_plan_f64(size_t size1, size_t size2)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_PLAN_F64*>(static_cast<plan_base*>(new dft_obj<double>(std::vector<long long>{ (long long)size1, (long long)size2 }))); },
                  (KFR_DFT_PLAN_F64*)nullptr);
}
KFR_API_SPEC KFR_DFT_PLAN_F64* kfr_dft_create_3d_plan_f64(size_t size1, size_t size2, size_t size3)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_PLAN_F64*>(static_cast<plan_base*>(new dft_obj<double>(std::vector<long long>{ (long long)size1, (long long)size2, (long long)size3 }))); },
                  (KFR_DFT_PLAN_F64*)nullptr);
}
KFR_API_SPEC KFR_DFT_PLAN_F64* kfr_dft_create_md_plan_f64(size_t dims, const unsigned* shape)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_PLAN_F64*>(static_cast<plan_base*>(new dft_obj<double>(to_shape(dims, shape)))); },
                  (KFR_DFT_PLAN_F64*)nullptr);
}
KFR_API_SPEC void kfr_dft_dump_f32(KFR_DFT_PLAN_F32* plan)
{
    try_void([&] { print_line(as<dft_obj<float>>(plan, TAG_DFT_F32)->describe()); });
}
KFR_API_SPEC void kfr_dft_dump_f64(KFR_DFT_PLAN_F64* plan)
{
    try_void([&] { print_line(as<dft_obj<double>>(plan, TAG_DFT_F64)->describe()); });
}
KFR_API_SPEC size_t kfr_dft_get_size_f32(KFR_DFT_PLAN_F32* plan)
{
    return try_fn([&] { return as<dft_obj<float>>(plan, TAG_DFT_F32)->n; }, size_t(0));
}
KFR_API_SPEC size_t kfr_dft_get_size_f64(KFR_DFT_PLAN_F64* plan)
{
    return try_fn([&] { return as<dft_obj<double>>(plan, TAG_DFT_F64)->n; }, size_t(0));
}
KFR_API_SPEC size_t kfr_dft_get_temp_size_batch_f32(KFR_DFT_PLAN_F32* plan, size_t batch)
{
    return try_fn([&] { return size_t(as<dft_obj<float>>(plan, TAG_DFT_F32)->scratch_elems(batch)) * 8; },
                  size_t(0));
}
KFR_API_SPEC size_t kfr_dft_get_temp_size_batch_f64(KFR_DFT_PLAN_F64* plan, size_t batch)
{
    return try_fn([&] { return size_t(as<dft_obj<double>>(plan, TAG_DFT_F64)->scratch_elems(batch)) * 16; },
                  size_t(0));
}
KFR_API_SPEC size_t kfr_dft_get_temp_size_f32(KFR_DFT_PLAN_F32* plan) { return kfr_dft_get_temp_size_batch_f32(plan, 1); }
KFR_API_SPEC size_t kfr_dft_get_temp_size_f64(KFR_DFT_PLAN_F64* plan) { return kfr_dft_get_temp_size_batch_f64(plan, 1); }
KFR_API_SPEC void kfr_dft_execute_f32(KFR_DFT_PLAN_F32* plan, kfr_c32* out, const kfr_c32* in, uint8_t* temp)
{
    try_void([&] { exec_dft<float>(plan, 1, out, in, temp, false, nullptr); });
}
KFR_API_SPEC void kfr_dft_execute_f64(KFR_DFT_PLAN_F64* plan, kfr_c64* out, const kfr_c64* in, uint8_t* temp)
{
    try_void([&] { exec_dft<double>(plan, 1, out, in, temp, false, nullptr); });
}
KFR_API_SPEC void kfr_dft_execute_inverse_f32(KFR_DFT_PLAN_F32* plan, kfr_c32* out, const kfr_c32* in, uint8_t* temp)
{
    try_void([&] { exec_dft<float>(plan, 1, out, in, temp, true, nullptr); });
}
KFR_API_SPEC void kfr_dft_execute_inverse_f64(KFR_DFT_PLAN_F64* plan, kfr_c64* out, const kfr_c64* in, uint8_t* temp)
{
    try_void([&] { exec_dft<double>(plan, 1, out, in, temp, true, nullptr); });
}
KFR_API_SPEC void kfr_dft_execute_batch_f32(KFR_DFT_PLAN_F32* plan, size_t batch, kfr_c32* out, const kfr_c32* in,
                                            uint8_t* temp, kfr_bool inverse, void* stream)
{
    try_void([&] { exec_dft<float>(plan, batch, out, in, temp, inverse, stream); });
}
KFR_API_SPEC void kfr_dft_execute_batch_f64(KFR_DFT_PLAN_F64* plan, size_t batch, kfr_c64* out, const kfr_c64* in,
                                            uint8_t* temp, kfr_bool inverse, void* stream)
{
    try_void([&] { exec_dft<double>(plan, batch, out, in, temp, inverse, stream); });
}
#define KFR_CONV_ENTRY(NAME, CT, T, CPLX, MODE)                                                             \
    KFR_API_SPEC size_t NAME(CT* out, const CT* a, size_t na, const CT* b, size_t nb)                        \
    {                                                                                                       \
        return try_fn([&] { return convolve_any<T>(out, a, na, b, nb, CPLX, MODE); }, size_t(0));           \
    }
KFR_CONV_ENTRY(kfr_convolve_f32, kfr_f32, float, false, 0)
KFR_CONV_ENTRY(kfr_convolve_f64, kfr_f64, double, false, 0)
KFR_CONV_ENTRY(kfr_convolve_c32, kfr_c32, float, true, 0)
KFR_CONV_ENTRY(kfr_convolve_c64, kfr_c64, double, true, 0)
KFR_CONV_ENTRY(kfr_correlate_f32, kfr_f32, float, false, 1)
KFR_CONV_ENTRY(kfr_correlate_f64, kfr_f64, double, false, 1)
KFR_CONV_ENTRY(kfr_correlate_c32, kfr_c32, float, true, 1)
KFR_CONV_ENTRY(kfr_correlate_c64, kfr_c64, double, true, 1)
#undef KFR_CONV_ENTRY
KFR_API_SPEC size_t kfr_autocorrelate_f32(kfr_f32* out, const kfr_f32* a, size_t n)
{
    return try_fn([&] { return autocorrelate_any<float>(out, a, n); }, size_t(0));
}
KFR_API_SPEC size_t kfr_autocorrelate_f64(kfr_f64* out, const kfr_f64* a, size_t n)
{
    return try_fn([&] { return autocorrelate_any<double>(out, a, n); }, size_t(0));
}
KFR_API_SPEC size_t kfr_dft_cache_size(void)
{
    return try_fn([&] { return plan_cache::instance().size(); }, size_t(0));
}
KFR_API_SPEC void kfr_dft_cache_clear(void)
{
    try_void([&] { plan_cache::instance().clear(); });
}

KFR_API_SPEC void kfr_fft_multiply_f32(kfr_c32* dest, const kfr_c32* src1, const kfr_c32* src2, size_t size,
                                       size_t batch, kfr_bool src2_shared, KFR_DFT_PACK_FORMAT fmt, void* stream)
{
    try_void([&] { fft_multiply_dev<float>(dest, nullptr, src1, src2, size, batch, src2_shared, fmt == Perm, stream); });
}
KFR_API_SPEC void kfr_fft_multiply_f64(kfr_c64* dest, const kfr_c64* src1, const kfr_c64* src2, size_t size,
                                       size_t batch, kfr_bool src2_shared, KFR_DFT_PACK_FORMAT fmt, void* stream)
{
    try_void([&] { fft_multiply_dev<double>(dest, nullptr, src1, src2, size, batch, src2_shared, fmt == Perm, stream); });
}
KFR_API_SPEC void kfr_fft_multiply_accumulate_f32(kfr_c32* dest, const kfr_c32* acc, const kfr_c32* src1,
                                                  const kfr_c32* src2, size_t size, size_t batch,
                                                  kfr_bool src2_shared, KFR_DFT_PACK_FORMAT fmt, void* stream)
{
    try_void(
        [&]
        {
            if (!acc)
                throw std::invalid_argument("fft_multiply_accumulate: NULL accumulator");
            fft_multiply_dev<float>(dest, acc, src1, src2, size, batch, src2_shared, fmt == Perm, stream);
        });
}
KFR_API_SPEC void kfr_fft_multiply_accumulate_f64(kfr_c64* dest, const kfr_c64* acc, const kfr_c64* src1,
                                                  const kfr_c64* src2, size_t size, size_t batch,
                                                  kfr_bool src2_shared, KFR_DFT_PACK_FORMAT fmt, void* stream)
{
    try_void(
        [&]
        {
            if (!acc)
                throw std::invalid_argument("fft_multiply_accumulate: NULL accumulator");
            fft_multiply_dev<double>(dest, acc, src1, src2, size, batch, src2_shared, fmt == Perm, stream);
        });
}
KFR_API_SPEC size_t kfr_dft_progressive_total_steps_f32(KFR_DFT_PLAN_F32* plan)
{
    return try_fn([&] { return progressive_total<float>(plan); }, size_t(0));
}
KFR_API_SPEC size_t kfr_dft_progressive_total_steps_f64(KFR_DFT_PLAN_F64* plan)
{
    return try_fn([&] { return progressive_total<double>(plan); }, size_t(0));
}
KFR_API_SPEC size_t kfr_dft_progressive_start_f32(KFR_DFT_PLAN_F32* plan, kfr_c32* out, const kfr_c32* in,
                                                  uint8_t* temp, kfr_bool inverse)
{
    return try_fn([&] { return progressive_start<float>(plan, out, in, temp, inverse != 0); }, size_t(0));
}
KFR_API_SPEC size_t kfr_dft_progressive_start_f64(KFR_DFT_PLAN_F64* plan, kfr_c64* out, const kfr_c64* in,
                                                  uint8_t* temp, kfr_bool inverse)
{
    return try_fn([&] { return progressive_start<double>(plan, out, in, temp, inverse != 0); }, size_t(0));
}
KFR_API_SPEC kfr_bool kfr_dft_progressive_step_f32(KFR_DFT_PLAN_F32* plan, size_t step)
{
    return try_fn([&] { return kfr_bool(progressive_step<float>(plan, step)); }, kfr_bool(0));
}
KFR_API_SPEC kfr_bool kfr_dft_progressive_step_f64(KFR_DFT_PLAN_F64* plan, size_t step)
{
    return try_fn([&] { return kfr_bool(progressive_step<double>(plan, step)); }, kfr_bool(0));
}
KFR_API_SPEC size_t kfr_dft_describe_f32(KFR_DFT_PLAN_F32* plan, char* buf, size_t size)
{
    return describe_into<float>(plan, TAG_DFT_F32, buf, size);
}
KFR_API_SPEC size_t kfr_dft_describe_f64(KFR_DFT_PLAN_F64* plan, char* buf, size_t size)
{
    return describe_into<double>(plan, TAG_DFT_F64, buf, size);
}
KFR_API_SPEC size_t kfr_dft_get_launch_count_f32(KFR_DFT_PLAN_F32* plan, size_t batch)
{
    return try_fn([&] { return size_t(as<dft_obj<float>>(plan, TAG_DFT_F32)->launches(batch)); }, size_t(0));
}
KFR_API_SPEC size_t kfr_dft_get_launch_count_f64(KFR_DFT_PLAN_F64* plan, size_t batch)
{
    return try_fn([&] { return size_t(as<dft_obj<double>>(plan, TAG_DFT_F64)->launches(batch)); }, size_t(0));
}

} // extern "C"

namespace kfr_gpu
{
// Body of kfr_dft_execute_static_scratch_f32 (static_scratch.cu owns the scratch array and passes its
// device address through `scratch_of`).  Nothing here allocates: no staging, no plan-owned scratch.
void run_static_scratch_f32(void* plan, size_t batch, void* out, const void* in, bool inverse, void* stream,
                            void* (*scratch_of)(), size_t scratch_limit)
{
    try_void(
        [&]
        {
            auto* p = as<dft_obj<float>>(plan, TAG_DFT_F32);
            if (batch == 0 || p->n == 0)
                return;
            if (!is_device_ptr(in) || !is_device_ptr(out))
                throw std::invalid_argument("kfr_dft_execute_static_scratch_f32 needs device pointers for in and out");
            const size_t need = size_t(p->scratch_elems((long long)batch)) * 2 * sizeof(float);
            if (need > scratch_limit)
                throw std::invalid_argument("kfr_dft_execute_static_scratch_f32: this plan and batch need " +
                                            std::to_string(need) + " bytes of scratch, more than the " +
                                            std::to_string(scratch_limit) + "-byte static scratch");
            // The per-device set-up runs on every call, so the first call on a device always does it,
            // whether or not this plan needs scratch.
            void* addr      = scratch_of();
            void* scr       = need ? addr : nullptr;
            cudaStream_t st = static_cast<cudaStream_t>(stream);
            p->execute(out, in, (long long)batch, inverse, scr, st);
            check(cudaGetLastError(), "kernel launch");
            if (!stream)
            {
                check(cudaStreamSynchronize(st), "execute");
                p->check_device_error();
            }
        });
}
} // namespace kfr_gpu

extern "C"
{
KFR_API_SPEC void kfr_dft_delete_plan_f32(KFR_DFT_PLAN_F32* plan)
{
    try_void([&] { if (plan) delete as<dft_obj<float>>(plan, TAG_DFT_F32); });
}
KFR_API_SPEC void kfr_dft_delete_plan_f64(KFR_DFT_PLAN_F64* plan)
{
    try_void([&] { if (plan) delete as<dft_obj<double>>(plan, TAG_DFT_F64); });
}

// ---- real DFT ------------------------------------------------------------------------------------
KFR_API_SPEC KFR_DFT_REAL_PLAN_F32* kfr_dft_real_create_plan_f32(size_t size, KFR_DFT_PACK_FORMAT fmt)
{
    return try_fn(
        [&] { return reinterpret_cast<KFR_DFT_REAL_PLAN_F32*>(static_cast<plan_base*>(new real_obj<float>(size, fmt == CCs))); },
        (KFR_DFT_REAL_PLAN_F32*)nullptr);
}
KFR_API_SPEC KFR_DFT_REAL_PLAN_F64* kfr_dft_real_create_plan_f64(size_t size, KFR_DFT_PACK_FORMAT fmt)
{
    return try_fn(
        [&] { return reinterpret_cast<KFR_DFT_REAL_PLAN_F64*>(static_cast<plan_base*>(new real_obj<double>(size, fmt == CCs))); },
        (KFR_DFT_REAL_PLAN_F64*)nullptr);
}
KFR_API_SPEC KFR_DFT_REAL_PLAN_F32* kfr_dft_real_create_2d_plan_f32(size_t size1, size_t size2, kfr_bool real_out_is_enough)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_REAL_PLAN_F32*>(static_cast<plan_base*>(new real_obj<float>(std::vector<long long>{ (long long)size1, (long long)size2 }, real_out_is_enough))); },
                  (KFR_DFT_REAL_PLAN_F32*)nullptr);
}
KFR_API_SPEC KFR_DFT_REAL_PLAN_F32* kfr_dft_real_create_3d_plan_f32(size_t size1, size_t size2, size_t size3, kfr_bool real_out_is_enough)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_REAL_PLAN_F32*>(static_cast<plan_base*>(new real_obj<float>(std::vector<long long>{ (long long)size1, (long long)size2, (long long)size3 }, real_out_is_enough))); },
                  (KFR_DFT_REAL_PLAN_F32*)nullptr);
}
KFR_API_SPEC KFR_DFT_REAL_PLAN_F32* kfr_dft_real_create_md_plan_f32(size_t dims, const unsigned* shape, kfr_bool real_out_is_enough)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_REAL_PLAN_F32*>(static_cast<plan_base*>(new real_obj<float>(to_shape(dims, shape), real_out_is_enough))); },
                  (KFR_DFT_REAL_PLAN_F32*)nullptr);
}
KFR_API_SPEC KFR_DFT_REAL_PLAN_F64* kfr_dft_real_create_2d_plan_f64(size_t size1, size_t size2, kfr_bool real_out_is_enough)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_REAL_PLAN_F64*>(static_cast<plan_base*>(new real_obj<double>(std::vector<long long>{ (long long)size1, (long long)size2 }, real_out_is_enough))); },
                  (KFR_DFT_REAL_PLAN_F64*)nullptr);
}
KFR_API_SPEC KFR_DFT_REAL_PLAN_F64* kfr_dft_real_create_3d_plan_f64(size_t size1, size_t size2, size_t size3, kfr_bool real_out_is_enough)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_REAL_PLAN_F64*>(static_cast<plan_base*>(new real_obj<double>(std::vector<long long>{ (long long)size1, (long long)size2, (long long)size3 }, real_out_is_enough))); },
                  (KFR_DFT_REAL_PLAN_F64*)nullptr);
}
KFR_API_SPEC KFR_DFT_REAL_PLAN_F64* kfr_dft_real_create_md_plan_f64(size_t dims, const unsigned* shape, kfr_bool real_out_is_enough)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_REAL_PLAN_F64*>(static_cast<plan_base*>(new real_obj<double>(to_shape(dims, shape), real_out_is_enough))); },
                  (KFR_DFT_REAL_PLAN_F64*)nullptr);
}
KFR_API_SPEC void kfr_dft_real_dump_f32(KFR_DFT_REAL_PLAN_F32* plan)
{
    try_void([&] { print_line(as<real_obj<float>>(plan, TAG_REAL_F32)->describe()); });
}
KFR_API_SPEC void kfr_dft_real_dump_f64(KFR_DFT_REAL_PLAN_F64* plan)
{
    try_void([&] { print_line(as<real_obj<double>>(plan, TAG_REAL_F64)->describe()); });
}
KFR_API_SPEC size_t kfr_dft_real_get_size_f32(KFR_DFT_REAL_PLAN_F32* plan)
{
    return try_fn([&] { return as<real_obj<float>>(plan, TAG_REAL_F32)->n; }, size_t(0));
}
KFR_API_SPEC size_t kfr_dft_real_get_size_f64(KFR_DFT_REAL_PLAN_F64* plan)
{
    return try_fn([&] { return as<real_obj<double>>(plan, TAG_REAL_F64)->n; }, size_t(0));
}
KFR_API_SPEC size_t kfr_dft_real_get_temp_size_batch_f32(KFR_DFT_REAL_PLAN_F32* plan, size_t batch)
{
    return try_fn([&] { return size_t(as<real_obj<float>>(plan, TAG_REAL_F32)->scratch_elems(batch)) * 8; },
                  size_t(0));
}
KFR_API_SPEC size_t kfr_dft_real_get_temp_size_batch_f64(KFR_DFT_REAL_PLAN_F64* plan, size_t batch)
{
    return try_fn([&] { return size_t(as<real_obj<double>>(plan, TAG_REAL_F64)->scratch_elems(batch)) * 16; },
                  size_t(0));
}
KFR_API_SPEC size_t kfr_dft_real_get_temp_size_f32(KFR_DFT_REAL_PLAN_F32* plan)
{
    return kfr_dft_real_get_temp_size_batch_f32(plan, 1);
}
KFR_API_SPEC size_t kfr_dft_real_get_temp_size_f64(KFR_DFT_REAL_PLAN_F64* plan)
{
    return kfr_dft_real_get_temp_size_batch_f64(plan, 1);
}
KFR_API_SPEC void kfr_dft_real_execute_f32(KFR_DFT_REAL_PLAN_F32* plan, kfr_c32* out, const kfr_f32* in, uint8_t* temp)
{
    try_void([&] { exec_real<float>(plan, 1, out, in, temp, false, nullptr); });
}
KFR_API_SPEC void kfr_dft_real_execute_f64(KFR_DFT_REAL_PLAN_F64* plan, kfr_c64* out, const kfr_f64* in, uint8_t* temp)
{
    try_void([&] { exec_real<double>(plan, 1, out, in, temp, false, nullptr); });
}
KFR_API_SPEC void kfr_dft_real_execute_inverse_f32(KFR_DFT_REAL_PLAN_F32* plan, kfr_f32* out, const kfr_c32* in,
                                                   uint8_t* temp)
{
    try_void([&] { exec_real<float>(plan, 1, out, in, temp, true, nullptr); });
}
KFR_API_SPEC void kfr_dft_real_execute_inverse_f64(KFR_DFT_REAL_PLAN_F64* plan, kfr_f64* out, const kfr_c64* in,
                                                   uint8_t* temp)
{
    try_void([&] { exec_real<double>(plan, 1, out, in, temp, true, nullptr); });
}
KFR_API_SPEC void kfr_dft_real_execute_batch_f32(KFR_DFT_REAL_PLAN_F32* plan, size_t batch, kfr_c32* out,
                                                 const kfr_f32* in, uint8_t* temp, void* stream)
{
    try_void([&] { exec_real<float>(plan, batch, out, in, temp, false, stream); });
}
KFR_API_SPEC void kfr_dft_real_execute_batch_f64(KFR_DFT_REAL_PLAN_F64* plan, size_t batch, kfr_c64* out,
                                                 const kfr_f64* in, uint8_t* temp, void* stream)
{
    try_void([&] { exec_real<double>(plan, batch, out, in, temp, false, stream); });
}
KFR_API_SPEC void kfr_dft_real_execute_inverse_batch_f32(KFR_DFT_REAL_PLAN_F32* plan, size_t batch, kfr_f32* out,
                                                         const kfr_c32* in, uint8_t* temp, void* stream)
{
    try_void([&] { exec_real<float>(plan, batch, out, in, temp, true, stream); });
}
KFR_API_SPEC void kfr_dft_real_execute_inverse_batch_f64(KFR_DFT_REAL_PLAN_F64* plan, size_t batch, kfr_f64* out,
                                                         const kfr_c64* in, uint8_t* temp, void* stream)
{
    try_void([&] { exec_real<double>(plan, batch, out, in, temp, true, stream); });
}
KFR_API_SPEC void kfr_dft_real_delete_plan_f32(KFR_DFT_REAL_PLAN_F32* plan)
{
    try_void([&] { if (plan) delete as<real_obj<float>>(plan, TAG_REAL_F32); });
}
KFR_API_SPEC void kfr_dft_real_delete_plan_f64(KFR_DFT_REAL_PLAN_F64* plan)
{
    try_void([&] { if (plan) delete as<real_obj<double>>(plan, TAG_REAL_F64); });
}

// ---- DCT -----------------------------------------------------------------------------------------------
KFR_API_SPEC KFR_DCT_PLAN_F32* kfr_dct_create_plan_f32(size_t size)
{
    return try_fn([&] { return reinterpret_cast<KFR_DCT_PLAN_F32*>(static_cast<plan_base*>(new dct_obj<float>(size))); },
                  (KFR_DCT_PLAN_F32*)nullptr);
}
KFR_API_SPEC KFR_DCT_PLAN_F64* kfr_dct_create_plan_f64(size_t size)
{
    return try_fn([&] { return reinterpret_cast<KFR_DCT_PLAN_F64*>(static_cast<plan_base*>(new dct_obj<double>(size))); },
                  (KFR_DCT_PLAN_F64*)nullptr);
}
KFR_API_SPEC void kfr_dct_dump_f32(KFR_DCT_PLAN_F32* plan)
{
    try_void([&] { print_line(as<dct_obj<float>>(plan, TAG_DCT_F32)->eng.describe()); });
}
KFR_API_SPEC void kfr_dct_dump_f64(KFR_DCT_PLAN_F64* plan)
{
    try_void([&] { print_line(as<dct_obj<double>>(plan, TAG_DCT_F64)->eng.describe()); });
}
KFR_API_SPEC size_t kfr_dct_get_size_f32(KFR_DCT_PLAN_F32* plan)
{
    return try_fn([&] { return as<dct_obj<float>>(plan, TAG_DCT_F32)->n; }, size_t(0));
}
KFR_API_SPEC size_t kfr_dct_get_size_f64(KFR_DCT_PLAN_F64* plan)
{
    return try_fn([&] { return as<dct_obj<double>>(plan, TAG_DCT_F64)->n; }, size_t(0));
}
KFR_API_SPEC size_t kfr_dct_get_temp_size_batch_f32(KFR_DCT_PLAN_F32* plan, size_t batch)
{
    return try_fn([&] { return size_t(as<dct_obj<float>>(plan, TAG_DCT_F32)->eng.scratch_elems(batch)) * 8; },
                  size_t(0));
}
KFR_API_SPEC size_t kfr_dct_get_temp_size_batch_f64(KFR_DCT_PLAN_F64* plan, size_t batch)
{
    return try_fn([&] { return size_t(as<dct_obj<double>>(plan, TAG_DCT_F64)->eng.scratch_elems(batch)) * 16; },
                  size_t(0));
}
KFR_API_SPEC size_t kfr_dct_get_temp_size_f32(KFR_DCT_PLAN_F32* plan) { return kfr_dct_get_temp_size_batch_f32(plan, 1); }
KFR_API_SPEC size_t kfr_dct_get_temp_size_f64(KFR_DCT_PLAN_F64* plan) { return kfr_dct_get_temp_size_batch_f64(plan, 1); }
KFR_API_SPEC void kfr_dct_execute_f32(KFR_DCT_PLAN_F32* plan, kfr_f32* out, const kfr_f32* in, uint8_t* temp)
{
    try_void([&] { exec_dct<float>(plan, 1, out, in, temp, false, nullptr); });
}
KFR_API_SPEC void kfr_dct_execute_f64(KFR_DCT_PLAN_F64* plan, kfr_f64* out, const kfr_f64* in, uint8_t* temp)
{
    try_void([&] { exec_dct<double>(plan, 1, out, in, temp, false, nullptr); });
}
KFR_API_SPEC void kfr_dct_execute_inverse_f32(KFR_DCT_PLAN_F32* plan, kfr_f32* out, const kfr_f32* in, uint8_t* temp)
{
    try_void([&] { exec_dct<float>(plan, 1, out, in, temp, true, nullptr); });
}
KFR_API_SPEC void kfr_dct_execute_inverse_f64(KFR_DCT_PLAN_F64* plan, kfr_f64* out, const kfr_f64* in, uint8_t* temp)
{
    try_void([&] { exec_dct<double>(plan, 1, out, in, temp, true, nullptr); });
}
KFR_API_SPEC void kfr_dct_execute_batch_f32(KFR_DCT_PLAN_F32* plan, size_t batch, kfr_f32* out, const kfr_f32* in,
                                            uint8_t* temp, kfr_bool inverse, void* stream)
{
    try_void([&] { exec_dct<float>(plan, batch, out, in, temp, inverse, stream); });
}
KFR_API_SPEC void kfr_dct_execute_batch_f64(KFR_DCT_PLAN_F64* plan, size_t batch, kfr_f64* out, const kfr_f64* in,
                                            uint8_t* temp, kfr_bool inverse, void* stream)
{
    try_void([&] { exec_dct<double>(plan, batch, out, in, temp, inverse, stream); });
}
KFR_API_SPEC void kfr_dct_delete_plan_f32(KFR_DCT_PLAN_F32* plan)
{
    try_void([&] { if (plan) delete as<dct_obj<float>>(plan, TAG_DCT_F32); });
}
KFR_API_SPEC void kfr_dct_delete_plan_f64(KFR_DCT_PLAN_F64* plan)
{
    try_void([&] { if (plan) delete as<dct_obj<double>>(plan, TAG_DCT_F64); });
}

// ---- filters -------------------------------------------------------------------------------------------
// FIR filters run through the DFT path: the reference's fir_filter (src/capi/capi.cpp:567-580) and its
// convolve_filter compute the same y[n] = sum_k taps[k] x[n - k] with state across calls (its docs:
// docs/docs/fir.md:94), so a FIR plan is a convolution-filter plan with the default block.
KFR_API_SPEC KFR_FILTER_F32* kfr_filter_create_fir_plan_f32(const kfr_f32* taps, size_t size)
{
    return try_fn(
        [&] { return reinterpret_cast<KFR_FILTER_F32*>(static_cast<plan_base*>(new filter_obj<float>(taps, size, 1024))); },
        (KFR_FILTER_F32*)nullptr);
}
KFR_API_SPEC KFR_FILTER_F64* kfr_filter_create_fir_plan_f64(const kfr_f64* taps, size_t size)
{
    return try_fn(
        [&] { return reinterpret_cast<KFR_FILTER_F64*>(static_cast<plan_base*>(new filter_obj<double>(taps, size, 1024))); },
        (KFR_FILTER_F64*)nullptr);
}
KFR_API_SPEC KFR_FILTER_F32* kfr_filter_create_iir_plan_f32(const kfr_f32*, size_t)
{
    return try_fn([]() -> KFR_FILTER_F32* { not_built("kfr_filter_create_iir_plan_f32"); }, (KFR_FILTER_F32*)nullptr);
}
KFR_API_SPEC KFR_FILTER_F64* kfr_filter_create_iir_plan_f64(const kfr_f64*, size_t)
{
    return try_fn([]() -> KFR_FILTER_F64* { not_built("kfr_filter_create_iir_plan_f64"); }, (KFR_FILTER_F64*)nullptr);
}
KFR_API_SPEC KFR_FILTER_F32* kfr_filter_create_convolution_plan_f32(const kfr_f32* taps, size_t size, size_t block_size)
{
    return try_fn(
        [&] {
            return reinterpret_cast<KFR_FILTER_F32*>(
                static_cast<plan_base*>(new filter_obj<float>(taps, size, block_size ? block_size : 1024)));
        },
        (KFR_FILTER_F32*)nullptr);
}
KFR_API_SPEC KFR_FILTER_F64* kfr_filter_create_convolution_plan_f64(const kfr_f64* taps, size_t size, size_t block_size)
{
    return try_fn(
        [&] {
            return reinterpret_cast<KFR_FILTER_F64*>(
                static_cast<plan_base*>(new filter_obj<double>(taps, size, block_size ? block_size : 1024)));
        },
        (KFR_FILTER_F64*)nullptr);
}
KFR_API_SPEC void kfr_filter_process_f32(KFR_FILTER_F32* plan, kfr_f32* output, const kfr_f32* input, size_t size)
{
    try_void([&] { filter_process<float>(plan, output, input, size); });
}
KFR_API_SPEC void kfr_filter_process_f64(KFR_FILTER_F64* plan, kfr_f64* output, const kfr_f64* input, size_t size)
{
    try_void([&] { filter_process<double>(plan, output, input, size); });
}
KFR_API_SPEC void kfr_filter_reset_f32(KFR_FILTER_F32* plan)
{
    try_void([&] { as<filter_obj<float>>(plan, TAG_FLT_F32)->f.reset(); });
}
KFR_API_SPEC void kfr_filter_reset_f64(KFR_FILTER_F64* plan)
{
    try_void([&] { as<filter_obj<double>>(plan, TAG_FLT_F64)->f.reset(); });
}
KFR_API_SPEC void kfr_filter_delete_plan_f32(KFR_FILTER_F32* plan)
{
    try_void([&] { if (plan) delete as<filter_obj<float>>(plan, TAG_FLT_F32); });
}
KFR_API_SPEC void kfr_filter_delete_plan_f64(KFR_FILTER_F64* plan)
{
    try_void([&] { if (plan) delete as<filter_obj<double>>(plan, TAG_FLT_F64); });
}

/* Adjoints (no counterpart in the reference) */
KFR_API_SPEC void kfr_dft_adjoint_batch_f32(KFR_DFT_PLAN_F32* plan, size_t batch, kfr_c32* grad_in,
                                            const kfr_c32* grad_out, uint8_t* temp, kfr_bool inverse, void* stream)
{
    try_void([&] { exec_dft<float>(plan, batch, grad_in, grad_out, temp, !inverse, stream); });
}
KFR_API_SPEC void kfr_dft_adjoint_batch_f64(KFR_DFT_PLAN_F64* plan, size_t batch, kfr_c64* grad_in,
                                            const kfr_c64* grad_out, uint8_t* temp, kfr_bool inverse, void* stream)
{
    try_void([&] { exec_dft<double>(plan, batch, grad_in, grad_out, temp, !inverse, stream); });
}
KFR_API_SPEC void kfr_dft_real_adjoint_batch_f32(KFR_DFT_REAL_PLAN_F32* plan, size_t batch, kfr_f32* grad_in,
                                                 const kfr_c32* grad_out, uint8_t* temp, void* stream)
{
    (void)temp;
    try_void([&] { adj_real<float>(plan, batch, grad_in, grad_out, false, stream); });
}
KFR_API_SPEC void kfr_dft_real_adjoint_batch_f64(KFR_DFT_REAL_PLAN_F64* plan, size_t batch, kfr_f64* grad_in,
                                                 const kfr_c64* grad_out, uint8_t* temp, void* stream)
{
    (void)temp;
    try_void([&] { adj_real<double>(plan, batch, grad_in, grad_out, false, stream); });
}
KFR_API_SPEC void kfr_dft_real_adjoint_inverse_batch_f32(KFR_DFT_REAL_PLAN_F32* plan, size_t batch, kfr_c32* grad_in,
                                                         const kfr_f32* grad_out, uint8_t* temp, void* stream)
{
    (void)temp;
    try_void([&] { adj_real<float>(plan, batch, grad_in, grad_out, true, stream); });
}
KFR_API_SPEC void kfr_dft_real_adjoint_inverse_batch_f64(KFR_DFT_REAL_PLAN_F64* plan, size_t batch, kfr_c64* grad_in,
                                                         const kfr_f64* grad_out, uint8_t* temp, void* stream)
{
    (void)temp;
    try_void([&] { adj_real<double>(plan, batch, grad_in, grad_out, true, stream); });
}
KFR_API_SPEC void kfr_dct_adjoint_batch_f32(KFR_DCT_PLAN_F32* plan, size_t batch, kfr_f32* grad_in,
                                            const kfr_f32* grad_out, uint8_t* temp, kfr_bool inverse, void* stream)
{
    (void)temp;
    try_void([&] { adj_dct<float>(plan, batch, grad_in, grad_out, inverse, stream); });
}
KFR_API_SPEC void kfr_dct_adjoint_batch_f64(KFR_DCT_PLAN_F64* plan, size_t batch, kfr_f64* grad_in,
                                            const kfr_f64* grad_out, uint8_t* temp, kfr_bool inverse, void* stream)
{
    (void)temp;
    try_void([&] { adj_dct<double>(plan, batch, grad_in, grad_out, inverse, stream); });
}
KFR_API_SPEC void kfr_fir_backward_f32(const kfr_f32* taps, size_t ntaps, size_t channels, size_t n, const kfr_f32* x,
                                       const kfr_f32* grad_y, kfr_f32* grad_x, kfr_f32* grad_taps, void* stream)
{
    try_void([&] { fir_bwd<float>(taps, ntaps, channels, n, x, grad_y, grad_x, grad_taps, stream); });
}
KFR_API_SPEC void kfr_fir_backward_f64(const kfr_f64* taps, size_t ntaps, size_t channels, size_t n, const kfr_f64* x,
                                       const kfr_f64* grad_y, kfr_f64* grad_x, kfr_f64* grad_taps, void* stream)
{
    try_void([&] { fir_bwd<double>(taps, ntaps, channels, n, x, grad_y, grad_x, grad_taps, stream); });
}

/* Uneven batch (extension) */
KFR_API_SPEC KFR_DFT_UNEVEN_F32* kfr_dft_create_uneven_plan_f32(const size_t* lengths, size_t count, kfr_bool autotune)
{
    return try_fn(
        [&]
        {
            if (!lengths && count)
                throw std::invalid_argument("lengths is NULL");
            std::vector<long long> l(lengths, lengths + count);
            return reinterpret_cast<KFR_DFT_UNEVEN_F32*>(static_cast<plan_base*>(new uneven_obj(l, autotune != 0)));
        },
        (KFR_DFT_UNEVEN_F32*)nullptr);
}
KFR_API_SPEC size_t kfr_dft_uneven_get_size_f32(KFR_DFT_UNEVEN_F32* plan)
{
    return try_fn([&] { return size_t(as<uneven_obj>(plan, TAG_UNEVEN)->plan.total()); }, size_t(0));
}
KFR_API_SPEC void kfr_dft_uneven_execute_f32(KFR_DFT_UNEVEN_F32* plan, kfr_c32* out, const kfr_c32* in, kfr_bool inverse,
                                             void* stream)
{
    try_void([&] { exec_uneven(plan, out, in, inverse != 0, stream, false); });
}
KFR_API_SPEC uint32_t kfr_set_wait_limit(uint32_t spins)
{
    static_assert(KFR_DEFAULT_WAIT_SPINS == kfr_gpu::kDefaultWaitSpins, "one default wait limit");
    return set_wait_limit(spins);
}
KFR_API_SPEC void kfr_dft_uneven_set_unreachable_stage_f32(KFR_DFT_UNEVEN_F32* plan, kfr_bool unreachable)
{
    try_void(
        [&]
        {
            auto* p = as<uneven_obj>(plan, TAG_UNEVEN);
            std::unique_lock<std::mutex> lock(p->mu);
            p->plan.set_unreachable_stage(unreachable != 0);
        });
}
KFR_API_SPEC void kfr_dft_uneven_execute_per_signal_f32(KFR_DFT_UNEVEN_F32* plan, kfr_c32* out, const kfr_c32* in,
                                                        kfr_bool inverse, void* stream)
{
    try_void([&] { exec_uneven(plan, out, in, inverse != 0, stream, true); });
}
KFR_API_SPEC size_t kfr_dft_uneven_describe_f32(KFR_DFT_UNEVEN_F32* plan, char* buf, size_t size)
{
    return try_fn(
        [&]
        {
            const std::string d = as<uneven_obj>(plan, TAG_UNEVEN)->plan.describe();
            if (buf && size)
            {
                const size_t k = std::min(size - 1, d.size());
                std::memcpy(buf, d.data(), k);
                buf[k] = 0;
            }
            return d.size();
        },
        size_t(0));
}
KFR_API_SPEC void kfr_dft_uneven_delete_plan_f32(KFR_DFT_UNEVEN_F32* plan)
{
    try_void([&] { if (plan) delete as<uneven_obj>(plan, TAG_UNEVEN); });
}

/* Multi-channel convolution filter (extension) */
KFR_API_SPEC KFR_FILTER_F32* kfr_filter_create_convolution_plan_channels_f32(const kfr_f32* taps, size_t size,
                                                                           size_t block_size, size_t channels)
{
    return try_fn(
        [&] {
            if (channels < 1 || channels > (1u << 16))
                throw std::invalid_argument("channels must be between 1 and 65536");
            return reinterpret_cast<KFR_FILTER_F32*>(static_cast<plan_base*>(
                new filter_obj<float>(taps, size, block_size ? block_size : 1024, int(channels))));
        },
        (KFR_FILTER_F32*)nullptr);
}
KFR_API_SPEC KFR_FILTER_F64* kfr_filter_create_convolution_plan_channels_f64(const kfr_f64* taps, size_t size,
                                                                           size_t block_size, size_t channels)
{
    return try_fn(
        [&] {
            if (channels < 1 || channels > (1u << 16))
                throw std::invalid_argument("channels must be between 1 and 65536");
            return reinterpret_cast<KFR_FILTER_F64*>(static_cast<plan_base*>(
                new filter_obj<double>(taps, size, block_size ? block_size : 1024, int(channels))));
        },
        (KFR_FILTER_F64*)nullptr);
}

/* Tensor-core plans (extension) */
KFR_API_SPEC KFR_DFT_PLAN_F32* kfr_dft_create_plan_tensor_f32(size_t size, int split)
{
    return try_fn([&] { return reinterpret_cast<KFR_DFT_PLAN_F32*>(static_cast<plan_base*>(new dft_obj<float>(size, split))); },
                  (KFR_DFT_PLAN_F32*)nullptr);
}

} // extern "C"
