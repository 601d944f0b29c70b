// Multi-dimensional DFTs (see md.hpp).
#include "md.hpp"

#include <algorithm>
#include <sstream>

namespace kfr_gpu
{

static long long product(const std::vector<long long>& v, size_t b, size_t e)
{
    long long p = 1;
    for (size_t i = b; i < e; i++)
        p *= v[i];
    return p;
}

template <typename T>
md_axes<T>::md_axes(const std::vector<long long>& cshape)
{
    const size_t d = cshape.size();
    total_         = product(cshape, 0, d);
    for (size_t i = 0; i + 1 < d; i++)
    {
        const long long n = cshape[i];
        if (n <= 1)
            continue;
        axis a;
        a.n     = n;
        a.inner = product(cshape, i + 1, d);
        a.outer = product(cshape, 0, i);
        a.tile  = 0;
        if (block_program<T>::feasible(n))
        {
            a.prog.reset(new block_program<T>());
            a.prog->build(int(n), CT_FOURSTEP);
            int t = tile_for(*a.prog);
            while (t > 1 && t / 2 >= a.inner)
                t /= 2;
            a.tile = t;
            if (t == 0)
                a.prog.reset();
        }
        if (!a.prog) // longer than one CTA: transposed 1-D pass
            a.eng.reset(new complex_engine<T>(n));
        axes_.push_back(std::move(a));
    }
}

template <typename T>
long long md_axes<T>::scratch_elems(long long batch) const
{
    long long need = 0;
    for (const axis& a : axes_)
        if (a.eng)
            need = std::max(need, batch * total_ + a.eng->scratch_elems(batch * a.outer * a.inner));
    return need;
}

template <typename T>
int md_axes<T>::launches(long long batch) const
{
    int n = 0;
    for (const axis& a : axes_)
        n += a.eng ? 2 + a.eng->launches(batch * a.outer * a.inner) : int((batch * a.outer + 65534) / 65535);
    return n;
}

template <typename T>
void md_axes<T>::run(void* data, long long batch, bool inverse, void* scratch, cudaStream_t st) const
{
    for (const axis& ax : axes_)
    {
        if (ax.eng)
        {
            // [batch outer][n][inner] -> [batch outer][inner][n], n-point DFTs of the rows, and back
            char* tr  = static_cast<char*>(scratch);
            char* scr = tr + batch * total_ * 2 * sizeof(T);
            check(launch_transpose<T>(tr, data, batch * ax.outer, ax.n, ax.inner, st), "transpose axis");
            ax.eng->execute(tr, tr, batch * ax.outer * ax.inner, ax.n, ax.n, inverse, scr, st);
            check(launch_transpose<T>(data, tr, batch * ax.outer, ax.inner, ax.n, st), "transpose axis back");
            continue;
        }
        const long long sigs = batch * ax.outer;
        for (long long b0 = 0; b0 < sigs; b0 += 65535)
        {
            const long long nb = std::min<long long>(65535, sigs - b0);
            char* base         = static_cast<char*>(data) + b0 * ax.n * ax.inner * 2 * sizeof(T);
            fourstep_args a;
            a.err         = nullptr;
            a.in          = base;
            a.out         = base;
            a.batch       = nb;
            a.sig_stride  = ax.n * ax.inner;
            a.n1          = int(ax.n);
            a.n2          = int(ax.inner);
            a.tile        = ax.tile;
            int sh        = 0;
            while ((1 << sh) < ax.tile)
                sh++;
            a.tile_shift  = sh;
            a.same_layout = 1;
            a.pingpong    = 0;
            a.conj_in     = inverse;
            a.conj_out    = inverse;
            a.tw          = ax.prog->tw.get();
            a.d           = ax.prog->desc;
            a.twA         = nullptr;
            a.twB         = nullptr;
            a.lbits       = 0;
            a.div_n       = make_fast_div(uint32_t(ax.n));
            block_cfg c   = ax.prog->cfg_tile(ax.tile);
            c.grid        = (ax.inner + ax.tile - 1) / ax.tile;
            check(launch_fs_cols<T>(a, c, st), "launch multi-dimensional axis pass");
        }
    }
}

template <typename T>
std::string md_axes<T>::describe() const
{
    std::ostringstream s;
    for (const axis& a : axes_)
    {
        if (a.eng)
            s << " axis{n=" << a.n << " inner=" << a.inner << " transposed [" << a.eng->describe() << "]}";
        else
            s << " axis{n=" << a.n << " inner=" << a.inner << " tile=" << a.tile << " " << a.prog->describe() << "}";
    }
    return s.str();
}

template <typename T>
static std::vector<long long> check_shape(const std::vector<long long>& shape)
{
    if (shape.empty())
        throw std::invalid_argument("multi-dimensional DFT: no dimensions");
    for (long long v : shape)
        if (v <= 0)
            throw std::invalid_argument("multi-dimensional DFT: every dimension must be positive");
    return shape;
}

// ------------------------------------------------------------------------------------------------------
// complex
// ------------------------------------------------------------------------------------------------------

template <typename T>
md_engine<T>::md_engine(const std::vector<long long>& shape)
    : shape_(check_shape<T>(shape)), total_(product(shape, 0, shape.size())), axes_(shape)
{
    if (shape_.back() > 1)
        last_.reset(new complex_engine<T>(shape_.back()));
}

template <typename T>
long long md_engine<T>::scratch_elems(long long batch) const
{
    return std::max(last_ ? last_->scratch_elems(batch * (total_ / shape_.back())) : 0LL, axes_.scratch_elems(batch));
}

template <typename T>
int md_engine<T>::launches(long long batch) const
{
    return (last_ ? last_->launches(batch * (total_ / shape_.back())) : 1) + axes_.launches(batch);
}

template <typename T>
void md_engine<T>::execute(void* out, const void* in, long long batch, bool inverse, void* scratch,
                           cudaStream_t st) const
{
    if (batch <= 0 || total_ == 0)
        return;
    const long long nl = shape_.back();
    if (last_)
        last_->execute(out, in, batch * (total_ / nl), nl, nl, inverse, scratch, st);
    else if (out != in)
        check(cudaMemcpyAsync(out, in, batch * total_ * 2 * sizeof(T), cudaMemcpyDeviceToDevice, st), "copy");
    axes_.run(out, batch, inverse, scratch, st);
}

template <typename T>
std::string md_engine<T>::describe() const
{
    std::ostringstream s;
    s << "md shape=(";
    for (size_t i = 0; i < shape_.size(); i++)
        s << (i ? "," : "") << shape_[i];
    s << ") last{" << (last_ ? last_->describe() : std::string("copy")) << "}" << axes_.describe();
    return s.str();
}

// ------------------------------------------------------------------------------------------------------
// real
// ------------------------------------------------------------------------------------------------------

template <typename T>
static std::vector<long long> complex_shape(std::vector<long long> s)
{
    s.back() = s.back() / 2 + 1;
    return s;
}

template <typename T>
md_real_engine<T>::md_real_engine(const std::vector<long long>& shape, bool real_out_is_enough)
    : shape_(check_shape<T>(shape)), cshape_(complex_shape<T>(shape)), real_out_is_enough_(real_out_is_enough),
      axes_(complex_shape<T>(shape))
{
    if (shape_.back() % 2)
        throw std::logic_error("dft_plan_real requires size to be even");
    total_real_ = product(shape_, 0, shape_.size());
    total_cplx_ = product(cshape_, 0, cshape_.size());
    last_.reset(new real_engine<T>(shape_.back()));
}

// Scratch: [W: batch complex arrays (inverse only)][R: the last axis's or the other axes' scratch].
template <typename T>
long long md_real_engine<T>::scratch_elems(long long batch) const
{
    const long long rows = batch * (total_real_ / shape_.back());
    return batch * total_cplx_ + std::max(last_->scratch_elems(rows), axes_.scratch_elems(batch));
}

template <typename T>
int md_real_engine<T>::launches(long long batch) const
{
    return last_->launches(batch * (total_real_ / shape_.back())) + axes_.launches(batch);
}

template <typename T>
void md_real_engine<T>::forward(void* out, const void* in, long long batch, void* scratch, cudaStream_t st) const
{
    if (batch <= 0)
        return;
    const long long rows = batch * (total_real_ / shape_.back());
    char* inner          = static_cast<char*>(scratch) + batch * total_cplx_ * 2 * sizeof(T);
    last_->forward(out, in, rows, true, inner, st);
    axes_.run(out, batch, false, inner, st);
}

template <typename T>
void md_real_engine<T>::inverse(void* out, const void* in, long long batch, void* scratch, cudaStream_t st) const
{
    if (batch <= 0)
        return;
    const long long rows = batch * (total_real_ / shape_.back());
    char* W              = static_cast<char*>(scratch);
    char* inner          = W + batch * total_cplx_ * 2 * sizeof(T);
    check(cudaMemcpyAsync(W, in, batch * total_cplx_ * 2 * sizeof(T), cudaMemcpyDeviceToDevice, st),
          "copy spectrum");
    axes_.run(W, batch, true, inner, st);
    last_->inverse(out, W, rows, true, inner, st);
}

template <typename T>
std::string md_real_engine<T>::describe() const
{
    std::ostringstream s;
    s << "md real shape=(";
    for (size_t i = 0; i < shape_.size(); i++)
        s << (i ? "," : "") << shape_[i];
    s << ") last{" << last_->describe() << "}" << axes_.describe();
    return s.str();
}

template class md_axes<float>;
template class md_axes<double>;
template class md_engine<float>;
template class md_engine<double>;
template class md_real_engine<float>;
template class md_real_engine<double>;

} // namespace kfr_gpu
