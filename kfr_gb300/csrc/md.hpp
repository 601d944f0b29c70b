// Multi-dimensional DFTs: dft_plan_md<T> and dft_plan_md_real<T> (include/kfr/dft/fft.hpp:568-924).
//
// The reference transforms the last axis of a row-major array, transposes, and repeats for every axis.  On
// the GPU the last axis runs as a batched 1-D transform over contiguous rows, and every other axis i whose
// length fits one CTA runs in place as a column pass over the [outer][n_i][inner] view (tiles of adjacent
// columns are staged in shared memory, transformed, and written back to the same places).  A longer axis
// (any length: four-step, Rader, Bluestein) is transposed to [outer][inner][n_i] in scratch, transformed
// there by the 1-D engine as outer x inner contiguous signals, and transposed back.  The real variant does
// the CCs real DFT along the last axis first (forward) or last (inverse), like the reference, so the
// complex array has the reference's complex_size() shape (last axis N/2 + 1).
#pragma once

#include "plan.hpp"

namespace kfr_gpu
{

template <typename T>
class md_axes
{
public:
    // Axes 0 .. dims-2 of `cshape` (complex element shape) with length > 1.
    explicit md_axes(const std::vector<long long>& cshape);
    // In place on `data` (batch arrays of the complex shape back to back); scratch: scratch_elems(batch)
    // complex elements (none unless an axis is longer than one CTA).
    void run(void* data, long long batch, bool inverse, void* scratch, cudaStream_t st) const;
    long long scratch_elems(long long batch) const;
    int launches(long long batch) const;
    std::string describe() const;
    void check_device_error() const
    {
        for (const axis& a : axes_)
            if (a.eng)
                a.eng->check_device_error();
    }

private:
    struct axis
    {
        long long n, inner, outer;
        int tile;
        std::unique_ptr<block_program<T>> prog; // column pass (axes that fit one CTA)
        std::unique_ptr<complex_engine<T>> eng; // transposed 1-D pass (longer axes)
    };
    std::vector<axis> axes_;
    long long total_ = 1;
};

template <typename T>
class md_engine
{
public:
    explicit md_engine(const std::vector<long long>& shape);
    long long size() const { return total_; }
    const std::vector<long long>& shape() const { return shape_; }
    long long scratch_elems(long long batch) const;
    void execute(void* out, const void* in, long long batch, bool inverse, void* scratch, cudaStream_t st) const;
    std::string describe() const;
    int launches(long long batch) const;
    void check_device_error() const
    {
        if (last_)
            last_->check_device_error();
        axes_.check_device_error();
    }

private:
    std::vector<long long> shape_;
    long long total_ = 0;
    std::unique_ptr<complex_engine<T>> last_;
    md_axes<T> axes_;
};

template <typename T>
class md_real_engine
{
public:
    md_real_engine(const std::vector<long long>& shape, bool real_out_is_enough);
    long long size() const { return total_real_; }
    long long complex_size() const { return total_cplx_; }
    const std::vector<long long>& shape() const { return shape_; }
    long long scratch_elems(long long batch) const;
    void forward(void* out, const void* in, long long batch, void* scratch, cudaStream_t st) const;
    void inverse(void* out, const void* in, long long batch, void* scratch, cudaStream_t st) const;
    std::string describe() const;
    int launches(long long batch) const;
    void check_device_error() const
    {
        last_->check_device_error();
        axes_.check_device_error();
    }

private:
    std::vector<long long> shape_, cshape_;
    long long total_real_ = 0, total_cplx_ = 0;
    bool real_out_is_enough_;
    std::unique_ptr<real_engine<T>> last_;
    md_axes<T> axes_;
};

} // namespace kfr_gpu
